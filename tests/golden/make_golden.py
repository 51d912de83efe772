"""Generate the golden vectors that pin the CPU oracle to the girih reference.

Runs the unmodified reference time stepper (spatial blocking, --target-ts 0,
src/kernels/nb_naive_ts.c:165-216) through the harness oracle/ref_golden.c,
which links the reference objects built by `make -C oracle ref` from the
reference's own sources.  Each case stores the reference's U1 and U2 after nt
steps (full padded local domain, float64) in tests/golden/golden_ref.npz.

Usage (needs the reference sources, i.e. only in the development container):
    make -C oracle ref && python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_golden")

# standard 8th-order central second-difference weights summed over 3 axes
# (sum of the 25 weights is 0, so the leapfrog is stable for small roc2)
LAP8 = [3 * (-205.0 / 72.0), 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0]

# name, op, nx, ny, nz, nt, init, seeded parameters
CASES = [
    ("k0_ref", 0, 12, 10, 9, 6, "ref", None),
    ("k0_seed", 0, 12, 10, 9, 6, "seeded", dict(seed=2, f=(-1, 1), roc2=(0.05, 0.15), c=(0, 0), coefs=LAP8)),
    ("k0_ragged", 0, 9, 5, 7, 3, "seeded", dict(seed=21, f=(-1, 1), roc2=(0.05, 0.15), c=(0, 0), coefs=LAP8)),
    ("k1_ref", 1, 13, 11, 9, 6, "ref", None),
    ("k1_ref_odd_nt", 1, 13, 11, 9, 5, "ref", None),
    ("k1_nt0", 1, 13, 11, 9, 0, "ref", None),
    ("k1_seed", 1, 13, 11, 9, 8, "seeded", dict(seed=0, f=(0, 1), roc2=(0, 0), c=(0, 0), coefs=None)),
    ("k1_tiny", 1, 1, 1, 1, 4, "ref", None),
    ("k1_thin", 1, 17, 2, 3, 4, "seeded", dict(seed=5, f=(0, 1), roc2=(0, 0), c=(0, 0), coefs=None)),
    ("k1_wide", 1, 40, 7, 6, 4, "seeded", dict(seed=6, f=(0, 1), roc2=(0, 0), c=(0, 0), coefs=[-0.5, 1.0 / 12])),
    ("k2_ref", 2, 13, 11, 9, 6, "ref", None),
    ("k2_seed", 2, 13, 11, 9, 6, "seeded", dict(seed=3, f=(0, 1), roc2=(0, 0), c=(0.01, 0.1), coefs=None)),
    ("k3_ref", 3, 13, 11, 9, 6, "ref", None),
    ("k3_seed", 3, 13, 11, 9, 6, "seeded", dict(seed=3, f=(0, 1), roc2=(0, 0), c=(0.01, 0.1), coefs=None)),
    ("k4_ref", 4, 12, 10, 9, 6, "ref", None),
    ("k4_seed", 4, 12, 10, 9, 6, "seeded", dict(seed=3, f=(0, 1), roc2=(0, 0), c=(0.01, 0.025), coefs=None)),
    ("k5_ref", 5, 13, 11, 9, 6, "ref", None),
    ("k5_seed", 5, 13, 11, 9, 6, "seeded", dict(seed=3, f=(0, 1), roc2=(0, 0), c=(0.01, 0.1), coefs=None)),
    ("k5_ragged", 5, 7, 3, 5, 3, "seeded", dict(seed=31, f=(0, 1), roc2=(0, 0), c=(0.01, 0.1), coefs=None)),
    ("k7_seed", 7, 13, 11, 9, 4, "seeded", dict(seed=7, f=(0, 1), roc2=(0, 0), c=(0, 0), coefs=[-0.5, 0.05, 0.02, 0.01])),
]
# with the reference's source-point update switched on (GIRIH_REF_SOURCE=1): the
# reference's centred point and source[i] = i
SOURCE_CASES = [
    ("k1_src", 1, 13, 11, 9, 6, "ref", None),
    ("k0_src", 0, 12, 10, 9, 6, "seeded", dict(seed=2, f=(-1, 1), roc2=(0.05, 0.15), c=(0, 0), coefs=LAP8)),
    ("k5_src", 5, 13, 11, 9, 4, "seeded", dict(seed=3, f=(0, 1), roc2=(0, 0), c=(0.01, 0.1), coefs=None)),
]


def run_case(op, nx, ny, nz, nt, init, sp, source=False):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "g.bin")
        cmd = [HARNESS, str(op), str(nx), str(ny), str(nz), str(nt), "0", init, out]
        if init == "seeded":
            cmd += [str(sp["seed"])] + [repr(float(x)) for x in (*sp["f"], *sp["roc2"], *sp["c"])]
            if sp.get("coefs"):
                cmd += [repr(float(x)) for x in sp["coefs"]]
        env = dict(os.environ, OMP_NUM_THREADS="2", GIRIH_REF_SOURCE="1" if source else "0")
        res = subprocess.run(cmd, check=True, capture_output=True, text=True, env=env)
        tok = res.stdout.split()
        nnx, nny, nnz = int(tok[1]), int(tok[2]), int(tok[3])
        pt = [int(x) for x in tok[7:10]]
        raw = np.fromfile(out, dtype=np.float64)
        n = nnx * nny * nnz
        assert raw.size == 2 * n
        return raw[:n].reshape(nnz, nny, nnx), raw[n:].reshape(nnz, nny, nnx), pt


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: make -C oracle ref")
    arrays, specs = {}, {}
    for (name, op, nx, ny, nz, nt, init, sp), source in ([(c, False) for c in CASES] +
                                                          [(c, True) for c in SOURCE_CASES]):
        u1, u2, pt = run_case(op, nx, ny, nz, nt, init, sp, source)
        arrays[name + "__U1"] = u1
        arrays[name + "__U2"] = u2
        specs[name] = dict(op=op, nx=nx, ny=ny, nz=nz, nt=nt, init=init, seeded=sp)
        if source:
            specs[name]["source_pt"] = pt  # (i, j, k) array indices; values source[i] = i
        print(f"{name}: ldomain {u1.shape[::-1]}")
    arrays["specs"] = np.frombuffer(json.dumps(specs).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "golden_ref.npz"), **arrays)


if __name__ == "__main__":
    main()
