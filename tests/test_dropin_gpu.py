"""The reference-side drop-in on the GPU: the girih driver built from the
reference's own objects (girih_gb300/host/_build/mwd_kernel_gpu) with the GPU
stepper as --target-ts 3, calling the real libgirih_gpu.so.

  * --verify 1 runs the reference's own verifier (src/verification.c:26-51): the
    GPU stepper's U1 after nt steps against the reference's serial operators,
    bit for bit (src/verification.c:842-849).  The stepper's default form,
    plain FP64 with the serial reference's rounding, passes it for every
    regular operator, the 27-point box included.
  * a performance run goes through the reference's performance_test
    (src/performance.c:28-127, timing around the stepper call) and prints the
    reference's report plus scripts/parse.py's keys and the stepper's JSON line.

Needs the reference sources to build the driver (the tree GIRIH_REF names, or
the copy staged in baseline/_ref/girih)."""
import json
import os
import re
import subprocess

import pytest

from __graft_entry__ import reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "girih_gb300", "host", "_build", "mwd_kernel_gpu")
REF = reference_tree()

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(REF is None, reason="reference sources not present")]


@pytest.fixture(scope="module")
def driver():
    jobs = f"-j{min(16, os.cpu_count() or 4)}"
    subprocess.run(["make", "-s", jobs, "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "girih_gb300", "host"), f"REF={REF}"], check=True)
    return EXE


def _run(driver, args, tmp_path, **env):
    e = dict(os.environ, OMP_NUM_THREADS="4", **env)
    # a failed verification writes error snapshots into the working directory
    return subprocess.run([driver] + [str(a) for a in args], capture_output=True, text=True, env=e,
                          cwd=str(tmp_path), timeout=300)


@pytest.mark.parametrize("kernel,shape,nt", [(1, (20, 14, 12), 6), (0, (21, 13, 11), 6), (2, (19, 12, 10), 4),
                                            (3, (19, 12, 10), 4), (4, (17, 12, 10), 4), (5, (20, 14, 12), 5),
                                            (7, (18, 13, 11), 4), (1, (64, 48, 40), 10)])
def test_reference_verifier_passes_gpu_stepper(driver, tmp_path, kernel, shape, nt):
    nx, ny, nz = shape
    r = _run(driver, ["--nx", nx, "--ny", ny, "--nz", nz, "--nt", nt, "--target-kernel", kernel,
                      "--target-ts", 3, "--verify", 1], tmp_path)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "-PASSED" in r.stdout and "eMax:0.000e+00" in r.stdout


def _report(stdout):
    keys = {}
    for line in stdout.splitlines():
        m = re.match(r"^(RANK0 MStencil/s  (MIN|AVG|MAX)|Time stepper name|Number of time steps|Number of tests):(.*)$",
                     line)
        if m:
            keys[m.group(1)] = m.group(3).strip()
    js = [ln.split("GPU stepper JSON: ", 1)[1] for ln in stdout.splitlines() if ln.startswith("GPU stepper JSON: ")]
    return keys, (json.loads(js[0]) if len(js) == 1 else None)


@pytest.mark.parametrize("kernel,precision,schedule", [(1, "fp64", "plain"), (1, "fp64df", "fused"),
                                                       (0, "mixed", "fused"), (0, "fp64df", "fused"),
                                                       (5, "mixed", "plain"), (7, "fp64", "plain"),
                                                       (7, "fp64df", "fused")])
def test_performance_run_reports_parse_py_keys(driver, tmp_path, kernel, precision, schedule):
    """The reference's performance harness timing the GPU stepper in each form
    (operator 8 has no reference id, so the reference CLI cannot name it)."""
    r = _run(driver, ["--nx", 96, "--ny", 96, "--nz", 96, "--nt", 20, "--target-kernel", kernel, "--target-ts", 3,
                      "--n-tests", 3], tmp_path, GIRIH_GPU_PRECISION=precision, GIRIH_GPU_SCHEDULE=schedule)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    keys, js = _report(r.stdout)
    assert keys["Time stepper name"] == "GPU (libgirih_gpu)"
    assert int(keys["Number of time steps"]) == 20 and int(keys["Number of tests"]) == 3
    mn, avg, mx = (float(keys[f"RANK0 MStencil/s  {k}"].split()[0]) for k in ("MIN", "AVG", "MAX"))
    assert 0 < mn <= avg * 1.0001 <= mx * 1.0002
    assert js is not None and js["calls"] == 3 and js["target_kernel"] == kernel
    assert js["precision"] == precision and js["schedule"] == schedule
    assert js["glups_device_max"] > 0
    if (kernel, precision) == (0, "fp64df"):  # the TMA-staged one-step pass of the 25-point operator
        assert js["kernel"] == "fused_df_tma" and js["fusion_depth"] == 1
