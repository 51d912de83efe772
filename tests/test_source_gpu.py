"""Source-point injection on the GPU (src/kernels/nb_naive_ts.c:190,196).

After sweep s of a run the updated array gets source[s] added at one interior
point.  The plain FP64 schedule in exact mode reproduces the reference's own
source runs bit for bit (golden cases with the reference's centred point and
source[i] = i); every fused form is held to its usual bound against the oracle,
with the point placed inside tiles, on tile edges and at the domain corners.
"""
import json
import os

import numpy as np
import pytest

from girih_gb300 import gpu
from gpu_helpers import gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")


def _golden():
    d = np.load(GOLD)
    specs = json.loads(bytes(d["specs"]).decode())
    return d, {k: v for k, v in specs.items() if "source_pt" in v}


@pytest.mark.parametrize("name", sorted(_golden()[1]))
def test_plain_exact_matches_reference_source_runs(name):
    import oracle
    d, specs = _golden()
    s = specs[name]
    g = oracle.Grid(s["op"], s["nx"], s["ny"], s["nz"])
    if s["init"] == "ref":
        g.fill_ref()
    else:
        sp = s["seeded"]
        g.fill_seeded(sp["seed"], tuple(sp["f"]), tuple(sp["roc2"]), tuple(sp["c"]), coefs=sp.get("coefs"))
        if not g.coef_arrays and not sp.get("coefs"):
            g.coef[:] = g.default_coefs()
    with gpu_context(g, precision="fp64", schedule="plain", exact=True) as ctx:
        ctx.set_source(s["source_pt"], np.arange(s["nt"], dtype=np.float64))
        ctx.run(s["nt"])
        u1, u2 = ctx.download()
    np.testing.assert_array_equal(u1, d[name + "__U1"])
    np.testing.assert_array_equal(u2, d[name + "__U2"])


def _points(g):
    r = g.r
    return [
        (g.nx // 2 + r, g.ny // 2 + r, g.nz // 2 + r),      # inside
        (r, r, r),                                           # first interior corner
        (g.nx - 1 + r, g.ny - 1 + r, g.nz - 1 + r),          # last interior corner
        (min(g.nx - 1, 59) + r, min(g.ny - 1, 27) + r, r + 1),  # near a 60 x 28 tile edge
    ]


FORMS = [("fp64", "fused", 1e-12), ("fp64df", "fused", 1e-12), ("fp32", "fused", None), ("mixed", "fused", None)]


@pytest.mark.parametrize("op", [1, 8, 0])
@pytest.mark.parametrize("form", FORMS, ids=[f[0] for f in FORMS])
def test_fused_source_point(op, form):
    precision, sched, tol = form
    shape = (70, 53, 41) if gpu.OP_INFO[op][0] == 1 else (61, 37, 29)
    nt = 9  # odd: the extra sweep has no source value
    rng = np.random.default_rng(5)
    vals = rng.uniform(0.5, 1.5, nt)
    g0 = oracle_grid(op, *shape, seed=31)
    plain_ref = g0.copy().run(nt, nthreads=4)
    for pt in _points(g0):
        ref = g0.copy().run_source(nt, pt, vals, nthreads=4)
        depths = range(1, 3) if precision == "fp64" or gpu.OP_INFO[op][0] == 4 else range(1, 4)
        for depth in depths:
            with gpu_context(g0.copy(), precision=precision, schedule=sched, fusion_depth=depth) as ctx:
                ctx.set_source(pt, vals)
                ctx.run(nt)
                u1, u2 = ctx.download()
            e1, e2 = max_rel(u1, ref.U1, ref), max_rel(u2, ref.U2, ref)
            if tol is None:  # FP32 storage: the error of the same form without a source, with margin
                with gpu_context(g0.copy(), precision=precision, schedule=sched, fusion_depth=depth) as c2:
                    c2.run(nt)
                    base = max(max_rel(c2.download()[1], plain_ref.U2, plain_ref), 1e-7)
                bound = 4 * base
            else:
                bound = tol
            assert e1 <= bound and e2 <= bound, (pt, depth, e1, e2, bound)
            # the source changed the result at the point
            i, j, k = pt
            assert u2[k, j, i] != plain_ref.U2[k, j, i]


@pytest.mark.parametrize("precision", ["fp64", "fp32", "mixed"])
def test_plain_source_point_var_operator(precision):
    op = 5
    g0 = oracle_grid(op, 40, 24, 20, seed=32)
    nt = 6
    vals = np.linspace(0.1, 0.6, nt)
    pt = (10, 7, 5)
    ref = g0.copy().run_source(nt, pt, vals, nthreads=4)
    with gpu_context(g0.copy(), precision=precision, schedule="plain", exact=precision == "fp64") as ctx:
        ctx.set_source(pt, vals)
        ctx.run(nt)
        u1, u2 = ctx.download()
    if precision == "fp64":
        np.testing.assert_array_equal(u2, ref.U2)
    else:
        assert max_rel(u2, ref.U2, ref) < (1e-2 if precision == "mixed" else 1e-5)


def test_source_restarts_each_run_and_can_be_switched_off():
    op = 8
    g0 = oracle_grid(op, 50, 40, 30, seed=33)
    vals = np.array([1.0, -0.5, 0.25, 2.0])
    pt = (20, 11, 9)
    ref = g0.copy()
    ref.run_source(4, pt, vals, nthreads=4)
    ref.run_source(4, pt, vals, nthreads=4)  # each run starts at sweep 0 again
    ref.run(4, nthreads=4)                   # then without the source
    with gpu_context(g0.copy(), precision="fp64", schedule="fused", fusion_depth=2) as ctx:
        ctx.set_source(pt, vals)
        ctx.run(4)
        ctx.run(4)
        ctx.set_source(None, None)
        ctx.run(4)
        u1, u2 = ctx.download()
    assert max_rel(u2, ref.U2, ref) <= 1e-12
    assert max_rel(u1, ref.U1, ref) <= 1e-12


def test_source_point_must_be_interior():
    with gpu.Context(1, 20, 20, 20) as ctx:
        for pt in [(0, 5, 5), (5, 21, 5), (5, 5, -1)]:
            with pytest.raises(gpu.GirihGpuError) as e:
                ctx.set_source(pt, [1.0])
            assert e.value.code == 1
