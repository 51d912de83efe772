"""The benchmark workloads as parity cases (reduced sizes where the CPU oracle
must follow), plus size-independent properties at the full 512^3 size.

star7 Jacobi 128^3: operator 1, nt=50, seed 0, U(0,1), default coefficients.
star7 leapfrog: operator 8, seed 1, U(0,1) -- 512^3 / nt=500 in the bench;
          96^3 / nt=100 here against the oracle, and exact power-of-two
          linearity at 512^3.
star25 leapfrog: operator 0, seed 2, U(-1,1), stable 8th-order weights, roc2
          U(0.05,0.15); 72^3 here, errors reported at nt = 50 (and 100 for FP32).
variable coefficients: operators 5 and 4, seed 3, coefficients U(0.01, 0.1/r);
          48^3 here.
"""
import numpy as np
import pytest

from girih_gb300 import gpu
from gpu_helpers import LAP2, LAP8, gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

import oracle


def _seeded(op, n, seed, f, roc2=(0.0, 0.0), c=(0.0, 0.0), coefs=None):
    g = oracle.Grid(op, n, n, n)
    g.fill_seeded(seed, f, roc2, c, coefs=coefs, f32_exact=True, nthreads=4)
    if not g.coef_arrays and coefs is None:
        g.coef[:] = g.default_coefs()
    return g


def test_star7_jacobi_128_exact_fp64_bit_identical():
    g = _seeded(1, 128, 0, (0.0, 1.0))
    with gpu_context(g.copy(), precision="fp64", exact=True) as ctx:
        ctx.run(50)
        u1, u2 = ctx.download()
    g.run(50, nthreads=8)
    np.testing.assert_array_equal(u1, g.U1)
    np.testing.assert_array_equal(u2, g.U2)


def test_star7_leapfrog_reduced_all_forms():
    g0 = _seeded(8, 96, 1, (0.0, 1.0), roc2=(0.5, 1.5), coefs=LAP2)
    ref = g0.copy().run(100, nthreads=8)
    for prec, sched, tol in (("fp64", "plain", 1e-12), ("fp64", "fused", 1e-12), ("fp64df", "fused", 1e-12),
                             ("mixed", "fused", 1e-5)):
        with gpu_context(g0.copy(), precision=prec, schedule=sched) as ctx:
            ctx.run(100)
            u1, _ = ctx.download()
        err = max_rel(u1, ref.U1, ref)
        assert err <= tol, (prec, sched, err)


@pytest.mark.parametrize("prec,sched,tol", [("fp64", "plain", 1e-12), ("fp64", "fused", 1e-12),
                                            ("fp32", "fused", 1e-5), ("mixed", "fused", 1e-5)])
def test_star25_leapfrog_reduced(prec, sched, tol):
    g0 = _seeded(0, 72, 2, (-1.0, 1.0), roc2=(0.05, 0.15), coefs=LAP8)
    ref = g0.copy()
    with gpu_context(g0.copy(), precision=prec, schedule=sched) as ctx:
        for nt in (50, 50):  # checkpoints at nt = 50 and 100
            ctx.run(nt)
            ref.run(nt, nthreads=8)
            u1, _ = ctx.download()
            err = max_rel(u1, ref.U1, ref)
            assert err <= tol, (prec, sched, err)


@pytest.mark.parametrize("op", [5, 4])
def test_var_coef_reduced(op):
    r = gpu.OP_INFO[op][0]
    g0 = _seeded(op, 48, 3, (0.0, 1.0), c=(0.01, 0.1 / r))
    ref = g0.copy().run(20, nthreads=8)
    with gpu_context(g0.copy(), precision="fp64") as ctx:
        ctx.run(20)
        u1, _ = ctx.download()
    assert max_rel(u1, ref.U1, ref) <= 1e-12
    with gpu_context(g0.copy(), precision="mixed") as ctx:
        ctx.run(20)
        u1, _ = ctx.download()
    err = max_rel(u1, ref.U1, ref)
    assert err < 1e-2  # BF16 coefficients: 2^-9 relative quantisation per coefficient


@pytest.mark.parametrize("prec,sched", [("fp64", "plain"), ("mixed", "fused")])
def test_fullsize_power_of_two_linearity(prec, sched):
    """The leapfrog operator is linear in (u, v): doubling the fields doubles
    every value exactly (scaling by 2 commutes with rounding), at 512^3."""
    n, nt = 512, 6
    outs = []
    for scale in (1.0, 2.0):
        with gpu.Context(8, n, n, n, precision=prec, schedule=sched) as ctx:
            ctx.fill_seeded(1, (0.0, scale), (0.5, 1.5), coefs=LAP2, f32_exact=True)
            ctx.run(nt)
            u1 = np.zeros(ctx.shape, np.float64)
            ctx.download(u1, None)
            outs.append(u1)
    np.testing.assert_array_equal(outs[1], 2.0 * outs[0])
    assert np.abs(outs[0]).max() > 0.1  # not a vacuous comparison
