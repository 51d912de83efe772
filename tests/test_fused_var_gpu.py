"""Time-fused kernels of the variable-coefficient operators (2, 3, 4, 5).

These operators read nc coefficient arrays per update (src/kernels/
stencils_spt_blk.ic, the `coef` loops of operators 2-5), so their plain sweep moves
8 + 4*nc bytes per FP32 update; a fused pass of depth T reads each coefficient
once per T steps.  Fusion is provided for FP32 fields with FP32 coefficients
("fp32") and with BF16 coefficients plus a per-array scale ("mixed").  The
fused FP32 result is held to the plain FP32 kernel's error against the FP64
oracle; the fused mixed result to the plain mixed kernel, which uses the same
BF16 coefficients.
"""
import numpy as np
import pytest

from girih_gb300 import gpu
from gpu_helpers import bf16_quantized_coefs, fused_block, gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

VAR_OPS = [2, 3, 4, 5]


def _shape(op):
    return (70, 53, 41) if gpu.OP_INFO[op][0] == 1 else (61, 37, 29)


def _max_depth(op):
    return 2 if gpu.OP_INFO[op][0] == 4 else 3


def _plain(g0, precision, nt):
    with gpu_context(g0.copy(), precision=precision, schedule="plain") as pc:
        pc.run(nt)
        return pc.download()


@pytest.mark.parametrize("op", VAR_OPS)
@pytest.mark.parametrize("variant", [0, 1])
def test_fused_var_fp32_all_depths(op, variant):
    g0 = oracle_grid(op, *_shape(op), seed=21)
    nt = 11
    ref = g0.copy().run(nt, nthreads=4)
    plain_u1, _ = _plain(g0, "fp32", nt)
    plain_err = max_rel(plain_u1, ref.U1, ref)
    r = gpu.OP_INFO[op][0]
    w, h = (64, 32) if variant == 0 else (32, 64)
    for depth in range(1, _max_depth(op) + 1):
        block = fused_block(r, w, h, depth, 2 if r == 1 else 1)
        g = g0.copy()
        with gpu_context(g, precision="fp32", schedule="fused", fusion_depth=depth, block=block) as ctx:
            info = ctx.info()
            assert info["schedule"] == gpu.FUSED and info["fusion_depth"] == depth
            ctx.run(nt)
            assert ctx.info()["launches_last_run"] == -(-12 // depth)
            u1, u2 = ctx.download()
        err = max_rel(u1, ref.U1, ref)
        assert err < max(4 * plain_err, 2e-6), (depth, err, plain_err)
        assert max_rel(u2, ref.U2, ref) < max(4 * plain_err, 2e-6), depth
        # halos and x padding are never written (the FP32 state holds the rounded inputs)
        h0 = g0.U1.astype(np.float32).astype(np.float64)
        np.testing.assert_array_equal(u1[:, :, g.nx + 2 * r:], h0[:, :, g.nx + 2 * r:])
        np.testing.assert_array_equal(u1[:r], h0[:r])
        np.testing.assert_array_equal(u1[:, :r], h0[:, :r])


@pytest.mark.parametrize("op", VAR_OPS)
def test_fused_var_mixed_matches_plain_mixed(op):
    g0 = oracle_grid(op, *_shape(op), seed=22)
    nt = 10
    ref = g0.copy().run(nt, nthreads=4)
    # the FP64 oracle with the mixed form's own (BF16-quantised) coefficients
    refq = g0.copy()
    refq.coef[...] = bf16_quantized_coefs(g0)
    refq.run(nt, nthreads=4)
    plain_u1, _ = _plain(g0, "mixed", nt)
    p32_u1, _ = _plain(g0, "fp32", nt)
    fp32_err = max_rel(p32_u1, ref.U1, ref)
    mixed_err = max_rel(plain_u1, ref.U1, ref)
    assert max_rel(plain_u1, refq.U1, refq) < max(4 * fp32_err, 2e-6)
    for depth in range(1, _max_depth(op) + 1):
        with gpu_context(g0.copy(), precision="mixed", schedule="fused", fusion_depth=depth) as ctx:
            assert ctx.info()["bytes_per_lup"] == 8 + 2 * gpu.OP_INFO[op][2]
            ctx.run(nt)
            u1, _ = ctx.download()
        # same BF16 coefficients: the two kernels differ by FP32 rounding only, and
        # both sit within FP32 arithmetic error of the FP64 oracle with those coefficients
        assert max_rel(u1, plain_u1, ref) < max(4 * fp32_err, 2e-6), depth
        assert max_rel(u1, refq.U1, refq) < max(4 * fp32_err, 2e-6), depth
        assert max_rel(u1, ref.U1, ref) < 2 * mixed_err + 1e-6, depth


@pytest.mark.parametrize("op", VAR_OPS)
@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 70, 2), (90, 2, 9), (64, 32, 5)])
def test_fused_var_edge_shapes(op, shape):
    g0 = oracle_grid(op, *shape, seed=23)
    nt = 5
    ref = g0.copy().run(nt)
    plain_u1, _ = _plain(g0, "fp32", nt)
    plain_err = max_rel(plain_u1, ref.U1, ref)
    for depth in (1, _max_depth(op)):
        with gpu_context(g0.copy(), precision="fp32", schedule="fused", fusion_depth=depth) as ctx:
            ctx.run(nt)
            u1, _ = ctx.download()
        assert max_rel(u1, ref.U1, ref) < max(4 * plain_err, 2e-6), (shape, depth)


def test_fused_var_fp64_stays_plain():
    """FP64 variable-coefficient operators run the plain kernel: fusion is not
    provided there, and an explicit fused request is refused."""
    with pytest.raises(gpu.GirihGpuError):
        gpu.Context(2, 40, 30, 20, precision="fp64", schedule="fused")
    with gpu.Context(2, 40, 30, 20, precision="fp64", schedule="auto") as ctx:
        assert ctx.info()["schedule"] == gpu.PLAIN


@pytest.mark.parametrize("op", VAR_OPS)
def test_autotune_var_ops(op):
    g0 = oracle_grid(op, 96, 64, 48, seed=24)
    nt = 6
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision="fp32", schedule="auto") as ctx:
        ctx.autotune(trial_steps=2)
        np.testing.assert_array_equal(ctx.download()[0], g0.U1.astype(np.float32).astype(np.float64))  # restored
        ctx.run(nt)
        u1, _ = ctx.download()
    plain_u1, _ = _plain(g0, "fp32", nt)
    assert max_rel(u1, ref.U1, ref) < max(4 * max_rel(plain_u1, ref.U1, ref), 2e-6)
