"""Time-fused passes of the 27-point box operator (operator 7, the reference's
box_ref_2space_1time, src/kernels/stencils.c:227-242).

The fused box kernel evaluates the operator through per-plane partial sums of
the in-plane face and diagonal neighbours (fused_box.cu), an association order
of its own, so it is held to the FP64 parity bound (1e-12 max-norm relative)
in FP64 and double-float, and to the plain FP32 kernel's error in FP32,
against the oracle's serial operator -- on ragged shapes, every depth and both
tile variants, with halos and padding never written.
"""
import numpy as np
import pytest

from girih_gb300 import gpu
from gpu_helpers import gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
OP = 7
# region of each tile variant: 32 x 32 and 64 x 16; the halo is one column per level
REGION = {0: (32, 32), 1: (64, 16)}
DEPTHS = {"fp64": 2, "fp32": 4, "mixed": 4, "fp64df": 3}


def _block(variant, depth):
    w, h = REGION[variant]
    return (w - 2 * depth, h - 2 * depth)


def _depths(precision, variant):
    top = DEPTHS[precision]
    if precision == "fp64df" and variant == 1:
        top = 2
    return [d for d in range(1, top + 1) if REGION[variant][1] - 2 * d > 0]


@pytest.mark.parametrize("precision", ["fp64", "fp64df"])
@pytest.mark.parametrize("variant", [0, 1])
def test_fused_box_fp64_forms_within_parity_bound(precision, variant):
    g0 = oracle_grid(OP, 45, 37, 29, seed=31)
    nt = 9
    ref = g0.copy().run(nt, nthreads=4)
    r = g0.r
    for depth in _depths(precision, variant):
        with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth,
                         block=_block(variant, depth)) as ctx:
            info = ctx.info()
            assert info["schedule"] == gpu.FUSED and info["fusion_depth"] == depth
            assert info["kernel_name"] == "fused_box_pass"
            ctx.run(nt)
            u1, u2 = ctx.download()
        assert max_rel(u1, ref.U1, ref) <= FP64_TOL, (depth, max_rel(u1, ref.U1, ref))
        assert max_rel(u2, ref.U2, ref) <= FP64_TOL, depth
        # halos and padding are never written
        np.testing.assert_array_equal(u1[:, :, g0.nx + 2 * r:], g0.U1[:, :, g0.nx + 2 * r:])
        np.testing.assert_array_equal(u1[:r], g0.U1[:r])
        np.testing.assert_array_equal(u1[:, :r], g0.U1[:, :r])
        np.testing.assert_array_equal(u1[:, :, :r], g0.U1[:, :, :r])


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("variant", [0, 1])
def test_fused_box_fp32_against_fp64_oracle(precision, variant):
    g0 = oracle_grid(OP, 45, 37, 29, seed=32)
    nt = 12
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision="fp32", schedule="plain") as pc:
        pc.run(nt)
        plain_u1, _ = pc.download()
    plain_err = max_rel(plain_u1, ref.U1, ref)
    for depth in _depths(precision, variant):
        with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth,
                         block=_block(variant, depth)) as ctx:
            ctx.run(nt)
            u1, _ = ctx.download()
        err = max_rel(u1, ref.U1, ref)
        assert err < max(4 * plain_err, 2e-6), (depth, err, plain_err)


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 70, 2), (90, 2, 9), (64, 32, 5), (31, 29, 40)])
@pytest.mark.parametrize("precision", ["fp64", "fp64df"])
def test_fused_box_edge_shapes(shape, precision):
    g0 = oracle_grid(OP, *shape, seed=33)
    nt = 5
    ref = g0.copy().run(nt)
    for depth in (1, 2):
        with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth) as ctx:
            ctx.run(nt)
            u1, u2 = ctx.download()
        assert max_rel(u1, ref.U1, ref) <= FP64_TOL, (shape, depth)
        assert max_rel(u2, ref.U2, ref) <= FP64_TOL, (shape, depth)


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_fused_box_source_point(precision):
    """The reference's source-point update (src/kernels/nb_naive_ts.c:190,196)
    in the fused box passes, at a tile edge and in the interior."""
    g0 = oracle_grid(OP, 40, 33, 21, seed=34)
    nt = 7
    src = np.linspace(0.5, 3.5, nt + 1)
    for pt in ((1 + 30, 1 + 28, 1 + 10), (1 + 5, 1 + 17, 1 + 3)):
        ref = g0.copy()
        ref.run_source(nt, pt, src, nthreads=4)
        with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=2) as ctx:
            ctx.set_source(pt, src)
            ctx.run(nt)
            u1, u2 = ctx.download()
        tol = FP64_TOL if precision != "fp32" else 5e-6
        assert max_rel(u1, ref.U1, ref) <= tol, (pt, max_rel(u1, ref.U1, ref))
        assert max_rel(u2, ref.U2, ref) <= tol, pt


def test_fused_box_autotune_and_auto_schedule():
    g0 = oracle_grid(OP, 96, 64, 48, seed=35)
    nt = 6
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision="fp64df", schedule="auto") as ctx:
        ctx.autotune(trial_steps=2)
        np.testing.assert_array_equal(ctx.download()[0], g0.U1)  # the grid state is restored
        ctx.run(nt)
        u1, _ = ctx.download()
    assert max_rel(u1, ref.U1, ref) <= FP64_TOL
