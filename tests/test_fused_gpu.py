"""Parity of the time-fused (temporally blocked) GPU kernels with the oracle.

FP64 fused passes use FMA contraction, so they are held to the FP64 parity
bound (max-norm relative <= 1e-12) rather than bit equality.  Every fusion
depth and both tile variants are exercised on grids that are not multiples of
the tile, with odd nt (the reference rounds nt up to even) and with nt not a
multiple of the depth (a shorter final pass).
"""
import numpy as np
import pytest

from girih_gb300 import gpu
from gpu_helpers import fused_block, gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FUSED_OPS = [1, 8, 0]
MAX_DEPTH = {("fp64", 1): 2, ("fp64", 4): 2, ("fp32", 1): 4, ("fp32", 4): 2, ("mixed", 1): 4, ("mixed", 4): 2}
TILE = {0: (64, 32), 1: (32, 64)}  # column region of the CTA variants
SMEM_MAX = 227 * 1024


def _block(op, depth, variant):
    r = gpu.OP_INFO[op][0]
    w, h = TILE[variant]
    return fused_block(r, w, h, depth, 2 if r == 1 else 1)  # radius 1: x pairs, 2-column alignment


def _fits(variant, depth, tsz):
    w, h = TILE[variant]
    return 2 * depth * w * h * tsz <= SMEM_MAX


def _shape(op):
    return (70, 53, 41) if gpu.OP_INFO[op][0] == 1 else (61, 37, 29)


@pytest.mark.parametrize("op", FUSED_OPS)
@pytest.mark.parametrize("variant", [0, 1])
def test_fused_fp64_all_depths(op, variant):
    r = gpu.OP_INFO[op][0]
    g0 = oracle_grid(op, *_shape(op), seed=7)
    nt = 9
    ref = g0.copy().run(nt, nthreads=4)
    for depth in range(1, MAX_DEPTH[("fp64", r)] + 1):
        if not _fits(variant, depth, 8):
            with pytest.raises(gpu.GirihGpuError):
                gpu.Context(op, *_shape(op), schedule="fused", fusion_depth=depth, block=_block(op, depth, variant))
            continue
        g = g0.copy()
        with gpu_context(g, precision="fp64", schedule="fused", fusion_depth=depth,
                         block=_block(op, depth, variant)) as ctx:
            info = ctx.info()
            assert info["schedule"] == gpu.FUSED and info["fusion_depth"] == depth
            ctx.run(nt)
            assert ctx.info()["launches_last_run"] == -(-10 // depth)
            u1, u2 = ctx.download()
        assert max_rel(u1, ref.U1, ref) <= FP64_TOL, (depth, max_rel(u1, ref.U1, ref))
        assert max_rel(u2, ref.U2, ref) <= FP64_TOL, depth
        # halos and padding are never written
        np.testing.assert_array_equal(u1[:, :, g.nx + 2 * r:], g0.U1[:, :, g.nx + 2 * r:])
        np.testing.assert_array_equal(u1[:r], g0.U1[:r])


@pytest.mark.parametrize("op", FUSED_OPS)
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_fused_fp32_against_fp64_oracle(op, precision):
    r = gpu.OP_INFO[op][0]
    g0 = oracle_grid(op, *_shape(op), seed=8)
    nt = 12
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision="fp32", schedule="plain") as pc:
        pc.run(nt)
        plain_u1, _ = pc.download()
    plain_err = max_rel(plain_u1, ref.U1, ref)
    for depth in range(1, MAX_DEPTH[(precision, r)] + 1):
        with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth) as ctx:
            ctx.run(nt)
            u1, _ = ctx.download()
        err = max_rel(u1, ref.U1, ref)
        # same order of error as the plain FP32 kernel (inputs are FP32-representable)
        assert err < max(4 * plain_err, 2e-6), (depth, err, plain_err)


@pytest.mark.parametrize("op", FUSED_OPS)
@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 70, 2), (90, 2, 9), (64, 32, 5)])
def test_fused_edge_shapes(op, shape):
    g0 = oracle_grid(op, *shape, seed=9)
    nt = 5
    ref = g0.copy().run(nt)
    r = gpu.OP_INFO[op][0]
    for depth in (1, MAX_DEPTH[("fp64", r)]):
        with gpu_context(g0.copy(), precision="fp64", schedule="fused", fusion_depth=depth) as ctx:
            ctx.run(nt)
            u1, u2 = ctx.download()
        assert max_rel(u1, ref.U1, ref) <= FP64_TOL
        assert max_rel(u2, ref.U2, ref) <= FP64_TOL


def test_fused_reference_init_and_nt0():
    g0 = oracle_grid(1, 40, 30, 20)  # reference ramp + boundary sources
    with gpu_context(g0.copy(), schedule="fused", fusion_depth=3) as ctx:
        ctx.run(0)
        u1, u2 = ctx.download()
        np.testing.assert_array_equal(u1, g0.U1)
        ctx.run(8)
        ctx.run(6)
        u1, u2 = ctx.download()
    ref = g0.copy().run(14)
    assert max_rel(u1, ref.U1, ref) <= FP64_TOL
    assert max_rel(u2, ref.U2, ref) <= FP64_TOL


def test_fused_requires_equal_halos():
    g = oracle_grid(8, 20, 20, 20, seed=1)
    g.U1[0, 0, 0] += 1.0  # U1 halo differs from U2's
    ctx = gpu.Context(8, 20, 20, 20, schedule="fused")
    with pytest.raises(gpu.GirihGpuError) as e:
        ctx.upload(g.U1, g.U2, g.U3, g.coef)
    assert e.value.code == 2
    ctx.close()
    # the plain schedule keeps the exact ping-pong semantics for unequal halos
    with gpu_context(g.copy(), schedule="plain", exact=True) as ctx:
        ctx.run(4)
        u1, _ = ctx.download()
    np.testing.assert_array_equal(u1, g.copy().run(4).U1)


def test_auto_schedule_untuned_defaults():
    """Untuned auto: fused where it measured faster (FP32 fields, radius-1 constant
    operators; double-float), plain elsewhere (FP64 arithmetic, radius 4,
    variable coefficients)."""
    for op, prec, want in ((1, "fp64", gpu.PLAIN), (8, "fp64", gpu.PLAIN), (0, "fp64", gpu.PLAIN),
                           (8, "fp64df", gpu.FUSED), (0, "fp64df", gpu.FUSED), (1, "mixed", gpu.FUSED),
                           (8, "mixed", gpu.FUSED),
                           (8, "fp32", gpu.FUSED), (0, "mixed", gpu.PLAIN),
                           (5, "fp64", gpu.PLAIN), (5, "mixed", gpu.PLAIN), (4, "mixed", gpu.PLAIN)):
        with gpu.Context(op, 32, 32, 32, precision=prec, schedule="auto") as ctx:
            assert ctx.info()["schedule"] == want, (op, prec)


@pytest.mark.parametrize("op,precision,sched", [(8, "mixed", "fused"), (1, "fp64", "auto"), (0, "fp32", "fused")])
def test_autotune_restores_state_and_stays_correct(op, precision, sched):
    g0 = oracle_grid(op, *_shape(op), seed=4)
    nt = 10
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision=precision, schedule=sched) as ctx:
        chosen = ctx.autotune(trial_steps=6)
        u1, u2 = ctx.download()
        np.testing.assert_array_equal(u1, g0.U1.astype(np.float32).astype(np.float64) if precision != "fp64" else g0.U1)
        assert chosen["schedule"] in (gpu.PLAIN, gpu.FUSED)
        ctx.run(nt)
        u1, _ = ctx.download()
    tol = FP64_TOL if precision == "fp64" else 5e-6
    assert max_rel(u1, ref.U1, ref) <= tol
    # a later context of the same operator, precision and size class reuses the choice
    with gpu.Context(op, *_shape(op), precision=precision, schedule=sched) as ctx2:
        i2 = ctx2.info()
        assert (i2["schedule"], i2["fusion_depth"]) == (chosen["schedule"], chosen["fusion_depth"])


@pytest.mark.parametrize("op", FUSED_OPS)
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_fused_double_float_within_fp64_bound(op, variant):
    """FP64 storage, double-float arithmetic: held to the FP64 parity bound."""
    r = gpu.OP_INFO[op][0]
    g0 = oracle_grid(op, *_shape(op), seed=17)
    nt = 9
    ref = g0.copy().run(nt, nthreads=4)
    # double-float regions: one column per thread (0-2), x pairs (3, 4); the output tile
    # keeps the general width w - 2H - (group - 1)
    w, h, grp = {0: (64, 32, 1), 1: (32, 32, 1), 2: (64, 16, 1), 3: (64, 32, 2), 4: (32, 64, 2)}[variant]
    if variant >= 2 and r != 1:
        return  # radius 1 only
    for depth in range(1, (3 if r == 1 else 2) + 1):
        if h - 2 * depth * r <= 0:
            continue
        with gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=depth,
                         block=(w - 2 * depth * r - (grp - 1), h - 2 * depth * r)) as ctx:
            ctx.run(nt)
            # the passes, plus the FP64 -> pair splits and the pair -> FP64 joins of the run
            split_join = (3 if gpu.OP_INFO[op][1] == 2 else 2) + 2
            assert ctx.info()["launches_last_run"] == -(-10 // depth) + split_join
            u1, u2 = ctx.download()
        assert max_rel(u1, ref.U1, ref) <= FP64_TOL, (depth, max_rel(u1, ref.U1, ref))
        assert max_rel(u2, ref.U2, ref) <= FP64_TOL, depth
        # the FP64 halos are kept bit for bit
        np.testing.assert_array_equal(u1[:r], g0.U1[:r])
        np.testing.assert_array_equal(u2[:, :r], g0.U2[:, :r])
        np.testing.assert_array_equal(u1[:, :, :r], g0.U1[:, :, :r])


@pytest.mark.parametrize("op", [1, 8])
@pytest.mark.parametrize("variant", [5, 6])
def test_fused_double_float_tma_equals_register_kernel(op, variant):
    """The TMA-staged double-float kernel (variants 5 and 6: 32 x 32 and 64 x 32
    regions, two adjacent rows per thread) performs the register
    kernel's arithmetic in the same order: results bit-identical to variant 4
    (32 x 64 region with x pairs in packed f32x2 lanes, another tiling) at both
    depths, with odd nt (a final pass of depth 1), grids smaller than one box,
    boxes over every domain edge, and several persistent pieces per CTA; held
    to the FP64 bound against the oracle."""
    cols, rows = {5: (32, 32), 6: (64, 32)}[variant]
    for shape in ((45, 38, 29), (5, 3, 4), (70, 2, 9), (97, 130, 67)):
        g0 = oracle_grid(op, *shape, seed=29)
        nt = 9
        ref = g0.copy().run(nt, nthreads=4)
        for depth in (1, 2):
            # boxes start on 16 bytes (2 columns): the aligned width at depth 2, the general one at depth 1
            block = (cols - 2 * depth - (depth % 2), rows - 2 * depth)
            with gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=depth,
                             block=block) as ctx, \
                    gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=depth,
                                block=(32 - 2 * depth - 1, 64 - 2 * depth)) as reg:
                assert ctx.info()["kernel_name"] == "fused_df_tma"
                assert reg.info()["kernel_name"] == "fused_pass"
                ctx.run(nt)
                reg.run(nt)
                u1, u2 = ctx.download()
                r1, r2 = reg.download()
            np.testing.assert_array_equal(u1, r1)
            np.testing.assert_array_equal(u2, r2)
            assert max_rel(u1, ref.U1, ref) <= FP64_TOL
            assert max_rel(u2, ref.U2, ref) <= FP64_TOL


@pytest.mark.parametrize("shape", [(61, 37, 29), (5, 3, 4), (70, 2, 9), (97, 130, 45), (400, 400, 12)])
def test_fused_double_float_tma_radius4_equals_register_kernel(shape):
    """The 25-point leapfrog (operator 0, radius 4) in double-float, one step
    per pass: the TMA-staged kernel (variant 5 of operator 0, a 32 x 32 tile
    with 40 x 40 boxes, fused_df_tma4.cu) performs the register kernel's
    arithmetic in the same order, so results are bit-identical to variant 0
    (64 x 32 region, 56 x 24 tile).  Covered: odd nt, grids smaller than one
    box, boxes over every domain edge, and (400 x 400: 169 tiles for 152
    persistent CTAs) CTAs that take a second piece.  Held to the FP64 bound
    against the oracle."""
    op = 0
    g0 = oracle_grid(op, *shape, seed=41)
    nt = 7 if shape[0] < 400 else 3
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=1, block=(32, 32)) as ctx, \
            gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=1, block=(56, 24)) as reg:
        assert ctx.info()["kernel_name"] == "fused_df_tma"
        assert reg.info()["kernel_name"] == "fused_pass"
        ctx.run(nt)
        reg.run(nt)
        u1, u2 = ctx.download()
        r1, r2 = reg.download()
    np.testing.assert_array_equal(u1, r1)
    np.testing.assert_array_equal(u2, r2)
    assert max_rel(u1, ref.U1, ref) <= FP64_TOL
    assert max_rel(u2, ref.U2, ref) <= FP64_TOL
    # untuned, the double-float form of operator 0 takes this kernel, one step per pass
    with gpu.Context(op, *shape, precision="fp64df", schedule="fused") as ctx:
        info = ctx.info()
        assert (info["kernel_name"], info["fusion_depth"], info["block_x"]) == ("fused_df_tma", 1, 32)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("shape", [(61, 37, 29), (5, 3, 4), (70, 2, 9), (400, 400, 12)])
def test_fused_fp32_tma_radius4_equals_register_kernel(precision, shape):
    """The 25-point leapfrog in FP32 storage, one step per pass: the TMA-staged
    kernel (variant 5 of operator 0, fused_df_tma4.cu; FP32 arithmetic, or the
    compensated leapfrog of the mixed form) performs the register kernel's
    arithmetic in the same order: bit-identical to variant 0 (56 x 24 tile),
    including grids smaller than one box, boxes over every domain edge and
    CTAs that take a second piece (400 x 400)."""
    op = 0
    g0 = oracle_grid(op, *shape, seed=43)
    nt = 7 if shape[0] < 400 else 3
    ref = g0.copy().run(nt, nthreads=4)
    with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=1, block=(32, 32)) as ctx, \
            gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=1, block=(56, 24)) as reg:
        assert ctx.info()["kernel_name"] == "fused_f32_tma4"
        assert reg.info()["kernel_name"] == "fused_pass"
        ctx.run(nt)
        reg.run(nt)
        u1, u2 = ctx.download()
        r1, r2 = reg.download()
    np.testing.assert_array_equal(u1, r1)
    np.testing.assert_array_equal(u2, r2)
    assert max_rel(u1, ref.U1, ref) < 5e-6


def test_fused_double_float_reference_init():
    """The reference ramp + 100.1 boundary sources (operator 1, default coefficients)."""
    g0 = oracle_grid(1, 45, 31, 27)
    ref = g0.copy().run(20)
    with gpu_context(g0.copy(), precision="fp64df", schedule="fused", fusion_depth=3) as ctx:
        ctx.run(20)
        u1, u2 = ctx.download()
    assert max_rel(u1, ref.U1, ref) <= FP64_TOL
    assert max_rel(u2, ref.U2, ref) <= FP64_TOL


def test_fused_double_float_reports_range_overflow():
    g = oracle_grid(1, 20, 20, 20, seed=1)
    g.U1 *= 1e300
    g.U2 *= 1e300
    with gpu_context(g, precision="fp64df", schedule="fused") as ctx:
        with pytest.raises(gpu.GirihGpuError) as e:
            ctx.run(2)
        assert e.value.code == 8


@pytest.mark.parametrize("op", FUSED_OPS)
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
@pytest.mark.parametrize("variant", [2, 3])
def test_fused_tma_variants(op, precision, variant):
    """Input planes staged into shared memory by TMA (cp.async.bulk.tensor):
    same results as the register/global-load variants, every depth, including
    grids smaller than one box and boxes hanging over every domain edge."""
    r = gpu.OP_INFO[op][0]
    w, h = TILE[variant - 2]
    for shape in (_shape(op), (5, 3, 4), (70, 2, 9)):
        g0 = oracle_grid(op, *shape, seed=23)
        nt = 7
        ref = g0.copy().run(nt, nthreads=4)
        for depth in range(1, MAX_DEPTH[(precision, r)] + 1):
            # FP32 boxes start on 16 bytes (4 columns); TMA tiles keep the general width.
            # Variant 3 at radius 1 and depth <= 2 is a 64 x 64 region (x quads)
            wt = 64 if (variant == 3 and r == 1 and depth <= 2) else w
            block = (wt - 2 * depth * r - 3, h - 2 * depth * r)
            with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth,
                             block=block) as ctx:
                with gpu_context(g0.copy(), precision=precision, schedule="fused", fusion_depth=depth,
                                 block=_block(op, depth, variant - 2)) as plain_ctx:
                    ctx.run(nt)
                    plain_ctx.run(nt)
                    u1, u2 = ctx.download()
                    p1, p2 = plain_ctx.download()
            np.testing.assert_array_equal(u1, p1)  # same arithmetic, different data movement
            np.testing.assert_array_equal(u2, p2)
            assert max_rel(u1, ref.U1, ref) < 5e-6
