"""Shared helpers for the GPU parity tests: build oracle grids and GPU contexts
from the same seeded or reference inputs."""
import numpy as np

import oracle
from girih_gb300 import gpu

# standard 8th-order second-difference weights over 3 axes (sum 0), rounded to
# FP32-representable values so FP32 and FP64 runs share one operator
LAP8 = [float(np.float32(x)) for x in (3 * (-205.0 / 72.0), 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0)]
LAP2 = [-0.75, 0.125]  # 7-point Laplacian weights (c0 = -6 c1), FP32-representable

SEED_PARAMS = {  # op -> (f range, roc2 range, coef range, constant coefs)
    0: ((-1.0, 1.0), (0.05, 0.15), (0.0, 0.0), LAP8),
    1: ((0.0, 1.0), (0.0, 0.0), (0.0, 0.0), None),  # reference default coefficients
    2: ((0.0, 1.0), (0.0, 0.0), (0.01, 0.1), None),
    3: ((0.0, 1.0), (0.0, 0.0), (0.01, 0.1), None),
    4: ((0.0, 1.0), (0.0, 0.0), (0.01, 0.025), None),
    5: ((0.0, 1.0), (0.0, 0.0), (0.01, 0.1), None),
    7: ((0.0, 1.0), (0.0, 0.0), (0.0, 0.0), [-0.5, 0.05, 0.02, 0.01]),  # box: 4 constant coefficients
    8: ((0.0, 1.0), (0.5, 1.5), (0.0, 0.0), LAP2),
}


def oracle_grid(op, nx, ny, nz, seed=None):
    """Oracle grid with seeded inputs (seed given) or the reference's own init."""
    g = oracle.Grid(op, nx, ny, nz)
    if seed is None:
        g.fill_ref()
        return g
    f, r2, c, coefs = SEED_PARAMS[op]
    g.fill_seeded(seed, f, r2, c, coefs=coefs)
    if not g.coef_arrays and coefs is None:
        g.coef[:] = g.default_coefs()
    return g


def gpu_context(g, **kw):
    ctx = gpu.Context(g.op, g.nx, g.ny, g.nz, pnx=g.pnx, **kw)
    ctx.upload(g.U1, g.U2, g.U3, g.coef)
    return ctx


def bf16_round(x):
    """Round float64 values to the nearest BF16 number (8 significant bits, ties
    to even), as __double2bfloat16 does for values in the normal range."""
    m, e = np.frexp(np.asarray(x, dtype=np.float64))
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def bf16_quantized_coefs(g):
    """The coefficient arrays the mixed form computes with: per array a scale
    s = FP32(max |c|), the BF16 value of c / s, and the effective coefficient
    FP32(FP32(bf16) * s) (the kernels' load: bf16 -> float times the scale)."""
    out = g.coef.copy()
    for m in range(out.shape[0]):
        c = g.coef[m]
        s = np.float32(np.max(np.abs(c)))
        q = bf16_round(c / np.float64(s)).astype(np.float32)
        out[m] = (q * s).astype(np.float64)
    return out


def max_rel(a, b, g):
    n = oracle.norms(a, b, g)
    return n[0] / n[1] if n[1] > 0 else n[0]


def fused_block(r, w, h, depth, align):
    """Output tile (BX, BY) of a register/global-load fused region w x h with
    halo depth*r whose start is aligned to `align` columns (the kernel's
    FusedShape: a multiple of align when that is at least as wide as the
    general w - 2H - (align-1); TMA tiles always take the general width)."""
    H = depth * r
    mis = (-H) % align
    bx = max((w - 2 * H - mis) // align * align, w - 2 * H - (align - 1))
    return (bx, h - 2 * H)
