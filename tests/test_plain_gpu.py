"""Parity of the plain (one step per launch) GPU kernels with the reference.

Bit-exact for the FP64 `exact` mode against the golden vectors produced by the
reference itself; max-norm relative error <= 1e-12 for the fast FP64 mode; FP32
and mixed forms against the FP64 oracle with the tolerances stated per test.
All calls go through the C ABI (girih_gb300.gpu binds libgirih_gpu.so).
"""
import json
import os

import numpy as np
import pytest

import oracle
from girih_gb300 import gpu
from gpu_helpers import bf16_quantized_coefs, gpu_context, max_rel, oracle_grid

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")
_data = np.load(GOLD)
SPECS = json.loads(bytes(_data["specs"]).decode())
GPU_CASES = sorted(n for n, s in SPECS.items() if s["op"] in gpu.OP_INFO)

FP64_TOL = 1e-12  # max-norm relative, FP64 plain against the serial reference


def _golden_grid(name):
    s = SPECS[name]
    g = oracle.Grid(s["op"], s["nx"], s["ny"], s["nz"])
    if s["init"] == "ref":
        g.fill_ref()
    else:
        sp = s["seeded"]
        g.fill_seeded(sp["seed"], tuple(sp["f"]), tuple(sp["roc2"]), tuple(sp["c"]), coefs=sp.get("coefs"))
        if not g.coef_arrays and not sp.get("coefs"):
            g.coef[:] = g.default_coefs()
    return g, s


def _set_golden_source(ctx, s):
    """Golden cases run with the reference's source update carry its point; the
    values are the reference's source[i] = i."""
    if "source_pt" in s:
        ctx.set_source(s["source_pt"], np.arange(s["nt"], dtype=np.float64))


@pytest.mark.parametrize("name", GPU_CASES)
def test_exact_fp64_is_bit_identical_to_reference(name):
    g, s = _golden_grid(name)
    with gpu_context(g, precision="fp64", schedule="plain", exact=True) as ctx:
        _set_golden_source(ctx, s)
        ctx.run(s["nt"])
        u1, u2 = ctx.download()
    np.testing.assert_array_equal(g.interior(u1), g.interior(_data[name + "__U1"]))
    np.testing.assert_array_equal(u1, _data[name + "__U1"])
    np.testing.assert_array_equal(u2, _data[name + "__U2"])


@pytest.mark.parametrize("name", GPU_CASES)
def test_fast_fp64_within_1e12(name):
    g, s = _golden_grid(name)
    with gpu_context(g, precision="fp64", schedule="plain") as ctx:
        _set_golden_source(ctx, s)
        ctx.run(s["nt"])
        u1, u2 = ctx.download()
        dev = gpu.rel_errors(ctx.error_norms(_data[name + "__U1"]))[0]
    assert max_rel(u1, _data[name + "__U1"], g) <= FP64_TOL
    assert max_rel(u2, _data[name + "__U2"], g) <= FP64_TOL
    assert dev <= FP64_TOL


@pytest.mark.parametrize("op", sorted(gpu.OP_INFO))
@pytest.mark.parametrize("shape", [(67, 45, 39), (33, 9, 70), (1, 1, 1), (130, 3, 2)])
def test_plain_fp64_seeded_against_oracle(op, shape):
    nt = 7  # odd: the reference runs 8 sweeps
    g = oracle_grid(op, *shape, seed=11)
    with gpu_context(g, precision="fp64", exact=True) as ctx:
        ctx.run(nt)
        u1, u2 = ctx.download()
    g.run(nt, nthreads=4)
    np.testing.assert_array_equal(u1, g.U1)
    np.testing.assert_array_equal(u2, g.U2)


@pytest.mark.parametrize("op", sorted(gpu.OP_INFO))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_seeded_init_matches_oracle(op, precision):
    g = oracle_grid(op, 21, 13, 11, seed=5)
    f, r2, c, coefs = __import__("gpu_helpers").SEED_PARAMS[op]
    with gpu.Context(op, 21, 13, 11, precision=precision) as ctx:
        if g.coef_arrays:
            coefs = None
        elif coefs is None:
            coefs = list(g.coef[:5])
        ctx.fill_seeded(5, f, r2, c, coefs=coefs)
        u1, u2 = ctx.download()
    want = g.U1 if precision == "fp64" else g.U1.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(u1, want)
    np.testing.assert_array_equal(u2, want)


@pytest.mark.parametrize("op", sorted(gpu.OP_INFO))
def test_plain_fp32_against_fp64_oracle(op):
    nt = 10
    g = oracle_grid(op, 40, 24, 20, seed=3)
    with gpu_context(g, precision="fp32") as ctx:
        ctx.run(nt)
        u1, _ = ctx.download()
    g.run(nt, nthreads=4)
    err = max_rel(u1, g.U1, g)
    assert err < 5e-6, err  # FP32 storage and arithmetic over 10 steps


@pytest.mark.parametrize("op", [2, 3, 4, 5])
def test_mixed_bf16_coefficients_error_is_bounded(op):
    """The mixed form stores the coefficient arrays as BF16 with a per-array
    FP32 scale.  Against the FP64 oracle run with those same quantised
    coefficients, only FP32 arithmetic separates the two (the FP32 bound of
    test_plain_fp32_against_fp64_oracle); against the oracle with the original
    coefficients the BF16 quantisation adds a bounded error: with positive
    coefficients and fields every coefficient is off by at most 2^-9 relative,
    so after n steps every point is off by at most n 2^-9 of its value."""
    nt = 10
    g = oracle_grid(op, 40, 24, 20, seed=3)
    gq = g.copy()
    gq.coef[...] = bf16_quantized_coefs(g)
    with gpu_context(g, precision="mixed") as ctx:
        ctx.run(nt)
        u1, _ = ctx.download()
        assert ctx.info()["bytes_per_lup"] == 8 + 2 * gpu.OP_INFO[op][2]
    g.run(nt, nthreads=4)
    gq.run(nt, nthreads=4)
    arith = max_rel(u1, gq.U1, gq)
    assert arith < 5e-6, arith  # FP32 storage and arithmetic over 10 steps
    quant = max_rel(gq.U1, g.U1, g)  # the BF16 representation alone
    assert 0 < quant < nt * 2 ** -9 * 1.001, quant
    err = max_rel(u1, g.U1, g)
    assert err < quant + arith * 1.01 + 1e-12, (err, quant, arith)


@pytest.mark.parametrize("precision,host_real_size", [("fp64", 8), ("fp32", 8), ("fp32", 4), ("fp64df", 8)])
def test_pinned_and_pageable_host_arrays_agree(precision, host_real_size):
    """Pinned host arrays are read and written by the layout kernels directly,
    pageable ones go through the staging buffer: the same values either way,
    halos included, and the caller's x padding is never written."""
    import torch
    op = 8
    g = oracle_grid(op, 37, 22, 19, seed=4)
    r = g.r
    nnx = g.nx + 2 * r
    assert g.pnx > nnx
    dt = np.float64 if host_real_size == 8 else np.float32
    sched = "fused" if precision == "fp64df" else "plain"

    def run(pinned):
        arrs = [np.ascontiguousarray(a, dtype=dt) for a in (g.U1, g.U2, g.U3)]
        if pinned:
            ts = [torch.from_numpy(a).pin_memory() for a in arrs]
            ptrs, views = [t.data_ptr() for t in ts], [t.numpy() for t in ts]
        else:
            ptrs, views = [a for a in arrs], arrs
        out = [np.full(g.shape, 7.0, dt), np.full(g.shape, -3.0, dt)]
        if pinned:
            outs = [torch.from_numpy(o).pin_memory() for o in out]
            optrs, oviews = [t.data_ptr() for t in outs], [t.numpy() for t in outs]
        else:
            optrs, oviews = out, out
        with gpu.Context(op, g.nx, g.ny, g.nz, pnx=g.pnx, precision=precision, schedule=sched,
                         host_real_size=host_real_size) as ctx:
            ctx.upload(ptrs[0], ptrs[1], ptrs[2], np.asarray(g.coef, dt))
            ctx.run(5)
            ctx.download(optrs[0], optrs[1])
        return [np.array(v) for v in oviews]

    a1, a2 = run(True)
    b1, b2 = run(False)
    np.testing.assert_array_equal(a1, b1)
    np.testing.assert_array_equal(a2, b2)
    assert np.all(a1[:, :, nnx:] == 7.0) and np.all(a2[:, :, nnx:] == -3.0)  # padding untouched
    g.run(5, nthreads=4)
    tol = 1e-12 if precision.startswith("fp64") else 5e-6
    assert max_rel(a1.astype(np.float64), g.U1, g) <= tol


def test_run_continues_from_state():
    g = oracle_grid(1, 30, 20, 10, seed=2)
    with gpu_context(g, exact=True) as ctx:
        ctx.run(4)
        ctx.run(6)
        u1, u2 = ctx.download()
    g.run(10)
    np.testing.assert_array_equal(u1, g.U1)
    np.testing.assert_array_equal(u2, g.U2)


def test_float_host_arrays():
    """Host arrays of a single-precision reference build (real_t = float)."""
    g = oracle_grid(1, 30, 20, 10, seed=2)
    ctx = gpu.Context(1, 30, 20, 10, precision="fp32", host_real_size=4)
    f32 = lambda a: a.astype(np.float32)
    ctx.upload(f32(g.U1), f32(g.U2), None, f32(g.coef))
    ctx.run(4)
    u1, _ = ctx.download()
    assert u1.dtype == np.float32
    g.run(4)
    assert max_rel(u1.astype(np.float64), g.U1, g) < 1e-5
    ctx.close()


def test_error_codes():
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(6, 8, 8, 8)  # solar operator: not a star/box operator on the GPU
    assert e.value.code == 2
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(1, 0, 8, 8)
    assert e.value.code == 1
    ctx = gpu.Context(1, 8, 8, 8)
    with pytest.raises(gpu.GirihGpuError) as e:
        ctx.run(2)  # before upload
    assert e.value.code == 5
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(1, 8, 8, 8, schedule="fused", exact=True)
    assert e.value.code == 2
    ctx.close()


def test_non_finite_result_is_visible_in_norms():
    g = oracle_grid(1, 16, 16, 16, seed=1)
    bad = g.U1.copy()
    with gpu_context(g) as ctx:
        ctx.run(0)
        bad[5, 5, 5] = np.nan
        n = ctx.error_norms(bad)
    assert np.isnan(n[1]) or np.isnan(n[0])
