"""The no-allocation entry point girih_gpu_fused_run_noalloc().

It serves callers that cannot call cudaMalloc (a host application that owns the
device memory through its own pool, or a path that must not take the device
synchronisation an allocation can cause): they pass their own device arrays and
the library keeps its two spare state arrays in a static device array.  This
test calls it through the C ABI on device arrays the test owns, twice in a row,
and checks each result against the context-based entry point girih_gpu_run()
on the same grid, within the FP64 parity tolerance used throughout (1e-12
max-norm relative; the arithmetic is the same, so the results should agree
exactly).  The cases cover an even and an odd number of fused passes (an odd
count leaves the final states in the spare arrays, which the call copies back),
FP64, FP32 and the mixed form, and nt = 0.  The file sorts last so that a run
stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

import oracle
from girih_gb300 import gpu
from gpu_helpers import oracle_grid

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
PAD_U1, PAD_U2 = 7.0, -3.0  # distinct x-padding values of the caller's two arrays


def _to_device(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


# op, precision, nt, fusion depth (0 = the library's default); passes = ceil(2*ceil(nt/2) / depth)
CASES = [
    (8, "fp64", 7, 2),   # 8 steps, 4 passes
    (8, "fp64", 1, 2),   # 2 steps, 1 pass (odd)
    (8, "fp64", 5, 2),   # 6 steps, 3 passes (odd)
    (1, "fp64", 7, 0),
    (1, "fp64", 5, 2),   # time order 1, odd: only the last pass writes the previous state
    (0, "fp64", 7, 0),
    (0, "fp64", 3, 2),   # radius 4, 4 steps, 2 passes
    (8, "mixed", 7, 0),
    (8, "mixed", 3, 4),  # 4 steps, 1 pass (odd)
    (1, "fp32", 5, 2),   # FP32, 3 passes (odd)
    (8, "fp64", 0, 2),   # nothing to do: the arrays come back unchanged
]


@pytest.mark.parametrize("op,precision,nt,depth", CASES)
def test_noalloc_matches_context_entry_point_twice(op, precision, nt, depth):
    import torch
    shape = (45, 38, 29) if gpu.OP_INFO[op][0] == 1 else (41, 30, 26)
    g = oracle_grid(op, *shape, seed=13)
    r = g.r
    nnx = g.nx + 2 * r
    assert g.pnx > nnx, "the grid must have x padding for the padding check"
    dtype = np.float64 if precision == "fp64" else np.float32
    coefs = list(g.coef[:5])
    h1, h2 = g.U1.copy(), g.U2.copy()
    h1[:, :, nnx:] = PAD_U1
    h2[:, :, nnx:] = PAD_U2
    d1, d2 = _to_device(h1, dtype), _to_device(h2, dtype)
    d3 = _to_device(g.U3, dtype) if g.U3 is not None else None
    with gpu.Context(op, g.nx, g.ny, g.nz, pnx=g.pnx, precision=precision, schedule="fused",
                     fusion_depth=depth) as ctx:
        ctx.upload(g.U1, g.U2, g.U3, g.coef)
        for call in range(2):
            ctx.run(nt)
            want1, want2 = ctx.download()
            gpu.fused_run_noalloc(op, g.nx, g.ny, g.nz, d1.data_ptr(), d2.data_ptr(),
                                  d3.data_ptr() if d3 is not None else None, coefs, nt,
                                  precision=precision, pnx=g.pnx, fusion_depth=depth)
            torch.cuda.synchronize()
            got1, got2 = d1.double().cpu().numpy(), d2.double().cpu().numpy()
            for got, want in ((got1, want1), (got2, want2)):
                n = oracle.norms(got, want, g)
                assert n[0] <= FP64_TOL * n[1], (call, n)
            if nt == 0:
                np.testing.assert_array_equal(got1[:, :, :nnx], np.asarray(g.U1, dtype)[:, :, :nnx])
                np.testing.assert_array_equal(got2[:, :, :nnx], np.asarray(g.U2, dtype)[:, :, :nnx])
            # halos are left as they were, and so is each array's own x padding
            np.testing.assert_array_equal(got1[:r, :, :nnx], want1[:r, :, :nnx])
            np.testing.assert_array_equal(got2[:, :r, :nnx], want2[:, :r, :nnx])
            assert np.all(got1[:, :, nnx:] == PAD_U1) and np.all(got2[:, :, nnx:] == PAD_U2)


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    n = 300  # two FP64 state arrays of 302^2 * 304 doubles exceed 64 MiB
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.fused_run_noalloc(1, n, n, n, t.data_ptr(), t.data_ptr(), None, [-0.5, 0.1], 2)
    assert e.value.code == 1
    assert "scratch" in str(e.value)
