"""The no-allocation entry point girih_gpu_fused_run_noalloc().

It serves callers that cannot call cudaMalloc (a host application that owns the
device memory through its own pool, or a path that must not take the device
synchronisation an allocation can cause): they pass their own device arrays and
the library keeps its two spare state arrays in a static device array.  This
test calls it through the C ABI on device arrays the test owns, twice in a row,
and checks each result against the context-based entry point girih_gpu_run()
on the same grid, within the FP64 parity tolerance used throughout (1e-12
max-norm relative; the arithmetic is the same, so the results should agree
exactly).  The file sorts last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

import oracle
from girih_gb300 import gpu
from gpu_helpers import oracle_grid

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _to_device(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


@pytest.mark.parametrize("op,precision", [(8, "fp64"), (1, "fp64"), (0, "fp64"), (8, "mixed")])
def test_noalloc_matches_context_entry_point_twice(op, precision):
    import torch
    shape = (45, 38, 29) if gpu.OP_INFO[op][0] == 1 else (40, 30, 26)
    g = oracle_grid(op, *shape, seed=13)
    dtype = np.float64 if precision == "fp64" else np.float32
    nt = 7
    coefs = list(g.coef[:5])
    d1, d2 = _to_device(g.U1, dtype), _to_device(g.U2, dtype)
    d3 = _to_device(g.U3, dtype) if g.U3 is not None else None
    with gpu.Context(op, g.nx, g.ny, g.nz, pnx=g.pnx, precision=precision, schedule="fused") as ctx:
        ctx.upload(g.U1, g.U2, g.U3, g.coef)
        for call in range(2):
            ctx.run(nt)
            want1, want2 = ctx.download()
            gpu.fused_run_noalloc(op, g.nx, g.ny, g.nz, d1.data_ptr(), d2.data_ptr(),
                                  d3.data_ptr() if d3 is not None else None, coefs, nt,
                                  precision=precision, pnx=g.pnx)
            torch.cuda.synchronize()
            got1, got2 = d1.double().cpu().numpy(), d2.double().cpu().numpy()
            for got, want in ((got1, want1), (got2, want2)):
                n = oracle.norms(got, want, g)
                assert n[0] <= FP64_TOL * n[1], (call, n)
            # halo and padding of the caller's arrays are left as they were
            r = g.r
            np.testing.assert_array_equal(got1[:r], want1[:r])
            np.testing.assert_array_equal(got1[:, :, g.nx + 2 * r:], want1[:, :, g.nx + 2 * r:])


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    n = 300  # two FP64 state arrays of 302^2 * 304 doubles exceed 64 MiB
    t = torch.zeros(1, dtype=torch.float64, device="cuda")
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.fused_run_noalloc(1, n, n, n, t.data_ptr(), t.data_ptr(), None, [-0.5, 0.1], 2)
    assert e.value.code == 1
    assert "scratch" in str(e.value)
