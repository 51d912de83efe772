"""Batched persistent kernel: many grids of uneven sizes and mixed operators in
one persistent launch per fused pass (CUDA graph).  Every grid is checked
against its own FP64 oracle run; the batched loop must give exactly what each
grid's single-grid kernels give (same arithmetic, different schedule)."""
import numpy as np
import pytest

import oracle
from girih_gb300 import gpu
from gpu_helpers import max_rel, oracle_grid

pytestmark = pytest.mark.gpu

GRIDS = [(8, 40, 33, 21), (0, 29, 22, 19), (1, 17, 64, 9), (8, 70, 12, 30), (0, 12, 10, 9), (1, 5, 5, 5),
         (8, 1, 1, 1)]


def _oracles(seed0=20):
    return [oracle_grid(op, nx, ny, nz, seed=seed0 + k) for k, (op, nx, ny, nz) in enumerate(GRIDS)]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 5e-6), ("mixed", 5e-6)])
def test_batched_matches_oracle_and_looped(precision, tol):
    nt = 7
    gs = _oracles()
    with gpu.Batch(GRIDS, precision=precision) as b, gpu.Batch(GRIDS, precision=precision) as bl:
        for k, g in enumerate(gs):
            b.grid(k).upload(g.U1, g.U2, g.U3, g.coef)
            bl.grid(k).upload(g.U1, g.U2, g.U3, g.coef)
        b.run(nt)
        info = b.info()
        assert info["items_last_run"] > 0 and info["launches_last_run"] >= 1
        bl.run_looped(nt)
        for k, g in enumerate(gs):
            u1, u2 = b.grid(k).download()
            l1, l2 = bl.grid(k).download()
            np.testing.assert_array_equal(u1, l1)
            np.testing.assert_array_equal(u2, l2)
            ref = g.copy().run(nt)
            assert max_rel(u1, ref.U1, ref) <= tol, (k, max_rel(u1, ref.U1, ref))
            assert max_rel(u2, ref.U2, ref) <= tol, k


def test_batched_autotune_keeps_state_and_continues():
    gs = _oracles(40)
    with gpu.Batch(GRIDS, precision="fp64") as b:
        for k, g in enumerate(gs):
            b.grid(k).upload(g.U1, g.U2, g.U3, g.coef)
        b.autotune(trial_steps=4)
        for k, g in enumerate(gs):
            u1, _ = b.grid(k).download()
            np.testing.assert_array_equal(u1, g.U1)
        b.run(4)
        b.run(6)  # the replayed graph continues from the rotated buffers
        for k, g in enumerate(gs):
            u1, u2 = b.grid(k).download()
            ref = g.copy().run(10)
            assert max_rel(u1, ref.U1, ref) <= 1e-12
            assert max_rel(u2, ref.U2, ref) <= 1e-12


def test_batch_rejects_mixed_precision_and_other_operators():
    lib = gpu.lib()
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Batch([(5, 8, 8, 8)])
    assert e.value.code == 2
