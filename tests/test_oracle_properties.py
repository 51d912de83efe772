"""Exact properties of the CPU oracle beyond the golden vectors (CPU only).

The golden vectors pin the restatement to the reference on the cases the
reference was run on; these properties hold for any input and any size:
  * scaling the fields by 2 scales every later state by 2 exactly (the
    operators are linear in the fields; scaling by a power of two commutes
    with rounding);
  * a constant field stays constant under a Laplacian whose weights sum to
    zero (leapfrog) or one (Jacobi smoother);
  * mirroring x (fields and coefficient arrays) commutes with the operators
    whose x pairs are summed as (+d) + (-d), because that sum is commutative;
  * halos and x padding are never written.
"""
import numpy as np
import pytest

import oracle

SHAPE = (21, 13, 11)
OPS = sorted(oracle.OP_INFO)


def _seeded(op, seed=5):
    g = oracle.Grid(op, *SHAPE)
    r = g.r
    if g.coef_arrays:
        return g.fill_seeded(seed, (0.0, 1.0), (0.0, 0.0), (0.01, 0.1 / r))
    if op == 0:
        return g.fill_seeded(seed, (-1.0, 1.0), (0.05, 0.15), coefs=[-8.541667, 1.6, -0.2, 0.025396826, -0.0017857143])
    if op == 8:
        return g.fill_seeded(seed, (0.0, 1.0), (0.5, 1.5), coefs=[-0.75, 0.125])
    if op == 7:
        return g.fill_seeded(seed, (0.0, 1.0), coefs=[0.5, 0.05, 0.02, 0.01])
    return g.fill_seeded(seed, (0.0, 1.0), coefs=[0.25, 0.125])


@pytest.mark.parametrize("op", OPS)
def test_fields_scale_exactly(op):
    nt = 6
    g = _seeded(op)
    h = g.copy()
    h.U1 *= 2.0
    h.U2 *= 2.0
    g.run(nt)
    h.run(nt)
    np.testing.assert_array_equal(h.U1, 2.0 * g.U1)
    np.testing.assert_array_equal(h.U2, 2.0 * g.U2)


@pytest.mark.parametrize("op,coefs", [(8, [-0.75, 0.125]), (1, [0.25, 0.125]),
                                      (0, [-7.5, 1.0, 0.25, 0.0, 0.0])])
def test_constant_field_is_a_fixed_point(op, coefs):
    g = oracle.Grid(op, *SHAPE)
    g.U1[...] = 3.0
    g.U2[...] = 3.0
    if g.U3 is not None:
        g.U3[...] = 0.75
    g.coef[:len(coefs)] = coefs
    g.run(8)
    np.testing.assert_array_equal(g.interior(g.U1), 3.0)
    np.testing.assert_array_equal(g.interior(g.U2), 3.0)


def _mirror_x(g, a):
    """Reverse the unpadded x extent (interior and halo) of every row."""
    nnx = g.nx + 2 * g.r
    a[..., :nnx] = a[..., :nnx][..., ::-1].copy()


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4, 8])
def test_x_mirror_commutes_with_symmetric_operators(op):
    nt = 4
    g = _seeded(op, seed=11)
    m = g.copy()
    for a in (m.U1, m.U2) + ((m.U3,) if m.U3 is not None else ()):
        _mirror_x(m, a)
    if m.coef_arrays:
        for k in range(m.n_coef):
            _mirror_x(m, m.coef[k])
    g.run(nt)
    m.run(nt)
    for a in (m.U1, m.U2):
        _mirror_x(m, a)
    np.testing.assert_array_equal(m.U1, g.U1)
    np.testing.assert_array_equal(m.U2, g.U2)


@pytest.mark.parametrize("op", OPS)
def test_halo_and_padding_are_never_written(op):
    g = _seeded(op, seed=3)
    pad = g.pnx - (g.nx + 2 * g.r)
    if pad:
        g.U1[..., -pad:] = 7.0
        g.U2[..., -pad:] = 7.0
    before1, before2 = g.U1.copy(), g.U2.copy()
    g.run(5)
    r = g.r
    inner = np.zeros(g.shape, dtype=bool)
    inner[r:r + g.nz, r:r + g.ny, r:r + g.nx] = True
    np.testing.assert_array_equal(g.U1[~inner], before1[~inner])
    np.testing.assert_array_equal(g.U2[~inner], before2[~inner])
