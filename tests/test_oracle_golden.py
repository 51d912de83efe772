"""The CPU oracle restatement against golden vectors from the reference itself.

Golden vectors (tests/golden/golden_ref.npz) were produced by the unmodified
reference time stepper (src/kernels/nb_naive_ts.c:165-216) through
oracle/ref_golden.c; see tests/golden/make_golden.py.  The restatement must be
bit-exact, as the reference's own verification is (src/verification.c:842-849).
"""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")
_data = np.load(GOLD)
SPECS = json.loads(bytes(_data["specs"]).decode())


def _grid_for(name):
    s = SPECS[name]
    g = oracle.Grid(s["op"], s["nx"], s["ny"], s["nz"])
    if s["init"] == "ref":
        g.fill_ref()
    else:
        sp = s["seeded"]
        g.fill_seeded(sp["seed"], tuple(sp["f"]), tuple(sp["roc2"]), tuple(sp["c"]),
                      coefs=sp.get("coefs"))
        if not g.coef_arrays and not sp.get("coefs"):
            g.coef[:] = g.default_coefs()
    return g, s


@pytest.mark.parametrize("name", sorted(SPECS))
@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_bit_exact_vs_reference(name, nthreads):
    g, s = _grid_for(name)
    assert g.U1.shape == _data[name + "__U1"].shape
    if "source_pt" in s:
        g.run_source(s["nt"], s["source_pt"], np.arange(s["nt"], dtype=np.float64), nthreads=nthreads)
    else:
        g.run(s["nt"], nthreads=nthreads)
    np.testing.assert_array_equal(g.U1, _data[name + "__U1"])
    np.testing.assert_array_equal(g.U2, _data[name + "__U2"])


def test_golden_cases_move():
    """Guard against a vacuous pin: every case with nt > 0 changes the interior."""
    for name, s in SPECS.items():
        if s["nt"] == 0:
            continue
        g, _ = _grid_for(name)
        assert not np.array_equal(g.interior(g.U1), g.interior(_data[name + "__U1"])), name


def test_planted_error_is_detected():
    """A single-ulp change in the oracle output must fail the bit-exact check."""
    g, s = _grid_for("k1_ref")
    g.run(s["nt"])
    u = g.U1.copy()
    u[5, 5, 5] = np.nextafter(u[5, 5, 5], np.inf)
    assert not np.array_equal(u, _data["k1_ref__U1"])


def _leapfrog7_numpy(u, v, roc2, c, r=1):
    """Operator 8 (radius-1 leapfrog) restated with numpy elementwise ops, in the
    evaluation order of operator 0 (src/verification.c:330-350)."""
    out = u.copy()
    C = (slice(1, -1),) * 3

    def sh(dz, dy, dx):
        nz, ny, nx = v.shape
        return v[1 + dz:nz - 1 + dz, 1 + dy:ny - 1 + dy, 1 + dx:nx - 1 + dx]

    lap = c[0] * sh(0, 0, 0)
    lap = lap + c[1] * (sh(0, 0, 1) + sh(0, 0, -1))
    lap = lap + c[1] * (sh(0, 1, 0) + sh(0, -1, 0))
    lap = lap + c[1] * (sh(1, 0, 0) + sh(-1, 0, 0))
    out[C] = 2.0 * v[C] - u[C] + roc2[C] * lap
    return out


def test_operator8_against_numpy_restatement():
    nx, ny, nz = 11, 9, 7
    g = oracle.Grid(8, nx, ny, nz, pnx=nx + 2)  # no padding: numpy slicing covers the interior
    g.fill_seeded(1, (0.0, 1.0), (0.1, 0.3), coefs=[-6.0 / 6, 1.0 / 6])
    u, v, roc2 = g.U1.copy(), g.U2.copy(), g.U3.copy()
    for _ in range(3):
        u = _leapfrog7_numpy(u, v, roc2, g.coef)
        v = _leapfrog7_numpy(v, u, roc2, g.coef)
    g.run(6)
    np.testing.assert_array_equal(g.U1, u)
    np.testing.assert_array_equal(g.U2, v)


def test_seeded_values_are_deterministic_and_in_range():
    a = [oracle.seeded_value(1, 0, i, 0.0, 1.0) for i in range(1000)]
    b = [oracle.seeded_value(1, 0, i, 0.0, 1.0) for i in range(1000)]
    assert a == b
    assert min(a) >= 0.0 and max(a) < 1.0
    assert abs(np.mean(a) - 0.5) < 0.05
    c = [oracle.seeded_value(2, 0, i, 0.0, 1.0) for i in range(1000)]
    assert a != c


def test_source_cases_differ_from_sourceless_runs():
    """The source-point golden cases are not the plain run: the update was on."""
    for name, s in SPECS.items():
        if "source_pt" not in s:
            continue
        g, _ = _grid_for(name)
        g.run(s["nt"])
        assert not np.array_equal(g.U2, _data[name + "__U2"]), name
        i, j, k = s["source_pt"]
        assert g.r <= i < g.nx + g.r and g.r <= j < g.ny + g.r and g.r <= k < g.nz + g.r


def test_oracle_source_rejects_halo_point():
    g, s = _grid_for("k1_src")
    with pytest.raises(ValueError):
        g.run_source(2, (0, 5, 5), [1.0, 2.0])


_HARNESS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "ref_golden")


@pytest.mark.skipif(not os.path.exists(_HARNESS), reason="reference harness not built (needs the reference sources)")
@pytest.mark.parametrize("name", ["k0_seed", "k1_ref_odd_nt", "k4_ref", "k5_src"])
def test_fixtures_are_what_the_reference_produces(name):
    """Re-running the reference's own stepper reproduces the committed fixture
    bit for bit (the fixtures are the reference's output, not the oracle's)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    cases = {c[0]: (c, False) for c in mg.CASES}
    cases.update({c[0]: (c, True) for c in mg.SOURCE_CASES})
    (_, op, nx, ny, nz, nt, init, sp), source = cases[name]
    u1, u2, _ = mg.run_case(op, nx, ny, nz, nt, init, sp, source)
    np.testing.assert_array_equal(u1, _data[name + "__U1"])
    np.testing.assert_array_equal(u2, _data[name + "__U2"])
