"""Host-side checks of bench.py: the workloads are the benchmark configurations
they are named for, the roofline's algorithmic bytes are the compulsory
traffic per lattice update, and the CPU baseline leg reports what it timed.
No GPU is used."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from girih_gb300 import gpu  # noqa: E402


def test_workloads_match_their_configurations():
    w = bench.WORKLOADS
    # 7-point leapfrog, 512^3, nt = 500, seed 1, U(0,1) fields
    assert (w["star7_leapfrog_512"]["op"], w["star7_leapfrog_512"]["n"], w["star7_leapfrog_512"]["nt"],
            w["star7_leapfrog_512"]["seed"], w["star7_leapfrog_512"]["f"]) == (8, 512, 500, 1, (0.0, 1.0))
    # 25-point leapfrog, 480^3, nt = 200, seed 2, U(-1,1), errors also at nt = 50 and 100
    s25 = w["star25_leapfrog_480"]
    assert (s25["op"], s25["n"], s25["nt"], s25["seed"], s25["f"]) == (0, 480, 200, 2, (-1.0, 1.0))
    assert s25["error_nts"] == [50, 100]
    # variable coefficients at 384^3, nt = 200, seed 3, coefficients U(0.01, 0.1 / radius)
    for name, op in (("var7_384", 5), ("var25_384", 4)):
        v = w[name]
        r = gpu.OP_INFO[op][0]
        assert (v["op"], v["n"], v["nt"], v["seed"], v["f"]) == (op, 384, 200, 3, (0.0, 1.0))
        assert v["c"] == pytest.approx((0.01, 0.1 / r))


@pytest.mark.parametrize("name", ["star7_leapfrog_512", "star25_leapfrog_480"])
def test_leapfrog_laplacians_vanish_on_constants(name):
    """c0 + 6 sum c_d = 0: a constant field is a fixed point, so the leapfrog
    stays bounded (the reference's default kernel-0 weights do not have this)."""
    c = bench.WORKLOADS[name]["coefs"]
    assert abs(c[0] + 6 * sum(c[1:])) < 1e-5 * abs(c[0])


def test_jacobi_workload_is_a_smoother():
    c0, c1 = bench.WORKLOADS["star7_jacobi_512"]["coefs"]
    assert c0 + 6 * c1 == 1.0 and abs(c0 - 6 * c1) < 1.0  # constants kept, checkerboard damped


def test_batched_grids_follow_the_configuration():
    grids = bench.batched_grids()
    assert grids == bench.batched_grids()  # seeded: the same 64 grids every run
    assert len(grids) == 64
    edges = {32, 48, 64, 96, 128, 160, 192}
    assert [g[0] for g in grids] == [8] * 32 + [0] * 32  # half 7-point, half 25-point leapfrog
    for k, (op, nx, ny, nz) in enumerate(grids):
        assert nx in edges
        if k % 2 == 0:
            assert nx == ny == nz  # cubes
        else:
            assert ny == nz == max(8, nx // 2)  # 2:1:1 boxes


@pytest.mark.parametrize("op,precision,schedule,want", [
    (1, "fp64", "plain", 16), (1, "fp32", "plain", 8),
    (8, "fp64", "plain", 32), (8, "mixed", "plain", 16), (0, "fp64", "plain", 32),
    (5, "fp64", "plain", 72), (5, "mixed", "plain", 22),
    (4, "fp64", "plain", 120), (4, "mixed", "plain", 34),
    # one fused launch: read cur, prev, roc2 and write two states (leapfrog), read one and write two
    # states (Jacobi's last pass writes U1 too; the bytes count the general pass)
    (8, "mixed", "fused", 20), (1, "mixed", "fused", 8), (8, "fp64df", "fused", 40),
])
def test_algorithmic_bytes(op, precision, schedule, want):
    tsz = 8 if precision in ("fp64", "fp64df") else 4
    assert bench.pass_bytes(gpu.OP_INFO[op], tsz, schedule, precision) == want


def test_cpu_baseline_reports_its_sample():
    wl = dict(bench.WORKLOADS["star7_leapfrog_512"], n=20)
    cb = bench.cpu_baseline(wl, 0.05)
    assert cb["kind"] == "port" and cb["unit"] == "GLUP/s" and cb["value"] > 0
    assert cb["cores"] == (os.cpu_count() or 1)
    assert cb["sample"].startswith("20^3 grid")


def test_measured_peak_is_read_from_the_driver_file():
    peak, kind = bench.measured_peak_hbm()
    assert peak > 0 and kind in ("measured", "fallback")
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert kind == "measured"


def test_committed_traffic_is_per_launch_bytes():
    t = bench.committed_traffic("fused_pass:star7_leapfrog_512:mixed")
    algorithmic = 20 * 514 ** 3  # one depth-4 pass over the 512^3 grid with its halo
    assert t is not None and 1.0 <= t / algorithmic < 1.2
    assert np.isfinite(t)
