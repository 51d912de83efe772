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


def test_port_baseline_reports_its_sample():
    wl = dict(bench.WORKLOADS["star7_leapfrog_512"], n=20)
    cb = bench.cpu_baseline_port(wl, 0.05)
    assert cb["kind"] == "port" and cb["unit"] == "GLUP/s" and cb["value"] > 0
    assert cb["cores"] == bench.host_threads()
    assert cb["sample"].startswith("20^3 grid")


needs_reference = pytest.mark.skipif(not bench.reference_binary_ok(), reason="reference build not present")


@needs_reference
def test_reference_binary_times_each_test():
    """The reference's own MWD build, run as the CPU baseline: one time per
    performance test, and MWD's raised nt read from its report."""
    times, nt_eff, threads, cmd = bench.run_reference_binary(1, 32, 3, nt=10, threads=2)
    assert len(times) == 3 and all(t > 0 for t in times)
    assert nt_eff == 18  # 2 + a multiple of 2 (t_dim + 1) = 16 at t_dim 7
    assert threads == 2 and "--target-ts 2" in cmd and "--mwd-type 2" in cmd


@needs_reference
@pytest.mark.parametrize("kernel", sorted(bench.REFERENCE_STEPPER))
def test_reference_stepper_settings_pass_the_reference_verifier(kernel, tmp_path):
    """The MWD settings timed as the CPU baseline compute what the reference's
    serial operators compute (its own --verify 1, bit for bit on this x86-64
    host, src/verification.c:842-849): a baseline that skipped work would fail."""
    import subprocess
    threads = min(4, os.cpu_count() or 1)
    args = bench.fit_thread_groups(bench.REFERENCE_STEPPER[kernel]["args"], threads)
    r = subprocess.run([bench.REFERENCE_BINARY, "--nx", "64", "--ny", "64", "--nz", "48", "--nt", "4",
                        "--target-kernel", str(kernel), "--verify", "1"] + args, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)), timeout=600, cwd=str(tmp_path))
    assert r.returncode == 0 and "-PASSED" in r.stdout, r.stdout[-1500:] + r.stderr[-500:]


def test_thread_groups_fit_the_host():
    a = ["--target-ts", "2", "--thread-group-size", "8", "--thz", "8"]
    assert bench.fit_thread_groups(a, 16) == a
    assert bench.fit_thread_groups(a, 2)[3:] == ["2", "--thz", "2"]
    assert bench.fit_thread_groups(a, 12)[3:] == ["6", "--thz", "6"]


@needs_reference
def test_cpu_baseline_is_the_reference_build(monkeypatch):
    monkeypatch.setattr(bench, "host_threads", lambda: 2)
    wl = dict(bench.WORKLOADS["star7_leapfrog_512"], n=32)
    cb = bench.cpu_baseline(wl, 1.0, tests=2)
    assert cb["kind"] == "reference" and cb["cores"] == 2 and cb["value"] > 0
    assert "kernel 1" in cb["sample"] and "MWD" in cb["sample"] and "stands in" in cb["sample"]


def test_reference_arm_shares_the_workload_config(monkeypatch):
    """Both arms print the same config, so the two lines describe one workload;
    the reference arm's steps are the samples it timed."""
    monkeypatch.setattr(bench, "reference_binary_ok", lambda: False)
    wl = dict(bench.WORKLOADS["star7_leapfrog_512"], n=16)

    class A:
        steps, warmup, cpu_seconds = 2, 1, 0.1
    line = bench.run_reference(A, wl, 0, 1)
    assert line["config"] == bench.workload_config(wl, 1)
    assert line["impl"] == "reference" and line["steps"] == 2 and "sampled" in line
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert bench.run_reference(A, wl, 1, 2) is None  # only rank 0 runs the CPU baseline


def test_measured_peak_is_read_from_the_driver_file():
    peak, kind = bench.measured_peak_hbm()
    assert peak > 0 and kind in ("measured", "fallback")
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert kind == "measured"


def test_committed_traffic_is_per_launch_bytes():
    t = bench.committed_traffic("fused_pass_tma:star7_leapfrog_512:mixed")
    algorithmic = 20 * 514 ** 3  # one depth-4 pass over the 512^3 grid with its halo
    assert t is not None and 1.0 <= t / algorithmic < 1.2
    assert np.isfinite(t)
