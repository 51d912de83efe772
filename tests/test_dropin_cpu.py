"""The reference-side drop-in (girih_gb300/host): the girih driver built from
the reference's own objects with the GPU stepper as --target-ts 3.  Needs the
reference sources to build (the tree GIRIH_REF names, or the copy staged in
baseline/_ref/girih), so it runs where they exist; without a GPU the stepper
must fail with a clear error code, never crash."""
import os
import subprocess

import pytest

from __graft_entry__ import reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "girih_gb300", "host", "_build", "mwd_kernel_gpu")
REF = reference_tree()

pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def driver():
    jobs = f"-j{min(16, os.cpu_count() or 4)}"
    subprocess.run(["make", "-s", jobs, "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "girih_gb300", "host"), f"REF={REF}"], check=True)
    return EXE


def test_list_shows_gpu_stepper(driver):
    out = subprocess.run([driver, "--list"], capture_output=True, text=True).stdout
    assert "03   GPU (libgirih_gpu)" in out
    assert "00   Spatial Blocking" in out


def test_cpu_steppers_still_verify(driver):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([driver, "--nx", "16", "--ny", "16", "--nz", "16", "--nt", "4", "--target-kernel", "1",
                        "--target-ts", "0", "--thread-group-size", "2", "--verify", "1"],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0 and "PASSED" in r.stdout


def test_gpu_stepper_without_gpu_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-GPU path")
    if not os.path.exists(EXE):
        pytest.skip("driver not built")
    r = subprocess.run([EXE, "--nx", "16", "--ny", "16", "--nz", "16", "--nt", "4", "--target-kernel", "1",
                        "--target-ts", "3", "--verify", "1"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "no usable CUDA device" in r.stderr


@pytest.fixture(scope="module")
def oracle_stub(tmp_path_factory, driver):
    """libgirih_gpu.so stand-in backed by the CPU oracle (tests/c/oracle_gpu_stub.c),
    loaded ahead of the real library through LD_LIBRARY_PATH (the driver's
    search path is a RUNPATH)."""
    d = tmp_path_factory.mktemp("stub")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "c", "oracle_gpu_stub.c"), os.path.join(ROOT, "oracle", "girih_oracle.c"),
                    "-o", str(d / "libgirih_gpu.so"), "-lm"], check=True)
    return dict(os.environ, LD_LIBRARY_PATH=str(d), OMP_NUM_THREADS="2")


@pytest.mark.parametrize("kernel", ["1", "0", "5", "7"])
def test_gpu_stepper_host_logic_verifies(driver, oracle_stub, kernel):
    """gpu_ts.c end to end (shapes, upload, run, download) against the
    reference's own --verify 1 bit-exact check, the device replaced by the oracle."""
    r = subprocess.run([driver, "--nx", "20", "--ny", "14", "--nz", "12", "--nt", "6", "--target-kernel", kernel,
                        "--target-ts", "3", "--verify", "1"], capture_output=True, text=True, env=oracle_stub)
    assert r.returncode == 0, r.stderr
    assert "PASSED" in r.stdout


@pytest.mark.parametrize("precision,schedule", [("fp64df", "fused"), ("mixed", "auto"), ("fp32", "plain")])
def test_gpu_stepper_accepts_every_form(driver, oracle_stub, precision, schedule):
    """Every precision and schedule of the library is selectable from the
    reference CLI's environment (the oracle stand-in computes exactly, so the
    reference's bit-exact --verify 1 still passes)."""
    env = dict(oracle_stub, GIRIH_GPU_PRECISION=precision, GIRIH_GPU_SCHEDULE=schedule)
    r = subprocess.run([driver, "--nx", "18", "--ny", "12", "--nz", "10", "--nt", "4", "--target-kernel", "1",
                        "--target-ts", "3", "--verify", "1"], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert "PASSED" in r.stdout


def test_gpu_stepper_t_dim_sets_fusion_depth_and_autotune(driver, oracle_stub):
    """--t-dim (the MWD time unroll) becomes the fusion depth t_dim + 1;
    GIRIH_GPU_AUTOTUNE=1 tunes when the stepper first sees the grid."""
    env = dict(oracle_stub, GIRIH_GPU_SCHEDULE="fused", GIRIH_GPU_PRECISION="mixed", GIRIH_GPU_AUTOTUNE="1")
    r = subprocess.run([driver, "--nx", "18", "--ny", "12", "--nz", "10", "--nt", "4", "--target-kernel", "1",
                        "--target-ts", "3", "--t-dim", "3", "--verify", "1"], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert "PASSED" in r.stdout
    assert "GPU stepper autotune: fused schedule, depth 4" in r.stdout
    assert "mixed fused depth 4" in r.stdout


def test_gpu_stepper_rejects_unknown_precision(driver, oracle_stub):
    env = dict(oracle_stub, GIRIH_GPU_PRECISION="fp16")
    r = subprocess.run([driver, "--nx", "8", "--ny", "8", "--nz", "8", "--nt", "2", "--target-kernel", "1",
                        "--target-ts", "3"], capture_output=True, text=True, env=env)
    assert r.returncode == 1
    assert "GIRIH_GPU_PRECISION=fp16" in r.stderr


def _parse_py_summary(text):
    """The key matching of the reference's scripts/parse.py get_summary():
    a line starting with '<field>:' gives the first token after the colon."""
    import re
    floats = ("RANK0 MStencil/s  MIN", "RANK0 MStencil/s  AVG", "RANK0 MStencil/s  MAX", "RANK0 Total",
              "RANK0 Computation")
    strs = ("Time stepper name", "Stencil Kernel name", "Stencil Kernel coefficients", "Precision")
    ints = ("Number of time steps", "Number of tests", "OpenMP Threads", "MPI size")
    out = {}
    for line in text.splitlines():
        for f in floats:
            if re.match("^" + re.escape(f) + ":", line):
                out[f] = float(line.split(":")[1].split()[0])
        for f in ints:
            if re.match("^" + re.escape(f) + ":", line):
                out[f] = int(line.split(":")[1].split()[0])
        for f in strs:
            if re.match("^" + re.escape(f) + ":", line):
                out[f] = line.split(":")[1].strip()
    return out


def test_gpu_stepper_report_has_parse_py_keys(driver, oracle_stub):
    r = subprocess.run([driver, "--nx", "24", "--ny", "24", "--nz", "24", "--nt", "4", "--target-kernel", "1",
                        "--target-ts", "3", "--n-tests", "3"], capture_output=True, text=True, env=oracle_stub)
    assert r.returncode == 0, r.stderr
    m = _parse_py_summary(r.stdout)
    assert m["Time stepper name"] == "GPU (libgirih_gpu)"
    assert m["Number of time steps"] == 4 and m["Number of tests"] == 3
    assert 0 < m["RANK0 MStencil/s  MIN"] <= m["RANK0 MStencil/s  AVG"] * 1.0001 <= m["RANK0 MStencil/s  MAX"] * 1.0002
    assert "GPU device MStencil/s MAX:" in r.stdout
    import json
    js = [ln.split("GPU stepper JSON: ", 1)[1] for ln in r.stdout.splitlines() if ln.startswith("GPU stepper JSON: ")]
    assert len(js) == 1
    d = json.loads(js[0])
    assert d["target_kernel"] == 1 and d["grid"] == [24, 24, 24] and d["nt"] == 4 and d["calls"] == 3
    assert d["precision"] == "fp64" and d["schedule"] == "plain" and d["bytes_per_lup"] == 16.0
    assert d["glups_device_max"] > 0 and d["algorithmic_gbs_device"] == pytest.approx(16.0 * d["glups_device_max"], rel=1e-3)
