"""The reference-side drop-in (girih_gb300/host): the girih driver built from
the reference's own objects with the GPU stepper as --target-ts 3.  Needs the
reference tree to build, so it runs where that tree exists; without a GPU the
stepper must fail with a clear error code, never crash."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "girih_gb300", "host", "_build", "mwd_kernel_gpu")
REF = "/root/reference"

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference tree not present")


@pytest.fixture(scope="module")
def driver():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
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
