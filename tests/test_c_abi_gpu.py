"""The C ABI called from C: tests/c/abi_check.c is compiled with gcc against
include/girih_gpu.h and libgirih_gpu.so (and the oracle restatement as the
checker) and must report every operator bit-identical to the serial reference
operators."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller_bit_identical(tmp_path):
    exe = tmp_path / "abi_check"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-std=gnu11",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "c", "abi_check.c"), os.path.join(ROOT, "oracle", "girih_oracle.c"),
                    "-L", os.path.join(ROOT, "girih_gb300"), "-lgirih_gpu",
                    "-Wl,-rpath," + os.path.join(ROOT, "girih_gb300"), "-lm", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("bit-identical") == 6
