"""The bounds-checked build of the library (libgirih_gpu_check.so).

Built with GIRIH_CHECK (girih_gb300/build.py --checked, csrc/check.cuh), every
kernel tests each global access range against the extent of its array and each
shared-memory block against the CTA's allocation, skipping an access outside
and recording it; and every store of a new state value is counted per point, so
that after a run each interior point of a buffer must have been written exactly
as often as the schedule writes that buffer, and no halo or padding point at
all.  girih_gpu_run() returns GIRIH_GPU_EBOUNDS or GIRIH_GPU_ECOVERAGE
otherwise.  The GPU parity suites of the plain, fused (star, box,
variable-coefficient, TMA, double-float), batched and source-point kernels are
run here against the checked library in a child process: any such report
fails them.  Nothing is planted: the suites' own ragged shapes, 1x1x1 grids and
tile-edge cases drive the kernels.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITES = ["test_plain_gpu.py", "test_fused_gpu.py", "test_fused_box_gpu.py", "test_fused_var_gpu.py",
          "test_batched_gpu.py", "test_source_gpu.py"]

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_env():
    sys.path.insert(0, ROOT)
    from girih_gb300 import build as gbuild
    gbuild.build(checked=True)  # a few minutes when not up to date
    return dict(os.environ, GIRIH_GPU_CHECKED="1")


def test_binding_loads_the_checked_library(checked_env):
    code = ("from girih_gb300 import gpu; L = gpu.lib(); print(gpu.LIB_PATH); "
            "print(L.girih_gpu_strerror(9).decode()); print(L.girih_gpu_strerror(10).decode())")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=checked_env, cwd=ROOT,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    path, e9, e10 = r.stdout.strip().splitlines()[-3:]
    assert path.endswith("libgirih_gpu_check.so")
    assert "bounds-checked" in e9 and "bounds-checked" in e10


def test_parity_suites_pass_under_the_checked_build(checked_env):
    files = [os.path.join(ROOT, "tests", f) for f in SUITES]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider"] + files,
                       capture_output=True, text=True, env=checked_env, cwd=ROOT, timeout=3000)
    tail = r.stdout[-3000:] + r.stderr[-2000:]
    assert r.returncode == 0, tail
    assert " passed" in r.stdout and "EBOUNDS" not in r.stdout and "ECOVERAGE" not in r.stdout, tail
