"""Build libgirih_gpu.so in-tree for sm_103a (GB300) with nvcc.

Each .cu translation unit is compiled in parallel and linked into
girih_gb300/libgirih_gpu.so.  Objects go to girih_gb300/_build/.
`--checked` builds the bounds-checked library instead (GIRIH_CHECK: every
kernel access range tested against its buffer, write-coverage counters;
csrc/check.cuh) into girih_gb300/libgirih_gpu_check.so, objects in
girih_gb300/_build_check/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgirih_gpu.so")
BUILD_CHECKED = os.path.join(HERE, "_build_check")
LIB_CHECKED = os.path.join(HERE, "libgirih_gpu_check.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-diag-suppress", "177", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-I" + os.path.join(HERE, "..", "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, extra, build_dir=BUILD):
    obj = os.path.join(build_dir, os.path.basename(src).replace(".cu", ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(p) for p in [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(HERE, "..", "include", "girih_gpu.h"))
    return hs


def build(verbose=False, extra=(), checked=False):
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    extra = list(extra) + (["-DGIRIH_CHECK"] if checked else [])
    os.makedirs(build_dir, exist_ok=True)
    srcs = sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cu"))
    jobs = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--checked"]
    build(verbose=True, extra=args, checked="--checked" in sys.argv[1:])
