"""CPU-side checks of the C ABI: the library builds, loads, and exports every
entry point include/girih_gpu.h declares; without a GPU, create() reports
ENODEV instead of crashing.  No compute calls are made here."""
import ctypes
import os
import re
import subprocess

import pytest

from girih_gb300 import gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(girih_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    for must in ("girih_gpu_create", "girih_gpu_upload", "girih_gpu_run", "girih_gpu_download",
                 "girih_gpu_error_norms", "girih_gpu_destroy", "girih_gpu_strerror"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = gpu.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", gpu.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (girih_\w+)", out))
    assert set(declared_symbols()) <= exported


def test_abi_version_and_strerror():
    lib = gpu.lib()
    assert lib.girih_gpu_abi_version() == 1
    for code in range(0, 8):
        assert lib.girih_gpu_strerror(code)
    assert lib.girih_gpu_strerror(99) == b"unknown error"


def test_create_validates_before_touching_the_device():
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(6, 8, 8, 8)  # solar operator: not a star operator on the GPU
    assert e.value.code == 2
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(1, 8, 8, 8, pnx=5)  # pitch smaller than nx + 2r
    assert e.value.code == 1


def test_null_arguments_are_rejected():
    lib = gpu.lib()
    assert lib.girih_gpu_create(None, None) == 1
    assert lib.girih_gpu_run(None, 2, None) == 1
    assert lib.girih_gpu_upload(None, None, None, None, None) == 1
    lib.girih_gpu_destroy(None)  # no-op


@pytest.mark.skipif(__import__("torch").cuda.is_available(), reason="checks the no-GPU path")
def test_no_device_is_an_error_code():
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(1, 8, 8, 8)
    assert e.value.code == 7


def test_noalloc_validates_before_touching_the_device():
    """The no-allocation entry point rejects bad requests before any CUDA call
    (the pointers below are never dereferenced on the host)."""
    fake = 1 << 20  # 16-byte aligned stand-ins for device addresses
    coefs = [-0.75, 0.125]
    cases = [
        (dict(op=5), 2),                                   # variable coefficients: no fused no-alloc form
        (dict(op=8, U3=None), 1),                           # time order 2 needs roc2
        (dict(op=1, nx=300, ny=300, nz=300), 1),            # two FP64 states beyond the static scratch
        (dict(op=8, precision="mixed", fusion_depth=4, block=(53, 24)), 2),  # a TMA tile
        (dict(op=1, U1=fake + 8), 1),                       # misaligned array
    ]
    for kw, code in cases:
        args = dict(op=1, nx=20, ny=16, nz=12, U1=fake, U2=fake, U3=fake, coefs=coefs, nt=2)
        args.update(kw)
        n = args.pop("nx")
        with pytest.raises(gpu.GirihGpuError) as e:
            gpu.fused_run_noalloc(args.pop("op"), n, args.pop("ny"), args.pop("nz"), args.pop("U1"),
                                  args.pop("U2"), args.pop("U3"), args.pop("coefs"), args.pop("nt"), **args)
        assert e.value.code == code, (kw, str(e.value))


def test_ctypes_structs_match_the_header_layout(tmp_path):
    """The Python binding's girih_gpu_desc / girih_gpu_info_t mirror the C
    header field by field (offsets and sizes from the C compiler)."""
    src = tmp_path / "layout.c"
    fields = {"girih_gpu_desc": [f for f, _ in gpu.Desc._fields_], "girih_gpu_info_t": [f for f, _ in gpu.Info._fields_]}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "girih_gpu.h"', "int main(void) {"]
    for st, names in fields.items():
        lines.append(f'  printf("{st} size %zu\\n", sizeof({st}));')
        for n in names:
            lines.append(f'  printf("{st} {n} %zu\\n", offsetof({st}, {n}));')
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln}
    for st, cls in (("girih_gpu_desc", gpu.Desc), ("girih_gpu_info_t", gpu.Info)):
        assert got[(st, "size")] == ctypes.sizeof(cls), st
        for n in fields[st]:
            assert got[(st, n)] == getattr(cls, n).offset, (st, n)


def test_binding_and_oracle_agree_on_operators():
    import oracle
    assert gpu.OP_INFO == {k: (r, to, nc, bool(arr)) for k, (r, to, nc, arr) in oracle.OP_INFO.items()}
