"""Python binding of the libgirih_gpu C ABI (include/girih_gpu.h).

The binding mirrors the reference's stepper interface: a context is created for
one operator (`target_kernel`, src/kernels/stencils.c:260-271) on one grid
(`stencil_shape` interior, `ldomain_shape` host arrays, src/utils.c:367-374),
the caller's arrays are uploaded, `run(nt)` advances the grid like
`TSList[ts].func(p)` (src/kernels/nb_naive_ts.c:187-203: nt rounded up to even,
U1 <- op(U2), U2 <- op(U1)), and `download()` returns U1 and U2.

There is no CPU fallback: loading fails loudly if the CUDA library is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# GIRIH_GPU_CHECKED=1 selects the bounds-checked build (build.py --checked):
# every kernel access range tested against its buffer, write-coverage counters
CHECKED = os.environ.get("GIRIH_GPU_CHECKED", "0") not in ("", "0")
LIB_PATH = os.path.join(HERE, "libgirih_gpu_check.so" if CHECKED else "libgirih_gpu.so")

FP64, FP32, MIXED, FP64_DF = 0, 1, 2, 3
PLAIN, FUSED, AUTO = 0, 1, 2
PRECISIONS = {"fp64": FP64, "fp32": FP32, "mixed": MIXED, "fp64df": FP64_DF}
SCHEDULES = {"plain": PLAIN, "fused": FUSED, "auto": AUTO}

# radius, time order, number of coefficients, coefficient arrays?  (stencils.c:260-271; 8 is new)
OP_INFO = {0: (4, 2, 5, False), 1: (1, 1, 2, False), 2: (1, 1, 2, True), 3: (1, 1, 4, True),
           4: (4, 1, 13, True), 5: (1, 1, 7, True), 7: (1, 1, 4, False), 8: (1, 2, 2, False)}

ERRORS = {1: "EINVAL", 2: "EUNSUPPORTED", 3: "ECUDA", 4: "ENOMEM", 5: "ESTATE", 6: "ETIMEOUT", 7: "ENODEV",
          8: "ERANGE", 9: "EBOUNDS", 10: "ECOVERAGE"}


class Desc(ctypes.Structure):
    _fields_ = [("target_kernel", ctypes.c_int), ("stencil_shape", ctypes.c_int * 3),
                ("ldomain_shape", ctypes.c_int * 3), ("host_real_size", ctypes.c_int),
                ("precision", ctypes.c_int), ("schedule", ctypes.c_int), ("fusion_depth", ctypes.c_int),
                ("block_x", ctypes.c_int), ("block_y", ctypes.c_int), ("exact", ctypes.c_int),
                ("device", ctypes.c_int)]


class Info(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("schedule", ctypes.c_int), ("fusion_depth", ctypes.c_int),
                ("block_x", ctypes.c_int), ("block_y", ctypes.c_int), ("launches_last_run", ctypes.c_int),
                ("steps_last_run", ctypes.c_int), ("bytes_per_lup", ctypes.c_double),
                ("device_bytes", ctypes.c_double), ("kernel_name", ctypes.c_char * 64)]


class GirihGpuError(RuntimeError):
    def __init__(self, code, where, detail):
        self.code = code
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({detail})")


_lib = None


def lib():
    """Load libgirih_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            how = "python girih_gb300/build.py" + (" --checked" if CHECKED else "")
            raise ImportError(f"{LIB_PATH} is missing: build it with `{how}`")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.girih_gpu_create.argtypes = [ctypes.POINTER(P), ctypes.POINTER(Desc)]
        L.girih_gpu_destroy.argtypes = [P]
        L.girih_gpu_destroy.restype = None
        L.girih_gpu_upload.argtypes = [P, P, P, P, P]
        L.girih_gpu_run.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.girih_gpu_download.argtypes = [P, P, P]
        L.girih_gpu_error_norms.argtypes = [P, P, ctypes.POINTER(ctypes.c_double)]
        L.girih_gpu_compare.argtypes = [P, P, ctypes.POINTER(ctypes.c_double)]
        L.girih_gpu_fill_seeded.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.girih_gpu_download_roc2.argtypes = [P, P]
        L.girih_gpu_set_source.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.girih_gpu_fused_run_noalloc.argtypes = [ctypes.POINTER(Desc), P, P, P, ctypes.POINTER(ctypes.c_double),
                                                  ctypes.c_int, P]
        L.girih_gpu_info.argtypes = [P, ctypes.POINTER(Info)]
        L.girih_gpu_autotune.argtypes = [P, ctypes.c_int, ctypes.POINTER(Info)]
        L.girih_gpu_batch_create.argtypes = [ctypes.POINTER(P), ctypes.c_int, ctypes.POINTER(Desc)]
        L.girih_gpu_batch_destroy.argtypes = [P]
        L.girih_gpu_batch_destroy.restype = None
        L.girih_gpu_batch_grid.argtypes = [P, ctypes.c_int]
        L.girih_gpu_batch_grid.restype = P
        L.girih_gpu_batch_autotune.argtypes = [P, ctypes.c_int]
        L.girih_gpu_batch_run.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.girih_gpu_batch_run_looped.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.girih_gpu_batch_info.argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)]
        L.girih_gpu_strerror.argtypes = [ctypes.c_int]
        L.girih_gpu_strerror.restype = ctypes.c_char_p
        L.girih_gpu_last_error.restype = ctypes.c_char_p
        L.girih_gpu_abi_version.restype = ctypes.c_int
        _lib = L
    return _lib


def _check(code, where):
    if code != 0:
        raise GirihGpuError(code, where, lib().girih_gpu_last_error().decode())


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous
        return a.ctypes.data
    return int(a)  # raw host address (e.g. pinned torch tensor .data_ptr())


def padded_nx(nx, r, alignment=8):
    """The reference's x padding of the local domain (src/utils.c:367-372)."""
    w = nx + 2 * r
    rem = w % alignment
    return w if rem == 0 else w + alignment - rem


class Context:
    """One grid of one operator on one GPU (a girih_gpu_ctx)."""

    def __init__(self, op, nx, ny, nz, precision="fp64", schedule="plain", pnx=None, host_real_size=8,
                 fusion_depth=0, block=(0, 0), exact=False, device=0):
        r = OP_INFO[op][0] if op in OP_INFO else 1
        self.op, self.r = op, r
        self.nx, self.ny, self.nz = nx, ny, nz
        self.pnx = padded_nx(nx, r) if pnx is None else pnx
        d = Desc()
        d.target_kernel = op
        d.stencil_shape[:] = [nx, ny, nz]
        d.ldomain_shape[:] = [self.pnx, ny + 2 * r, nz + 2 * r]
        d.host_real_size = host_real_size
        d.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
        d.schedule = SCHEDULES[schedule] if isinstance(schedule, str) else schedule
        d.fusion_depth = fusion_depth
        d.block_x, d.block_y = block
        d.exact = 1 if exact else 0
        d.device = device
        self.desc = d
        self.host_dtype = np.float64 if host_real_size == 8 else np.float32
        self._h = ctypes.c_void_p()
        _check(lib().girih_gpu_create(ctypes.byref(self._h), ctypes.byref(d)), "girih_gpu_create")

    @property
    def shape(self):
        return (self.nz + 2 * self.r, self.ny + 2 * self.r, self.pnx)

    def close(self):
        if self._h:
            lib().girih_gpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, U1, U2, U3=None, coef=None):
        _check(lib().girih_gpu_upload(self._h, _ptr(U1), _ptr(U2), _ptr(U3), _ptr(coef)), "girih_gpu_upload")

    def fill_seeded(self, seed, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.0, 0.0), coefs=None, f32_exact=False):
        rng = (ctypes.c_double * 6)(f[0], f[1], roc2[0], roc2[1], c[0], c[1])
        cc = None
        if coefs is not None:
            cc = (ctypes.c_double * 5)(*(list(coefs)[:5] + [0.0] * (5 - len(coefs[:5]))))
        _check(lib().girih_gpu_fill_seeded(self._h, seed, rng, cc, 1 if f32_exact else 0), "girih_gpu_fill_seeded")

    def set_source(self, pt, values):
        """Source-point update of later runs: after sweep s, values[s] is added at
        array point pt = (i, j, k) (halo included).  values=None switches it off."""
        if values is None or len(values) == 0:
            _check(lib().girih_gpu_set_source(self._h, None, None, 0), "girih_gpu_set_source")
            return
        v = np.ascontiguousarray(values, dtype=np.float64)
        p3 = (ctypes.c_int * 3)(*pt)
        _check(lib().girih_gpu_set_source(self._h, p3, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(v)),
               "girih_gpu_set_source")

    def download_roc2(self, U3=None):
        if U3 is None:
            U3 = np.zeros(self.shape, self.host_dtype)
        _check(lib().girih_gpu_download_roc2(self._h, _ptr(U3)), "girih_gpu_download_roc2")
        return U3

    def run(self, nt):
        """Advance like the reference stepper; returns the device time in ms."""
        ms = ctypes.c_float()
        _check(lib().girih_gpu_run(self._h, nt, ctypes.byref(ms)), "girih_gpu_run")
        return ms.value

    def download(self, U1=None, U2=None):
        if U1 is None and U2 is None:
            U1 = np.zeros(self.shape, self.host_dtype)
            U2 = np.zeros(self.shape, self.host_dtype)
        _check(lib().girih_gpu_download(self._h, _ptr(U1), _ptr(U2)), "girih_gpu_download")
        return U1, U2

    def error_norms(self, ref_U1):
        out = (ctypes.c_double * 4)()
        _check(lib().girih_gpu_error_norms(self._h, _ptr(np.ascontiguousarray(ref_U1, self.host_dtype)), out),
               "girih_gpu_error_norms")
        return list(out)

    def compare(self, ref_ctx):
        out = (ctypes.c_double * 4)()
        _check(lib().girih_gpu_compare(self._h, ref_ctx._h, out), "girih_gpu_compare")
        return list(out)

    def autotune(self, trial_steps=0):
        """Time the candidate schedules/tiles/depths on this grid and keep the fastest."""
        inf = Info()
        _check(lib().girih_gpu_autotune(self._h, trial_steps, ctypes.byref(inf)), "girih_gpu_autotune")
        return {k: (getattr(inf, k).decode() if k == "kernel_name" else getattr(inf, k)) for k, _ in Info._fields_}

    def info(self):
        inf = Info()
        _check(lib().girih_gpu_info(self._h, ctypes.byref(inf)), "girih_gpu_info")
        return {k: (getattr(inf, k).decode() if k == "kernel_name" else getattr(inf, k)) for k, _ in Info._fields_}


class _GridView(Context):
    """A grid owned by a Batch: the single-grid calls on its context, no ownership."""

    def __init__(self, handle, op, nx, ny, nz, pnx, precision):
        r = OP_INFO[op][0]
        self.op, self.r = op, r
        self.nx, self.ny, self.nz, self.pnx = nx, ny, nz, pnx
        self.host_dtype = np.float64
        self._h = ctypes.c_void_p(handle)

    def close(self):
        self._h = ctypes.c_void_p()  # the batch destroys its grids


class Batch:
    """Many grids advanced together by the persistent batched kernel."""

    def __init__(self, grids, precision="mixed", device=0):
        """grids: list of (op, nx, ny, nz)."""
        n = len(grids)
        descs = (Desc * n)()
        self.views = []
        for k, (op, nx, ny, nz) in enumerate(grids):
            r = OP_INFO[op][0]
            d = descs[k]
            d.target_kernel = op
            d.stencil_shape[:] = [nx, ny, nz]
            d.ldomain_shape[:] = [padded_nx(nx, r), ny + 2 * r, nz + 2 * r]
            d.host_real_size = 8
            d.precision = PRECISIONS[precision]
            d.schedule = FUSED
            d.device = device
        self._h = ctypes.c_void_p()
        _check(lib().girih_gpu_batch_create(ctypes.byref(self._h), n, descs), "girih_gpu_batch_create")
        for k, (op, nx, ny, nz) in enumerate(grids):
            hnd = lib().girih_gpu_batch_grid(self._h, k)
            self.views.append(_GridView(hnd, op, nx, ny, nz, padded_nx(nx, OP_INFO[op][0]), precision))

    def grid(self, k):
        return self.views[k]

    def autotune(self, trial_steps=0):
        _check(lib().girih_gpu_batch_autotune(self._h, trial_steps), "girih_gpu_batch_autotune")

    def run(self, nt):
        ms = ctypes.c_float()
        _check(lib().girih_gpu_batch_run(self._h, nt, ctypes.byref(ms)), "girih_gpu_batch_run")
        return ms.value

    def run_looped(self, nt):
        ms = ctypes.c_float()
        _check(lib().girih_gpu_batch_run_looped(self._h, nt, ctypes.byref(ms)), "girih_gpu_batch_run_looped")
        return ms.value

    def info(self):
        la, it = ctypes.c_int(), ctypes.c_int()
        dep = (ctypes.c_int * len(self.views))()
        _check(lib().girih_gpu_batch_info(self._h, ctypes.byref(la), ctypes.byref(it), dep), "girih_gpu_batch_info")
        return {"launches_last_run": la.value, "items_last_run": it.value, "depths": list(dep)}

    def close(self):
        if self._h:
            lib().girih_gpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def fused_run_noalloc(op, nx, ny, nz, U1, U2, U3, coefs, nt, precision="fp64", pnx=None, fusion_depth=0,
                      device=0, stream=None, block=(0, 0)):
    """Fused time loop on caller-owned DEVICE arrays (reference layout, raw
    device addresses) without any device allocation by the library."""
    r = OP_INFO[op][0]
    d = Desc()
    d.target_kernel = op
    d.stencil_shape[:] = [nx, ny, nz]
    d.ldomain_shape[:] = [padded_nx(nx, r) if pnx is None else pnx, ny + 2 * r, nz + 2 * r]
    d.host_real_size = 8 if precision == "fp64" else 4
    d.precision = PRECISIONS[precision]
    d.schedule = FUSED
    d.fusion_depth = fusion_depth
    d.block_x, d.block_y = block
    d.device = device
    cc = (ctypes.c_double * 5)(*(list(coefs)[:5] + [0.0] * (5 - len(list(coefs)[:5]))))
    _check(lib().girih_gpu_fused_run_noalloc(ctypes.byref(d), U1, U2, U3, cc, nt, stream),
           "girih_gpu_fused_run_noalloc")


def rel_errors(norms):
    """(max-norm relative, L2 relative) from {max|a-b|, max|b|, sum(a-b)^2, sum b^2}."""
    me, mb, se, sb = norms
    return (me / mb if mb > 0 else float(me)), ((se / sb) ** 0.5 if sb > 0 else float(se) ** 0.5)
