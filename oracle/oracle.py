"""ctypes wrapper around the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle restates the girih reference's serial operators
(src/verification.c:315-479, 786-819), its initialisation (src/utils.c:436-497,
605-697) and its ping-pong loop (src/verification.c:281-284) in C
(oracle/girih_oracle.c).  Only tests, the smoke check and the benchmark's CPU
baseline leg use it, always as the checker or the timed CPU baseline, never as
the GPU product path.

Arrays are numpy float64 with shape (nz+2r, ny+2r, pnx): x fastest, the
reference's padded local domain (src/utils.c:367-374).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgirih_oracle.so")
_lib = None

OP_INFO = {  # op id -> (radius, time order, n coef, coef arrays?)   stencils.c:260-271
    0: (4, 2, 5, False),
    1: (1, 1, 2, False),
    2: (1, 1, 2, True),
    3: (1, 1, 4, True),
    4: (4, 1, 13, True),
    5: (1, 1, 7, True),
    7: (1, 1, 4, False),
    8: (1, 2, 2, False),
}


def build():
    """Compile the oracle shared library with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE, "libgirih_oracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        d = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int
        L.go_fill_ref.argtypes = [i, i, i, i, i, d, d, d, d]
        L.go_fill_seeded.argtypes = [i, i, i, i, i, ctypes.c_uint64] + [ctypes.c_double] * 6 + [d] * 4 + [i, i]
        L.go_step.argtypes = [i, i, i, i, i, d, d, d, d, i]
        L.go_run.argtypes = [i, i, i, i, i, i, d, d, d, d, i]
        L.go_norms.argtypes = [d, d, i, i, i, i, i, d]
        L.go_run_source.argtypes = [i, i, i, i, i, i, d, d, d, d, ctypes.POINTER(ctypes.c_int), d, i, i]
        L.go_seeded_value.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_double]
        L.go_seeded_value.restype = ctypes.c_double
        L.go_default_coefs.argtypes = [d]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def padded_nx(nx, r, alignment=8):
    """The reference's x padding (src/utils.c:367-372), alignment in elements."""
    w = nx + 2 * r
    rem = w % alignment
    return w if rem == 0 else w + alignment - rem


class Grid:
    """Host arrays of one operator on one grid, in the reference layout."""

    def __init__(self, op, nx, ny, nz, pnx=None):
        r, to, nc, arr = OP_INFO[op]
        self.op, self.r, self.time_order, self.n_coef, self.coef_arrays = op, r, to, nc, arr
        self.nx, self.ny, self.nz = nx, ny, nz
        self.pnx = padded_nx(nx, r) if pnx is None else pnx
        self.shape = (nz + 2 * r, ny + 2 * r, self.pnx)
        self.U1 = np.zeros(self.shape)
        self.U2 = np.zeros(self.shape)
        self.U3 = np.zeros(self.shape) if to == 2 else None
        self.coef = np.zeros((nc,) + self.shape) if arr else np.zeros(11)

    def default_coefs(self):
        c = np.zeros(11)
        lib().go_default_coefs(_p(c))
        return c

    def fill_ref(self):
        lib().go_fill_ref(self.op, self.nx, self.ny, self.nz, self.pnx,
                          _p(self.U1), _p(self.U2), _p(self.U3), _p(self.coef))
        return self

    def fill_seeded(self, seed, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.0, 0.0), coefs=None, f32_exact=False,
                    nthreads=1):
        lib().go_fill_seeded(self.op, self.nx, self.ny, self.nz, self.pnx, seed,
                             f[0], f[1], roc2[0], roc2[1], c[0], c[1],
                             _p(self.U1), _p(self.U2), _p(self.U3),
                             _p(self.coef) if self.coef_arrays else None, 1 if f32_exact else 0, nthreads)
        if coefs is not None and not self.coef_arrays:
            self.coef[:len(coefs)] = coefs
        return self

    def run(self, nt, nthreads=1):
        e = lib().go_run(self.op, self.nx, self.ny, self.nz, self.pnx, nt,
                         _p(self.U1), _p(self.U2), _p(self.U3), _p(self.coef), nthreads)
        if e:
            raise ValueError(f"oracle go_run error {e}")
        return self

    def run_source(self, nt, pt, source, nthreads=1):
        """run() with source[it] added at array point pt = (i, j, k) after sweep it
        (src/kernels/nb_naive_ts.c:190,196)."""
        src = np.ascontiguousarray(source, dtype=np.float64)
        p3 = (ctypes.c_int * 3)(*pt)
        e = lib().go_run_source(self.op, self.nx, self.ny, self.nz, self.pnx, nt, _p(self.U1), _p(self.U2),
                                _p(self.U3), _p(self.coef), p3, _p(src), len(src), nthreads)
        if e:
            raise ValueError(f"oracle go_run_source error {e}")
        return self

    def step(self, u, v, nthreads=1):
        return lib().go_step(self.op, self.nx, self.ny, self.nz, self.pnx, _p(self.coef),
                             _p(u), _p(v), _p(self.U3), nthreads)

    def interior(self, a):
        r = self.r
        return a[r:r + self.nz, r:r + self.ny, r:r + self.nx]

    def copy(self):
        g = Grid(self.op, self.nx, self.ny, self.nz, self.pnx)
        g.U1[...] = self.U1
        g.U2[...] = self.U2
        if self.U3 is not None:
            g.U3[...] = self.U3
        g.coef[...] = self.coef
        return g


def norms(a, b, g):
    """{max|a-b|, max|b|, sum (a-b)^2, sum b^2} over the interior of grid g."""
    out = np.zeros(4)
    lib().go_norms(_p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)),
                   g.nx, g.ny, g.nz, g.pnx, g.r, _p(out))
    return out


def seeded_value(seed, stream, idx, lo, hi):
    return lib().go_seeded_value(seed, stream, idx, lo, hi)
