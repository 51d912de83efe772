"""girih_gb300: GB300 (sm_103a) implementation of the girih star-stencil hot path.

The product is the CUDA library libgirih_gpu.so behind the C ABI in
include/girih_gpu.h; `girih_gb300.gpu` binds it for Python callers and tests.
"""
from . import gpu  # noqa: F401

__all__ = ["gpu"]
