"""Maximum sizes: a grid whose arrays exceed 2^31 elements.

The fused kernels index with 32-bit offsets and are limited to smaller grids,
so the auto schedule falls back to the plain kernel (64-bit offsets) and an
explicit fused request is refused.  The run is checked with an exact property:
an affine field is a fixed point of a Jacobi smoother whose weights sum to one
(c0 + 6 c1 = 1 with power-of-two weights; every intermediate is an FP32 integer
below 2^24).  The field varies along y and z, so a wrapped 32-bit offset in
the planes past 2^31 elements would read a wrong value.
"""
import numpy as np
import pytest

from girih_gb300 import gpu

pytestmark = pytest.mark.gpu

N = 1290  # (1290 + 2) rows and planes of a 1312-element device pitch: 2.2e9 elements per array


def test_affine_field_is_fixed_point_beyond_2_31_elements():
    op, r = 1, 1
    with pytest.raises(gpu.GirihGpuError) as e:
        gpu.Context(op, N, N, N, precision="fp32", schedule="fused", host_real_size=4)
    assert e.value.code == 2  # EUNSUPPORTED
    with gpu.Context(op, N, N, N, precision="fp32", schedule="auto", host_real_size=4) as ctx:
        assert ctx.info()["schedule"] == gpu.PLAIN
        nnz, nny, pnx = ctx.shape
        assert pnx * nny * nnz > 2 ** 31
        k = np.arange(nnz, dtype=np.float32)[:, None, None]
        j = np.arange(nny, dtype=np.float32)[None, :, None]
        field = np.ascontiguousarray(np.broadcast_to(4096.0 * j + k, (nnz, nny, pnx)), dtype=np.float32)
        coefs = np.zeros(11, dtype=np.float32)
        coefs[:2] = (0.25, 0.125)
        ctx.upload(field, field, None, coefs)
        ctx.run(2)
        mx, _, se, _ = ctx.error_norms(field)
        assert mx == 0.0 and se == 0.0
