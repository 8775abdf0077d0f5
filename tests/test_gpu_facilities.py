"""Facilities on the GPU against the oracle: mov_fov moves `size` 8-byte
units between regions that may overlap, in either direction
(nesl/cvl/serial/facilt.c:160-183: every unit is read before it is
overwritten), bit-exact, at sizes below and above 64 MB and at distances
from one unit to more than the size."""
import numpy as np
import pytest

from neslgpu_gb300.cvl import DeviceVector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("size,delta", [
    (5, 1), (5, -1), (1000, 3), (1000, -3), (4097, 4096), (4097, -4096), (4097, 5000),
    ((9 << 20) + 5, 1), ((9 << 20) + 5, -1), ((9 << 20) + 5, 12345), ((9 << 20) + 5, -12345),
    ((9 << 20) + 5, (8 << 20) + 1), ((9 << 20) + 5, -((8 << 20) + 1)), ((20 << 20) + 3, -(2 << 20)),
])
def test_mov_fov_overlapping(gpu, oracle, size, delta):
    c, o = gpu.cvl, oracle.cvl
    total = size + abs(delta) + 16
    r = np.random.default_rng(size * 31 + delta)
    host = r.integers(0, 2 ** 63, size=total, dtype=np.int64).view(np.float64)
    dev = DeviceVector(c, total, "d")
    dev.upload(host)
    s_off, d_off = (abs(delta), 0) if delta < 0 else (0, delta)  # delta < 0: move down
    s_off += 7
    d_off += 7
    c.mov_fov(c.add_fov(dev.ptr, d_off), c.add_fov(dev.ptr, s_off), size, None)
    gpu.done()
    got = dev.numpy(total)
    want = host.copy()
    base = want.ctypes.data
    o.mov_fov(base + 8 * d_off, base + 8 * s_off, size, None)
    assert np.array_equal(got.view(np.int64), want.view(np.int64))
