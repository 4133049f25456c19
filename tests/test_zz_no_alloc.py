"""shdom_render_noalloc (rays staged in the library's fixed device array)
against shdom_render on the same handle, two calls in a row, and its
refusal of more rays than the array holds.  Named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from at3d_gb300.scenes import cloud_blob, orthographic_views

pytestmark = pytest.mark.gpu

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def solved():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from at3d_gb300.solver import RTE
    pb = cloud_blob(seed=12, nx=12, ny=12, nz=10, dx=0.04, dz=0.08)
    r = RTE.from_problem(pb)
    r.solve(100, verbose=False)
    return pb, r


def _noalloc(r, x, y, z, mu, phi):
    from at3d_gb300 import _lib
    x = np.ascontiguousarray(x, np.float32); y = np.ascontiguousarray(y, np.float32)
    z = np.ascontiguousarray(z, np.float32)
    mu = np.ascontiguousarray(mu, np.float64); phi = np.ascontiguousarray(phi, np.float64)
    out = np.full(len(x), -1.0, np.float32)
    L = _lib.lib()
    rc = L.shdom_render_noalloc(r._h, len(x), x.ctypes.data_as(_f), y.ctypes.data_as(_f), z.ctypes.data_as(_f),
                                mu.ctypes.data_as(_d), phi.ctypes.data_as(_d), out.ctypes.data_as(_f))
    return rc, out


def test_noalloc_matches_render_twice(solved):
    pb, r = solved
    rays = orthographic_views(pb, 16, 16)
    ref = r.render(*rays)
    rc1, out1 = _noalloc(r, *rays)
    rc2, out2 = _noalloc(r, *rays)
    assert rc1 == 0 and rc2 == 0
    assert np.array_equal(out1, ref)
    assert np.array_equal(out2, ref)
    # a smaller second set right after a larger one: no stale values
    sub = tuple(np.asarray(a)[:37] for a in rays)
    rc3, out3 = _noalloc(r, *sub)
    assert rc3 == 0 and np.array_equal(out3, ref[:37])


def test_noalloc_refuses_too_many_rays(solved):
    from at3d_gb300 import _lib
    pb, r = solved
    n = (1 << 16) + 1
    z = np.full(n, 1.0, np.float32)
    rc, _ = _noalloc(r, np.zeros(n), np.zeros(n), z, np.ones(n), np.zeros(n))
    assert rc == 1
    assert b"at most 65536 rays" in _lib.lib().shdom_last_error(r._h)
