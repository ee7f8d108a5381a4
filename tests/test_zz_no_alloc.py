"""rrg_intersect_rrray_noalloc (static device scratch, no allocation) against
rrg_intersect_rrray on the same RRRay batches, several calls in a row, through
the C ABI.  Named to run last: it must pass both alone in a fresh process and
after every other test."""
import ctypes as C

import numpy as np
import pytest

from lightsprintsdk_gb300 import collider as col
from lightsprintsdk_gb300 import scenes

pytestmark = pytest.mark.gpu

MAX_RAYS = 16384           # RRG_NOALLOC_MAX_RAYS in include/rrgpu.h
RRG_OK, RRG_ERR_TOO_LARGE = 0, 9


def noalloc():
    f = col._lib().rrg_intersect_rrray_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def both(c, rays, flags):
    """The same records through rrg_intersect_rrray and the no-alloc entry
    point; returns (records, hits) of each."""
    # two zero-filled buffers: ndarray.copy() of this structured dtype does
    # not copy the unnamed padding bytes (89..91) of each record
    a = col.make_rrrays(rays, flags)
    b = col.make_rrrays(rays, flags)
    assert a.tobytes() == b.tobytes()
    ha = np.zeros(len(a), np.uint8)
    hb = np.full(len(b), 0xEE, np.uint8)
    assert col._lib().rrg_intersect_rrray(c.handle, a.ctypes.data, len(a), ha.ctypes.data, None) == RRG_OK
    assert col._lib().rrg_collider_status(c.handle, None) == RRG_OK
    assert noalloc()(c.handle, b.ctypes.data, len(b), hb.ctypes.data, None) == RRG_OK
    return a, ha, b, hb


def test_noalloc_allocates_no_device_memory():
    """A fresh collider's first query is a no-alloc call of the largest
    batch: the device's free memory is the same before and after (measured
    by cudaMemGetInfo).  A call of the largest batch on another collider
    comes first, so that the set-up it does on the device (loading the
    modules that hold the array and the kernel) is not counted; then the
    result comparison runs on the fresh collider as on any other."""
    import torch
    v0, t0 = scenes.icosphere_c0()
    warm = col.RRCollider.create(v0, t0)
    w = col.make_rrrays(scenes.shell_rays(MAX_RAYS))
    assert noalloc()(warm.handle, w.ctypes.data, len(w), None, None) == RRG_OK
    fresh = col.RRCollider.create(v0, t0)
    b = col.make_rrrays(scenes.shell_rays(MAX_RAYS))
    hb = np.zeros(len(b), np.uint8)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert noalloc()(fresh.handle, b.ctypes.data, len(b), hb.ctypes.data, None) == RRG_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    a, ha, b2, hb2 = both(fresh, scenes.shell_rays(MAX_RAYS), col.FILL_ALL)
    np.testing.assert_array_equal(hb2, ha)
    assert a.tobytes() == b2.tobytes()
    warm.close()
    fresh.close()


def test_noalloc_matches_rrg_intersect_rrray_on_calls_in_a_row():
    v0, t0 = scenes.icosphere_c0()
    sphere = col.RRCollider.create(v0, t0)
    room = scenes.interior_c1()
    interior = col.RRCollider.create(room.vertices, room.indices)
    calls = [
        (sphere, scenes.shell_rays(12000), col.FILL_ALL),
        (interior, scenes.surface_rays(room.vertices, room.indices, MAX_RAYS),
         col.FILL_DISTANCE | col.FILL_TRIANGLE | col.FILL_SIDE),
        (sphere, scenes.shell_rays(777)[::-1].copy(), col.FILL_ALL),
    ]
    for k, (c, rays, flags) in enumerate(calls):
        a, ha, b, hb = both(c, rays, flags)
        assert ha.any(), k
        np.testing.assert_array_equal(hb, ha, err_msg=f"call {k}: hit flags")
        assert a.tobytes() == b.tobytes(), f"call {k}: RRRay records differ"
    sphere.close()
    interior.close()


def test_noalloc_rejects_batches_above_the_maximum():
    v0, t0 = scenes.icosphere_c0()
    c = col.RRCollider.create(v0, t0)
    big = col.make_rrrays(scenes.shell_rays(MAX_RAYS + 1))
    before = big.tobytes()
    hit = np.zeros(len(big), np.uint8)
    assert noalloc()(c.handle, big.ctypes.data, len(big), hit.ctypes.data, None) == RRG_ERR_TOO_LARGE
    assert big.tobytes() == before and not hit.any()
    assert "RRG_NOALLOC_MAX_RAYS" in col._lib().rrg_status_string(RRG_ERR_TOO_LARGE).decode()
    assert noalloc()(c.handle, big.ctypes.data, 0, hit.ctypes.data, None) == RRG_OK
    # the largest allowed batch still runs after the refusal
    a, ha, b, hb = both(c, scenes.shell_rays(MAX_RAYS), col.FILL_ALL)
    np.testing.assert_array_equal(hb, ha)
    assert a.tobytes() == b.tobytes()
    c.close()
