"""The C-ABI library builds, loads and exports every symbol include/*.h
declares; host-side argument checks.  No GPU compute is called here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from lightsprintsdk_gb300 import build as B
from lightsprintsdk_gb300 import collider as col

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = []
    for f in sorted(os.listdir(INCLUDE)):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, f)).read()
        names += re.findall(r"RRG_API\s+[\w\s\*]+?\b(rr\w+)\s*\(", txt)
    return sorted(set(names))


def test_library_builds_and_exports_all_declared_symbols():
    lib = B.build()
    assert os.path.exists(lib)
    syms = declared_symbols()
    assert len(syms) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (\w+)$", out, re.M))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    L = C.CDLL(lib)
    for s in syms:
        getattr(L, s)


def test_status_strings_and_version():
    L = col._lib()
    for code, text in col.STATUS.items():
        assert L.rrg_status_string(code).decode() == text
    assert L.rrg_version() >> 16 == 1


def test_rrray_dtype_matches_reference_layout():
    """Offsets of include/Lightsprint/RRCollider.h:85-137 on LP64."""
    d = col.RRRAY_DTYPE
    assert d.itemsize == 128
    off = {n: d.fields[n][1] for n in d.names}
    assert off == {"rayOrigin": 0, "rayDir": 16, "rayLengthMin": 32, "rayLengthMax": 36, "rayFlags": 40,
                   "hitDistance": 44, "hitTriangle": 48, "hitPoint2d": 52, "hitPlane": 60, "hitPoint3d": 76,
                   "hitFrontSide": 88, "hitPadding1": 92, "hitPadding2": 104, "hitObject": 112,
                   "collisionHandler": 120}


def test_invalid_arguments_rejected_before_any_device_work():
    L = col._lib()
    out = C.c_void_p()
    v = np.zeros((3, 3), np.float32)
    t = np.zeros((0, 3), np.uint32)
    assert L.rrg_collider_create(v.ctypes.data, 3, t.ctypes.data, 0, None, None, 0, C.byref(out)) == 7  # empty
    assert L.rrg_collider_create(None, 3, None, 1, None, None, 0, C.byref(out)) == 1
    assert L.rrg_collider_create(v.ctypes.data, 3, v.ctypes.data, 1, None, None, 0, None) == 1
    assert L.rrg_intersect_device(None, None, 1, None, None, None, None) == 1
    assert L.rrg_intersect_host(None, None, 1, None, None) == 1


def test_batch_arguments_rejected_before_any_device_work():
    from lightsprintsdk_gb300 import batch as rb
    L = rb._lib()
    out = C.c_void_p()
    v = np.zeros((6, 3), np.float32)
    t = np.zeros((2, 3), np.uint32)
    vo = np.array([0, 3, 6], np.uint32)
    bad = np.array([0, 2, 1], np.uint32)            # not ascending
    assert L.rrg_batch_create(v.ctypes.data, vo.ctypes.data, t.ctypes.data, bad.ctypes.data, 2, None, 0,
                              C.byref(out)) == 1
    assert L.rrg_batch_create(v.ctypes.data, vo.ctypes.data, t.ctypes.data, vo.ctypes.data, 0, None, 0,
                              C.byref(out)) == 1
    z = np.zeros(3, np.uint32)
    assert L.rrg_batch_create(v.ctypes.data, vo.ctypes.data, t.ctypes.data, z.ctypes.data, 2, None, 0,
                              C.byref(out)) == 7    # no triangles at all
    assert L.rrg_batch_intersect_device(None, None, None, 1, None, None) == 1
    assert L.rrg_batch_set_rays_per_warp(None, 32) == 1


def test_decode_hits():
    h = np.zeros((3, 4), np.float32)
    h[0] = [1.5, 0, 0.25, 0.5]
    h[0, 1:2].view(np.uint32)[0] = 7 | 0x80000000
    h[1, 1:2].view(np.uint32)[0] = 0xFFFFFFFF
    h[2] = [2.0, 0, 0.1, 0.2]
    h[2, 1:2].view(np.uint32)[0] = 3
    d = col.decode_hits(h)
    assert list(d["hit"]) == [True, False, True]
    assert list(d["tri"]) == [7, 0xFFFFFFFF, 3]
    assert list(d["side"]) == [True, False, False]


def test_no_cpu_fallback_without_gpu():
    """Without a usable device the collider raises instead of answering on
    the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.uint32)
    with pytest.raises(col.RRGError) as e:
        col.RRCollider.create(v, t)
    assert e.value.status in (3, 6)
