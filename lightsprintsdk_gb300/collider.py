"""Python mirror of rr::RRCollider over the C ABI (include/rrgpu.h).

Names follow the reference interface (include/Lightsprint/RRCollider.h):
``RRCollider.create`` (RRCollider.h:183), ``intersect`` (:228),
``getMemoryOccupied`` (:259), ``getTechnique`` (:250), ``update`` (:190), and
the ``RRRay`` record (:85-137) as a numpy structured dtype with the
reference's 128-byte layout.  Batched calls are the fast path; ``intersect``
of a single RRRay exists for parity with the reference API.

There is no CPU fallback: if the CUDA library cannot be loaded or no GPU is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

# RRRay::Flags (RRCollider.h:98-106)
FILL_DISTANCE, FILL_POINT3D, FILL_POINT2D, FILL_PLANE, FILL_TRIANGLE, FILL_SIDE = 1, 2, 4, 8, 16, 32
FILL_ALL = 63
RAY_ORDER_DEFAULT, RAY_ORDER_AS_GIVEN, RAY_ORDER_BINNED = 0, 1, 2

# RRCollider::IntersectTechnique (RRCollider.h:156-166) plus the GPU technique
IT_LINEAR, IT_BSP_COMPACT, IT_BSP_FAST, IT_BSP_FASTER, IT_BSP_FASTEST, IT_BVH_COMPACT, IT_BVH_FAST, IT_VERIFICATION = range(8)
IT_GPU = 100

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "traversal stack overflow",
          5: "aborted", 6: "no usable CUDA device", 7: "mesh has no valid triangle", 8: "device wait timed out"}

# rr::RRRay, LP64 layout (include/Lightsprint/RRCollider.h:85-137)
RRRAY_DTYPE = np.dtype({
    "names": ["rayOrigin", "rayDir", "rayLengthMin", "rayLengthMax", "rayFlags", "hitDistance", "hitTriangle",
              "hitPoint2d", "hitPlane", "hitPoint3d", "hitFrontSide", "hitPadding1", "hitPadding2", "hitObject",
              "collisionHandler"],
    "formats": [("<f4", 4), ("<f4", 4), "<f4", "<f4", "<u4", "<f4", "<u4", ("<f4", 2), ("<f4", 4), ("<f4", 3),
                "u1", ("<f4", 3), ("<f4", 2), "<u8", "<u8"],
    "offsets": [0, 16, 32, 36, 40, 44, 48, 52, 60, 76, 88, 92, 104, 112, 120],
    "itemsize": 128,
})


class RRGError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = STATUS.get(status, f"status {status}")
        if status == 3:
            msg += ": " + _lib().rrg_last_cuda_error().decode()
        super().__init__(f"{what}: {msg}" if what else msg)


_L = None


class _BuildParams(C.Structure):
    _fields_ = [("size", C.c_uint32), ("max_leaf_size", C.c_uint32), ("sah_bins", C.c_uint32),
                ("traversal", C.c_uint32), ("bvh_width", C.c_uint32), ("reserved", C.c_uint32 * 3)]


def _lib():
    """Loads the in-tree CUDA library (building it first if it is missing or
    stale).  Raises when it cannot be built or loaded: there is no fallback."""
    global _L
    if _L is None:
        path = _build.build()
        L = C.CDLL(path)
        P, U, I = C.c_void_p, C.c_uint32, C.c_int
        L.rrg_collider_create.argtypes = [P, U, P, U, P, P, I, C.POINTER(P)]
        L.rrg_collider_create_device.argtypes = [P, U, P, U, P, P, P, C.POINTER(P)]
        L.rrg_collider_update.argtypes = [P, P]
        L.rrg_collider_destroy.argtypes = [P]
        L.rrg_collider_destroy.restype = None
        L.rrg_collider_memory.argtypes = [P]
        L.rrg_collider_memory.restype = C.c_size_t
        for f in ("rrg_collider_triangles", "rrg_collider_valid_triangles", "rrg_collider_nodes"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = U
        L.rrg_collider_build_ms.argtypes = [P]
        L.rrg_collider_build_ms.restype = C.c_float
        L.rrg_intersect_device.argtypes = [P, P, U, P, P, P, P]
        L.rrg_occluded_device.argtypes = [P, P, U, P, P]
        L.rrg_intersect_host.argtypes = [P, P, U, P, P]
        L.rrg_intersect_rrray.argtypes = [P, P, U, P, P]
        L.rrg_intersect_rrray_device.argtypes = [P, P, U, P, P]
        L.rrg_intersect_rrray_one.argtypes = [P, P, P]
        L.rrg_collider_combined.argtypes = [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.rrg_collider_status.argtypes = [P, P]
        L.rrg_collider_set_traversal.argtypes = [P, U]
        L.rrg_collider_set_compact_tuning.argtypes = [P, U, U, U]
        L.rrg_collider_trace_timing.argtypes = [P, C.c_int, P, P]
        L.rrg_intersect_rrray_one_after.argtypes = [P, P, C.c_float, U, P, P]
        L.rrg_collider_set_ray_order.argtypes = [P, U]
        L.rrg_status_string.argtypes = [I]
        L.rrg_status_string.restype = C.c_char_p
        L.rrg_last_cuda_error.restype = C.c_char_p
        L.rrg_version.restype = U
        L.rrg_launch_count.restype = C.c_uint64
        _L = L
    return _L


def library_path() -> str:
    return _build.LIB


def launch_count() -> int:
    """Kernels the library has launched in this process so far (all threads
    and devices; a kernel inside a CUDA graph counts once per graph launch)."""
    return int(_lib().rrg_launch_count())


def _check(st: int, what: str):
    if st != 0:
        raise RRGError(st, what)


def decode_hits(h: np.ndarray) -> dict:
    """(n,4) float32 hit records -> dict(hit, tri, dist, uv, side)."""
    h = np.asarray(h, np.float32).reshape(-1, 4)
    bits = h[:, 1].view(np.uint32)
    hit = bits != 0xFFFFFFFF
    tri = np.where(hit, bits & 0x7FFFFFFF, 0xFFFFFFFF).astype(np.uint32)
    side = hit & ((bits >> 31) == 1)
    return {"hit": hit, "tri": tri, "dist": np.where(hit, h[:, 0], 0).astype(np.float32),
            "uv": np.where(hit[:, None], h[:, 2:4], 0).astype(np.float32), "side": side}


class RRCollider:
    """GPU collider for one triangle mesh (post-import triangle i = row i of
    `indices`).  Mirrors rr::RRCollider created with the GPU technique."""

    def __init__(self, handle, vertices=None, indices=None):
        self._h = handle
        self._v = vertices
        self._t = indices

    # ------------------------------------------------------------ creation
    @classmethod
    def create(cls, vertices, indices, technique: int = IT_GPU, aborting=None, build_params: dict | None = None,
               device: int = 0) -> "RRCollider":
        """RRCollider::create(mesh, nullptr, technique, aborting, cacheLocation,
        buildParams) for an indexed triangle list.  `aborting` may be a
        ctypes.c_int that another thread sets to nonzero."""
        if technique != IT_GPU:
            raise ValueError("this library implements only the GPU technique")
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        bp = None
        if build_params:
            bp = _BuildParams(C.sizeof(_BuildParams), build_params.get("max_leaf_size", 0),
                              build_params.get("sah_bins", 0), build_params.get("traversal", 0),
                              build_params.get("bvh_width", 0))
        h = C.c_void_p()
        st = _lib().rrg_collider_create(v.ctypes.data, v.shape[0], t.ctypes.data, t.shape[0],
                                        C.byref(bp) if bp else None,
                                        C.byref(aborting) if aborting is not None else None, device, C.byref(h))
        _check(st, "rrg_collider_create")
        return cls(h, v, t)

    @classmethod
    def create_device(cls, xyz_dev_ptr: int, nv: int, idx_dev_ptr: int, nt: int, stream: int = 0,
                      build_params: dict | None = None) -> "RRCollider":
        bp = None
        if build_params:
            bp = _BuildParams(C.sizeof(_BuildParams), build_params.get("max_leaf_size", 0),
                              build_params.get("sah_bins", 0), build_params.get("traversal", 0),
                              build_params.get("bvh_width", 0))
        h = C.c_void_p()
        st = _lib().rrg_collider_create_device(xyz_dev_ptr, nv, idx_dev_ptr, nt, C.byref(bp) if bp else None, None,
                                               stream, C.byref(h))
        _check(st, "rrg_collider_create_device")
        return cls(h)

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None) and _L is not None:
            _L.rrg_collider_destroy(self._h)
            self._h = None

    def update(self, vertices) -> None:
        """RRCollider::update: re-read vertex positions, rebuild."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        _check(_lib().rrg_collider_update(self._h, v.ctypes.data), "rrg_collider_update")
        self._v = v

    # ------------------------------------------------------------ queries
    def set_traversal(self, traversal: int) -> None:
        """RRG_TRAVERSAL_IF_IF (1), RRG_TRAVERSAL_WHILE_WHILE (2),
        RRG_TRAVERSAL_COMPACT (3) or RRG_TRAVERSAL_ROOT_QUEUE (4, the default;
        0 selects it too)."""
        _check(_lib().rrg_collider_set_traversal(self._h, traversal), "rrg_collider_set_traversal")

    def set_compact_tuning(self, stack_smem: int = 8, rays_per_warp: int = 0, blocks_per_sm: int = 9) -> None:
        """Knobs of RRG_TRAVERSAL_COMPACT: shared-memory stack entries per
        thread (0, 8, 16, 32), rays a warp claims at a time (multiple of 32
        up to 1024; 0 = 32) and the register cap (9 blocks per SM, or 0 =
        none)."""
        _check(_lib().rrg_collider_set_compact_tuning(self._h, stack_smem, rays_per_warp, blocks_per_sm),
               "rrg_collider_set_compact_tuning")

    def trace_timing(self, enable: bool = True) -> tuple[float, int]:
        """(milliseconds, launches) of the closest-hit traversal kernel timed
        since the previous call; timing continues while enable."""
        ms = np.zeros(1, np.float32)
        k = np.zeros(1, np.uint32)
        _check(_lib().rrg_collider_trace_timing(self._h, 1 if enable else 0, ms.ctypes.data, k.ctypes.data),
               "rrg_collider_trace_timing")
        return float(ms[0]), int(k[0])

    def set_ray_order(self, order: int) -> None:
        """RAY_ORDER_DEFAULT (0: binned from 2^22 rays), RAY_ORDER_AS_GIVEN (1)
        or RAY_ORDER_BINNED (2); results do not depend on it."""
        _check(_lib().rrg_collider_set_ray_order(self._h, order), "rrg_collider_set_ray_order")

    def getTechnique(self) -> int:
        return IT_GPU

    def getMemoryOccupied(self) -> int:
        return int(_lib().rrg_collider_memory(self._h))

    @property
    def triangles(self) -> int:
        return int(_lib().rrg_collider_triangles(self._h))

    @property
    def valid_triangles(self) -> int:
        return int(_lib().rrg_collider_valid_triangles(self._h))

    @property
    def nodes(self) -> int:
        return int(_lib().rrg_collider_nodes(self._h))

    @property
    def build_ms(self) -> float:
        return float(_lib().rrg_collider_build_ms(self._h))

    @property
    def handle(self):
        return self._h

    def status(self, stream: int = 0) -> int:
        return int(_lib().rrg_collider_status(self._h, stream))

    def intersect_batch(self, rays: np.ndarray) -> dict:
        """Closest hit for host rays (n,8) -> decoded dict; host buffers in
        and out (rrg_intersect_host)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        out = np.empty((n, 4), np.float32)
        _check(_lib().rrg_intersect_host(self._h, rays.ctypes.data, n, out.ctypes.data, None), "rrg_intersect_host")
        _check(self.status(), "trace")
        return decode_hits(out)

    def intersect_device(self, rays_ptr: int, n: int, hits_ptr: int, planes_ptr: int = 0, points_ptr: int = 0,
                         stream: int = 0) -> None:
        _check(_lib().rrg_intersect_device(self._h, rays_ptr, n, hits_ptr, planes_ptr or None, points_ptr or None,
                                           stream or None), "rrg_intersect_device")

    def occluded_device(self, rays_ptr: int, n: int, occ_ptr: int, stream: int = 0) -> None:
        _check(_lib().rrg_occluded_device(self._h, rays_ptr, n, occ_ptr, stream or None), "rrg_occluded_device")

    def intersect_rrrays(self, rays: np.ndarray) -> np.ndarray:
        """rr::RRRay array (RRRAY_DTYPE) -> per-ray bool, outputs written in
        place as RRCollider::intersect would (rrg_intersect_rrray)."""
        assert rays.dtype == RRRAY_DTYPE and rays.flags.c_contiguous
        hit = np.zeros(rays.shape[0], np.uint8)
        _check(_lib().rrg_intersect_rrray(self._h, rays.ctypes.data, rays.shape[0], hit.ctypes.data, None),
               "rrg_intersect_rrray")
        _check(self.status(), "trace")
        return hit.astype(bool)

    def intersect(self, ray: np.ndarray, index: int = 0) -> bool:
        """RRCollider::intersect(RRRay&) for record `index` of an RRRAY_DTYPE
        array (modified in place).  Thread-safe: Python threads calling it at
        once (ctypes releases the GIL) are traced together as one device batch
        (rrg_intersect_rrray_one)."""
        assert ray.dtype == RRRAY_DTYPE and ray.flags.c_contiguous and 0 <= index < ray.shape[0]
        hit = C.c_uint8(0)
        _check(_lib().rrg_intersect_rrray_one(self._h, ray.ctypes.data + RRRAY_DTYPE.itemsize * index,
                                              C.byref(hit)), "rrg_intersect_rrray_one")
        return bool(hit.value)

    def combined(self) -> tuple[int, int]:
        """(batches, rays) traced so far by the combined single-ray path."""
        b, r = C.c_uint64(0), C.c_uint64(0)
        _check(_lib().rrg_collider_combined(self._h, C.byref(b), C.byref(r)), "rrg_collider_combined")
        return b.value, r.value


def make_rrrays(rays: np.ndarray, flags: int = FILL_ALL) -> np.ndarray:
    """(n,8) float rays -> RRRAY_DTYPE records as the RRRay constructor leaves
    them (RRCollider/RRRay.cpp:19-26: zeroed, origin w = 1)."""
    rays = np.asarray(rays, np.float32).reshape(-1, 8)
    a = np.zeros(rays.shape[0], RRRAY_DTYPE)
    a["rayOrigin"][:, :3] = rays[:, 0:3]
    a["rayOrigin"][:, 3] = 1.0
    a["rayDir"][:, :3] = rays[:, 4:7]
    a["rayLengthMin"] = rays[:, 3]
    a["rayLengthMax"] = rays[:, 7]
    a["rayFlags"] = flags
    return a


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False
