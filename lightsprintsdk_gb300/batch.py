"""Uneven batches of meshes and ray sets (include/rrgpu_batch.h) through
ctypes: one multi-root BVH build for all meshes, one persistent closest-hit
launch for all rays, replayed from a CUDA graph.

The reference handles this case with one rr::RRCollider per mesh
(RRCollider/RRCollider.cpp:186-241) and intersect() per ray (RRCollider.h:228);
each ray's result here equals what RRCollider.intersect_device on a collider
of its own mesh returns (triangle indices local to the mesh)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import collider as col

MAX_MESHES = 8192          # RRG_BATCH_MAX_MESHES
RAYS_PER_WARP = (32, 64, 128, 256)

_bound = False


def _lib():
    global _bound
    L = col._lib()
    if not _bound:
        P, U, I = C.c_void_p, C.c_uint32, C.c_int
        L.rrg_batch_create.argtypes = [P, P, P, P, U, P, I, C.POINTER(P)]
        L.rrg_batch_destroy.argtypes = [P]
        L.rrg_batch_destroy.restype = None
        L.rrg_batch_set_rays_per_warp.argtypes = [P, U]
        L.rrg_batch_set_stack_smem.argtypes = [P, U]
        L.rrg_batch_set_root_queue.argtypes = [P, C.c_int]
        L.rrg_batch_set_vertices_device.argtypes = [P, P, P]
        L.rrg_batch_rebuild_intersect_device.argtypes = [P, P, P, U, P, P]
        L.rrg_batch_intersect_device.argtypes = [P, P, P, U, P, P]
        L.rrg_batch_status.argtypes = [P, P]
        for f in ("rrg_batch_meshes", "rrg_batch_nodes"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = U
        L.rrg_batch_memory.argtypes = [P]
        L.rrg_batch_memory.restype = C.c_size_t
        L.rrg_batch_build_ms.argtypes = [P]
        L.rrg_batch_build_ms.restype = C.c_float
        _bound = True
    return L


class RRColliderBatch:
    """All meshes of a batch on one GPU.  `vertices` (V,3) float32 and
    `indices` (T,3) uint32 are the meshes concatenated, indices local to each
    mesh; vert_off / tri_off are the (M+1,) prefix offsets."""

    def __init__(self, handle, nmesh: int):
        self._h = handle
        self.nmesh = nmesh

    @classmethod
    def create(cls, vertices, indices, vert_off, tri_off, build_params: dict | None = None,
               device: int = 0) -> "RRColliderBatch":
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        vo = np.ascontiguousarray(vert_off, np.uint32)
        to = np.ascontiguousarray(tri_off, np.uint32)
        if vo.shape != to.shape or vo.ndim != 1 or vo.shape[0] < 2:
            raise ValueError("vert_off and tri_off must be (M+1,) arrays")
        bp = None
        if build_params:
            bp = col._BuildParams(C.sizeof(col._BuildParams), build_params.get("max_leaf_size", 0),
                                  build_params.get("sah_bins", 0), 0, build_params.get("bvh_width", 0))
        h = C.c_void_p()
        st = _lib().rrg_batch_create(v.ctypes.data, vo.ctypes.data, t.ctypes.data, to.ctypes.data, vo.shape[0] - 1,
                                     C.byref(bp) if bp else None, device, C.byref(h))
        col._check(st, "rrg_batch_create")
        return cls(h, vo.shape[0] - 1)

    @classmethod
    def from_meshes(cls, mb, build_params: dict | None = None) -> "RRColliderBatch":
        """From a scenes.MeshBatch."""
        return cls.create(mb.vertices, mb.indices, mb.vert_off, mb.tri_off, build_params)

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None) and col._L is not None:
            col._L.rrg_batch_destroy(self._h)
        self._h = None

    @property
    def handle(self):
        return self._h

    def set_rays_per_warp(self, k: int) -> None:
        col._check(_lib().rrg_batch_set_rays_per_warp(self._h, int(k)), "rrg_batch_set_rays_per_warp")

    def set_stack_smem(self, entries: int) -> None:
        """Traversal-stack entries per thread in shared memory (0, 8, 16, 32)."""
        col._check(_lib().rrg_batch_set_stack_smem(self._h, int(entries)), "rrg_batch_set_stack_smem")

    def set_root_queue(self, on: bool) -> None:
        """Root-box queue in the closest-hit kernel (binary trees)."""
        col._check(_lib().rrg_batch_set_root_queue(self._h, 1 if on else 0), "rrg_batch_set_root_queue")

    def set_vertices_device(self, xyz_ptr: int, stream: int = 0) -> None:
        """New positions for all vertices (device float[3 * nv], create's layout)."""
        col._check(_lib().rrg_batch_set_vertices_device(self._h, xyz_ptr, stream or None),
                   "rrg_batch_set_vertices_device")

    def rebuild_intersect_device(self, rays_ptr: int, ray_off_ptr: int, n: int, hits_ptr: int,
                                 stream: int = 0) -> None:
        """Every mesh's tree rebuilt from the current positions, then the
        closest hits, in one CUDA graph replay."""
        col._check(_lib().rrg_batch_rebuild_intersect_device(self._h, rays_ptr, ray_off_ptr, n, hits_ptr,
                                                              stream or None), "rrg_batch_rebuild_intersect_device")

    def intersect_device(self, rays_ptr: int, ray_off_ptr: int, n: int, hits_ptr: int, stream: int = 0) -> None:
        """Closest hit for n device rays; ray_off_ptr = (M+1,) uint32 device
        offsets.  Asynchronous (a CUDA graph launch)."""
        col._check(_lib().rrg_batch_intersect_device(self._h, rays_ptr, ray_off_ptr, n, hits_ptr, stream or None),
                   "rrg_batch_intersect_device")

    def status(self, stream: int = 0) -> int:
        return _lib().rrg_batch_status(self._h, stream or None)

    @property
    def nodes(self) -> int:
        return int(_lib().rrg_batch_nodes(self._h))

    @property
    def memory(self) -> int:
        return int(_lib().rrg_batch_memory(self._h))

    @property
    def build_ms(self) -> float:
        return float(_lib().rrg_batch_build_ms(self._h))
