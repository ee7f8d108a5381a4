"""Two-level scene collider (include/rrgpu_scene.h) through ctypes: objects
are instances of the meshes of an RRColliderBatch under 3 x 4 world
matrices; replaces rr::RRColliderMulti (RRCollider/RRColliderMulti.cpp:59-165)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import batch as rb
from . import collider as col

_bound = False


def _lib():
    global _bound
    L = rb._lib()
    if not _bound:
        P, U = C.c_void_p, C.c_uint32
        L.rrg_scene_create.argtypes = [P, U, P, P, C.POINTER(P)]
        L.rrg_scene_destroy.argtypes = [P]
        L.rrg_scene_destroy.restype = None
        L.rrg_scene_set_matrices.argtypes = [P, P]
        L.rrg_scene_set_enabled.argtypes = [P, P]
        L.rrg_scene_intersect_device.argtypes = [P, P, U, P, P, P]
        L.rrg_scene_status.argtypes = [P, P]
        _bound = True
    return L


class RRScene:
    """Objects (mesh index, world matrix) over a batch of meshes; the batch
    must outlive the scene (the scene keeps a reference to it)."""

    def __init__(self, meshes: rb.RRColliderBatch, obj_mesh, world):
        self.meshes = meshes
        om = np.ascontiguousarray(obj_mesh, np.uint32)
        w = np.ascontiguousarray(world, np.float32).reshape(-1, 12)
        if w.shape[0] != om.shape[0]:
            raise ValueError("one 3x4 matrix per object")
        h = C.c_void_p()
        col._check(_lib().rrg_scene_create(meshes.handle, om.shape[0], om.ctypes.data, w.ctypes.data, C.byref(h)),
                   "rrg_scene_create")
        self._h = h
        self.nobj = int(om.shape[0])

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None) and col._L is not None:
            col._L.rrg_scene_destroy(self._h)
        self._h = None

    def set_matrices(self, world) -> None:
        w = np.ascontiguousarray(world, np.float32).reshape(self.nobj, 12)
        col._check(_lib().rrg_scene_set_matrices(self._h, w.ctypes.data), "rrg_scene_set_matrices")

    def set_enabled(self, enabled) -> None:
        e = np.ascontiguousarray(enabled, np.uint8).reshape(self.nobj)
        col._check(_lib().rrg_scene_set_enabled(self._h, e.ctypes.data), "rrg_scene_set_enabled")

    def intersect_device(self, rays_ptr: int, n: int, hits_ptr: int, objects_ptr: int = 0, stream: int = 0) -> None:
        col._check(_lib().rrg_scene_intersect_device(self._h, rays_ptr, n, hits_ptr, objects_ptr or None,
                                                     stream or None), "rrg_scene_intersect_device")

    def status(self, stream: int = 0) -> int:
        return _lib().rrg_scene_status(self._h, stream or None)

    def intersect(self, rays: np.ndarray):
        """Host convenience: (decoded hits dict, object per ray)."""
        import torch
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        d = torch.from_numpy(rays).cuda()
        h = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        o = torch.empty(n, dtype=torch.int32, device="cuda")
        self.intersect_device(d.data_ptr(), n, h.data_ptr(), o.data_ptr())
        torch.cuda.synchronize()
        col._check(self.status(), "scene trace")
        return col.decode_hits(h.cpu().numpy()), o.cpu().numpy().view(np.uint32)
