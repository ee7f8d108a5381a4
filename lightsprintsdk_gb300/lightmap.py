"""Python mirror of the lightmap final gather (include/rrgpu_gather.h).

Mirrors RRSolver::updateLightmaps with UpdateParameters(quality) for the
plain N-bounce estimator (RRSolver/lightmap.cpp:943-1163,
RRSolver/gather.cpp:600-836): a lightmapper is bound to a collider and the
scene's materials and unwrap; texel ranges of its atlases are gathered on the
GPU.  No CPU fallback: every call goes to the CUDA library or raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import collider as col

SUBTEXEL_DTYPE = np.dtype([("tri", "<u4"), ("uv", "<f4", (3, 2)), ("area", "<f4")])   # 32 bytes


class GatherParams(C.Structure):
    _fields_ = [("size", C.c_uint32), ("quality", C.c_uint32), ("max_depth", C.c_uint32),
                ("mode", C.c_uint32), ("seed", C.c_uint64), ("ray_length_min", C.c_float),
                ("locality", C.c_float), ("dir_direction", C.c_float * 3), ("dir_color", C.c_float * 3),
                ("point_position", C.c_float * 3), ("point_color", C.c_float * 3), ("ao_intensity", C.c_float),
                ("ao_size", C.c_float)]


class FilterParams(C.Structure):
    """rrg_filter_params: RRSolver::FilteringParameters plus the stage mask."""
    _fields_ = [("size", C.c_uint32), ("stages", C.c_uint32), ("smoothing_amount", C.c_float),
                ("spread_foreground", C.c_uint32), ("background", C.c_float * 4), ("wrap", C.c_uint32),
                ("seams", C.c_uint32)]


FILTER_SMOOTH, FILTER_GROW_BILINEAR, FILTER_GROW, FILTER_FILL_BACKGROUND, FILTER_ALL = 1, 2, 4, 8, 15

_bound = False


def _lib():
    global _bound
    L = col._lib()
    if not _bound:
        P, U = C.c_void_p, C.c_uint32
        L.rrg_lightmapper_create.argtypes = [P, P, P, P, U, U, C.POINTER(P)]
        L.rrg_lightmapper_destroy.argtypes = [P]
        L.rrg_lightmapper_destroy.restype = None
        L.rrg_lightmapper_subtexels.argtypes = [P]
        L.rrg_lightmapper_subtexels.restype = C.c_uint64
        L.rrg_lightmapper_ray_length_min.argtypes = [P]
        L.rrg_lightmapper_ray_length_min.restype = C.c_float
        L.rrg_lightmapper_copy_subtexels.argtypes = [P, P, P]
        L.rrg_lightmap_gather.argtypes = [P, C.POINTER(GatherParams), C.c_uint64, C.c_uint64, P, P]
        L.rrg_lightmap_gather_host.argtypes = [P, C.POINTER(GatherParams), C.c_uint64, C.c_uint64, P, P]
        L.rrg_lightmap_gather_ex.argtypes = [P, C.POINTER(GatherParams), C.c_uint64, C.c_uint64, P, P, P]
        L.rrg_lightmap_gather_directional.argtypes = [P, C.POINTER(GatherParams), C.c_uint64, C.c_uint64, P, P, P, P,
                                                      P, P]
        L.rrg_lightmapper_status.argtypes = [P, P]
        L.rrg_lightmapper_copy_flags.argtypes = [P, P]
        L.rrg_lightmapper_bake_solver.argtypes = [P, C.POINTER(GatherParams), U, U, P]
        L.rrg_lightmapper_copy_solver.argtypes = [P, P, P, P]
        L.rrg_lightmapper_copy_factor_hits.argtypes = [P, P, C.c_uint64]
        L.rrg_lightmapper_copy_factor_hits.restype = C.c_uint64
        L.rrg_lightmap_filter.argtypes = [P, C.POINTER(FilterParams), C.c_uint32, C.c_uint32, P, P]
        L.rrg_lightmapper_seams.argtypes = [P]
        L.rrg_lightmapper_seams.restype = C.c_uint64
        L.rrg_lightmapper_seam_runs.argtypes = [P]
        L.rrg_lightmapper_seam_runs.restype = C.c_uint64
        L.rrg_filter_defaults.argtypes = [C.POINTER(FilterParams)]
        L.rrg_filter_defaults.restype = None
        _bound = True
    return L


GATHER_AUTO, GATHER_WARP, GATHER_WAVEFRONT = 0, 1, 2
# flag OR-ed into the mode: the hemisphere reads the baked radiosity solver at its first hit
GATHER_SOLVER = 4


def make_params(lights: dict, quality: int = 64, max_depth: int = 8, seed: int = 0xC2, ray_length_min: float = 0.0,
                locality: float = 100000.0, ao_intensity: float = 0.0, ao_size: float = 0.0,
                mode: int = GATHER_AUTO) -> GatherParams:
    return GatherParams(C.sizeof(GatherParams), quality, max_depth, mode, seed, ray_length_min, locality,
                        (C.c_float * 3)(*lights["dir_direction"]), (C.c_float * 3)(*lights["dir_color"]),
                        (C.c_float * 3)(*lights["point_position"]), (C.c_float * 3)(*lights["point_color"]),
                        ao_intensity, ao_size)


def filter_params(smoothing: float = 1.0, spread: int = 1000, background=(0.0, 0.0, 0.0, 0.0), wrap: bool = False,
                  seams: bool = True, stages: int = FILTER_ALL) -> FilterParams:
    """FilteringParameters (RRSolver.h:596-621); the defaults are the reference's."""
    return FilterParams(C.sizeof(FilterParams), stages, smoothing, spread, (C.c_float * 4)(*background), int(wrap),
                        int(seams))


class RRLightmapper:
    """Sub-texel enumeration and plain gather for the atlases of one scene."""

    def __init__(self, collider: col.RRCollider, albedo, tri_atlas, uv, natlas: int, size: int):
        self.c = collider
        self.albedo = np.ascontiguousarray(albedo, np.float32)
        self.tri_atlas = np.ascontiguousarray(tri_atlas, np.int32)
        self.uv = np.ascontiguousarray(uv, np.float32)
        self.natlas, self.size = natlas, size
        h = C.c_void_p()
        st = _lib().rrg_lightmapper_create(collider.handle, self.albedo.ctypes.data, self.tri_atlas.ctypes.data,
                                           self.uv.ctypes.data, natlas, size, C.byref(h))
        if st:
            raise col.RRGError(st, "rrg_lightmapper_create")
        self._h = h

    @classmethod
    def from_scene(cls, collider, gs) -> "RRLightmapper":
        return cls(collider, gs.albedo, gs.tri_atlas, gs.uv, gs.natlas, gs.size)

    def __del__(self):
        self.close()

    def close(self):
        if getattr(self, "_h", None):
            _lib().rrg_lightmapper_destroy(self._h)
            self._h = None

    @property
    def ntexels(self) -> int:
        return self.natlas * self.size * self.size

    @property
    def nsubtexels(self) -> int:
        return int(_lib().rrg_lightmapper_subtexels(self._h))

    @property
    def ray_length_min(self) -> float:
        return float(_lib().rrg_lightmapper_ray_length_min(self._h))

    def subtexels(self):
        off = np.zeros(self.ntexels + 1, np.uint32)
        st = np.zeros(self.nsubtexels, SUBTEXEL_DTYPE)
        r = _lib().rrg_lightmapper_copy_subtexels(self._h, off.ctypes.data, st.ctypes.data if len(st) else None)
        if r:
            raise col.RRGError(r, "rrg_lightmapper_copy_subtexels")
        return off, st

    def gather(self, params: GatherParams, first: int = 0, count: int | None = None) -> np.ndarray:
        """Texels [first, first+count) -> (count, 4) float32 host array."""
        if count is None:
            count = self.ntexels - first
        out = np.zeros((count, 4), np.float32)
        r = _lib().rrg_lightmap_gather_host(self._h, C.byref(params), first, count, out.ctypes.data, None)
        if r:
            raise col.RRGError(r, "rrg_lightmap_gather_host")
        self.check()
        return out

    def gather_device(self, params: GatherParams, first: int, count: int, out_ptr: int, stream: int = 0,
                      bent_ptr: int = 0) -> None:
        """Device form; bent_ptr (16-byte aligned, 4 floats per texel) also receives the bent normals."""
        if bent_ptr:
            r = _lib().rrg_lightmap_gather_ex(self._h, C.byref(params), first, count, out_ptr, bent_ptr,
                                              stream or None)
        else:
            r = _lib().rrg_lightmap_gather(self._h, C.byref(params), first, count, out_ptr, stream or None)
        if r:
            raise col.RRGError(r, "rrg_lightmap_gather")

    def gather_directional(self, params: GatherParams, first: int = 0, count: int | None = None):
        """Directional mode (rrg_lightmap_gather_directional): host arrays (LS_LIGHTMAP (count,4),
        LS_DIRECTION1..3 (count,3,4), bent normals (count,4))."""
        import torch
        if count is None:
            count = self.ntexels - first
        n = max(count, 1)
        bufs = [torch.empty((n, 4), dtype=torch.float32, device="cuda") for _ in range(5)]
        sp = torch.cuda.current_stream().cuda_stream
        r = _lib().rrg_lightmap_gather_directional(self._h, C.byref(params), first, count,
                                                   *[b.data_ptr() for b in bufs], sp)
        if r:
            raise col.RRGError(r, "rrg_lightmap_gather_directional")
        self.check(sp)
        host = [b[:count].cpu().numpy() for b in bufs]
        return host[0], np.stack(host[1:4], axis=1), host[4]

    def gather_bent(self, params: GatherParams, first: int = 0, count: int | None = None):
        """Texels [first, first+count) -> ((count, 4) irradiance, (count, 4) bent normals) host arrays,
        the bent normals in the reference's LS_BENT_NORMALS encoding (RRSolver/gather.cpp:811-830)."""
        import torch
        if count is None:
            count = self.ntexels - first
        out = torch.empty((max(count, 1), 4), dtype=torch.float32, device="cuda")
        bent = torch.empty((max(count, 1), 4), dtype=torch.float32, device="cuda")
        self.gather_device(params, first, count, out.data_ptr(), torch.cuda.current_stream().cuda_stream,
                           bent.data_ptr())
        self.check(torch.cuda.current_stream().cuda_stream)
        return out[:count].cpu().numpy(), bent[:count].cpu().numpy()

    def bake_solver(self, params: GatherParams, rays_per_triangle: int = 0, iterations: int = 32,
                    stream: int = 0) -> None:
        """The reference's default-bake radiosity solver on the device
        (rrg_lightmapper_bake_solver): first gather per triangle, form-factor
        rays, Jacobi propagation, corner smoothing.  Gathers with
        mode | GATHER_SOLVER then read it at the first hit."""
        r = _lib().rrg_lightmapper_bake_solver(self._h, C.byref(params), rays_per_triangle, iterations, stream or None)
        if r:
            raise col.RRGError(r, "rrg_lightmapper_bake_solver")

    def solver(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(direct irradiance (T,3), indirect irradiance (T,3), smoothed
        corner indirect irradiance (T,3,3))."""
        T = int(self.albedo.shape[0])
        d = np.zeros((T, 3), np.float32)
        i = np.zeros((T, 3), np.float32)
        c = np.zeros((T, 3, 3), np.float32)
        r = _lib().rrg_lightmapper_copy_solver(self._h, d.ctypes.data, i.ctypes.data, c.ctypes.data)
        if r:
            raise col.RRGError(r, "rrg_lightmapper_copy_solver")
        return d, i, c

    def factor_hits(self) -> np.ndarray:
        """The last bake's form-factor ray hits (triangles x rays) uint32."""
        n = int(_lib().rrg_lightmapper_copy_factor_hits(self._h, None, 0))
        out = np.zeros(n, np.uint32)
        if n and int(_lib().rrg_lightmapper_copy_factor_hits(self._h, out.ctypes.data, n)) != n:
            raise col.RRGError(1, "rrg_lightmapper_copy_factor_hits")
        return out

    def flags(self) -> np.ndarray:
        """TexelFlags of every texel (ntexels,) uint8."""
        out = np.zeros(self.ntexels, np.uint8)
        r = _lib().rrg_lightmapper_copy_flags(self._h, out.ctypes.data)
        if r:
            raise col.RRGError(r, "rrg_lightmapper_copy_flags")
        return out

    def filter_device(self, params: FilterParams, first_atlas: int, natlas: int, lightmaps_ptr: int,
                      stream: int = 0) -> None:
        """Post-filters atlases [first_atlas, first_atlas+natlas) of a device lightmap array laid out as the
        gather writes it (float4 per texel, all atlases), in place (rrg_lightmap_filter)."""
        r = _lib().rrg_lightmap_filter(self._h, C.byref(params), first_atlas, natlas, lightmaps_ptr, stream or None)
        if r:
            raise col.RRGError(r, "rrg_lightmap_filter")

    @property
    def nseams(self) -> int:
        return int(_lib().rrg_lightmapper_seams(self._h))

    @property
    def seam_runs(self) -> int:
        return int(_lib().rrg_lightmapper_seam_runs(self._h))

    def set_ray_order(self, order: int) -> None:
        """col.RAY_ORDER_BINNED (live paths sorted by their rays' key before
        each closest-hit pass) or col.RAY_ORDER_DEFAULT / _AS_GIVEN (path
        order)."""
        L = _lib()
        L.rrg_lightmapper_set_ray_order.argtypes = [C.c_void_p, C.c_uint32]
        col._check(L.rrg_lightmapper_set_ray_order(self._h, int(order)), "rrg_lightmapper_set_ray_order")

    def count_rays(self, enable: bool = True) -> tuple[int, int]:
        """(closest-hit rays, shadow rays) the wavefront gather traced since
        the previous call; counting continues while enable."""
        L = _lib()
        L.rrg_lightmapper_count_rays.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        a = np.zeros(2, np.uint64)
        col._check(L.rrg_lightmapper_count_rays(self._h, 1 if enable else 0, a[0:].ctypes.data,
                                                a[1:].ctypes.data), "rrg_lightmapper_count_rays")
        return int(a[0]), int(a[1])

    def check(self, stream: int = 0) -> None:
        r = _lib().rrg_lightmapper_status(self._h, stream or None)
        if r:
            raise col.RRGError(r, "gather")
