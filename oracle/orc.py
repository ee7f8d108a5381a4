"""ctypes front end of the C oracle (rr_oracle.c).  Test infrastructure only:
tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py call it as
the checker; the product never imports it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
SRC = [os.path.join(HERE, "rr_oracle.c"), os.path.join(HERE, "rr_gather.c"), os.path.join(HERE, "rr_mlp.c"),
       os.path.join(HERE, "rr_filter.c")]
HDRS = [os.path.join(HERE, "rr_oracle.h"), os.path.join(HERE, "rr_gather.h")]

_lib = None


def build(force: bool = False) -> str:
    """gcc -O2 -ffp-contract=off -fopenmp: one rounding per float operation, as
    in the reference's own x86-64 build, and the same results on aarch64."""
    newest = max(os.path.getmtime(p) for p in SRC + HDRS)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
                        "-std=c11", "-o", tmp] + SRC + ["-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


class _Hits(C.Structure):
    _fields_ = [("hit", C.c_void_p), ("tri", C.c_void_p), ("dist", C.c_void_p), ("uv", C.c_void_p),
                ("plane", C.c_void_p), ("point3d", C.c_void_p), ("side", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        U = C.c_uint32
        L.orc_collide_linear.argtypes = [P, U, P, U, P, U, C.c_int, C.POINTER(_Hits)]
        L.orc_bvh_build.argtypes = [P, U, P, U]
        L.orc_bvh_build.restype = P
        L.orc_bvh_free.argtypes = [P]
        L.orc_collide_fastest.argtypes = [P, P, U, C.c_int, C.c_int, C.POINTER(_Hits)]
        L.orc_collide_exact64.argtypes = [P, P, U, C.c_int, P, P]
        L.orc_delta_bsp.argtypes = [P, U]
        L.orc_delta_bsp.restype = C.c_float
        L.orc_max_threads.restype = C.c_int
        L.orc_enumerate.argtypes = [P, P, U, U, P, P, P]
        L.orc_enumerate.restype = C.c_uint64
        L.orc_texel_flags.argtypes = [P, U, U, P]
        L.orc_unwrap_seams.argtypes = [P, P, U, P, U]
        L.orc_unwrap_seams.restype = U
        L.orc_lightmap_smooth.argtypes = [P, U, U, C.c_float, C.c_int, P, U]
        L.orc_lightmap_grow_bilinear.argtypes = [P, U, U, C.c_int]
        L.orc_lightmap_grow.argtypes = [P, U, U, U, C.c_int]
        L.orc_lightmap_fill_background.argtypes = [P, U, U, P]
        L.orc_gather.argtypes = [P, C.POINTER(GatherScene), P, U, P, P, C.c_int, C.c_int, P]
        L.orc_gather_ex.argtypes = [P, C.POINTER(GatherScene), P, U, P, P, C.c_int, C.c_int, P, P]
        L.orc_gather_dir.argtypes = [P, C.POINTER(GatherScene), P, U, P, P, C.c_int, C.c_int, P, P, P]
        L.orc_hash.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_bake_direct.argtypes = [P, C.POINTER(GatherScene), C.c_int, P]
        L.orc_bake_factors.argtypes = [P, C.POINTER(GatherScene), U, C.c_int, P]
        L.orc_bake_propagate.argtypes = [C.POINTER(GatherScene), P, P, U, U, P]
        L.orc_bake_stitch.argtypes = [P, P, U, P, P]
        L.orc_bake_stitch.restype = U
        L.orc_bake_smooth.argtypes = [U, P, P, U, P, P]
        L.orc_hash.restype = C.c_uint64
        L.orc_mlp_encode.argtypes = [P, P, P, P, P, P]
        L.orc_mlp_grad.argtypes = [P, P, P, C.c_int, C.c_int, P, P, P]
        L.orc_mlp_encode_hash.argtypes = [P, P, P, P, P, P, P, C.c_uint32, P]
        L.orc_mlp_grad_hash.argtypes = [P, P, P, C.c_uint32, P, P, P, P, P, P, C.c_int, C.c_int, P, P, P, P]
        L.orc_bf16.argtypes = [C.c_double]
        L.orc_bf16.restype = C.c_double
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _alloc_hits(n: int):
    h = {"hit": np.zeros(n, np.uint8), "tri": np.zeros(n, np.uint32), "dist": np.zeros(n, np.float32),
         "uv": np.zeros((n, 2), np.float32), "plane": np.zeros((n, 4), np.float32),
         "point3d": np.zeros((n, 3), np.float32), "side": np.zeros(n, np.uint8)}
    s = _Hits(*[h[k].ctypes.data for k in ("hit", "tri", "dist", "uv", "plane", "point3d", "side")])
    return h, s


def _finish(h):
    h["hit"] = h["hit"].astype(bool)
    h["side"] = h["side"].astype(bool)
    return h


def max_threads() -> int:
    return int(lib().orc_max_threads())


def delta_bsp(v) -> float:
    v = np.ascontiguousarray(v, np.float32)
    return float(lib().orc_delta_bsp(_ptr(v), v.shape[0]))


def collide_linear(v, t, rays, threads: int = 0) -> dict:
    """IT_LINEAR: exhaustive nearest Moller-Trumbore hit."""
    v = np.ascontiguousarray(v, np.float32)
    t = np.ascontiguousarray(t, np.uint32)
    rays = np.ascontiguousarray(rays, np.float32)
    h, s = _alloc_hits(rays.shape[0])
    lib().orc_collide_linear(_ptr(v), v.shape[0], _ptr(t), t.shape[0], _ptr(rays), rays.shape[0], threads,
                             C.byref(s))
    return _finish(h)


class FastestOracle:
    """IT_BSP_FASTEST arithmetic over the oracle's own BVH."""

    def __init__(self, v, t):
        self.v = np.ascontiguousarray(v, np.float32)
        self.t = np.ascontiguousarray(t, np.uint32)
        self.h = lib().orc_bvh_build(_ptr(self.v), self.v.shape[0], _ptr(self.t), self.t.shape[0])

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_bvh_free(self.h)
            self.h = None

    def collide(self, rays, threads: int = 0, any_hit: bool = False) -> dict:
        rays = np.ascontiguousarray(rays, np.float32)
        h, s = _alloc_hits(rays.shape[0])
        lib().orc_collide_fastest(self.h, _ptr(rays), rays.shape[0], threads, int(any_hit), C.byref(s))
        return _finish(h)

    def exact64(self, rays, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        tri = np.zeros(n, np.uint32)
        dist = np.zeros(n, np.float64)
        lib().orc_collide_exact64(self.h, _ptr(rays), n, threads, _ptr(tri), _ptr(dist))
        return tri, dist


# ------------------------------------------------------------------ gather
SUBTEXEL_DTYPE = np.dtype([("tri", "<u4"), ("uv", "<f4", (3, 2)), ("area", "<f4")])   # 32 bytes


class GatherScene(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("idx", C.c_void_p), ("nt", C.c_uint32), ("albedo", C.c_void_p),
                ("dir_direction", C.c_float * 3), ("dir_color", C.c_float * 3), ("point_position", C.c_float * 3),
                ("point_color", C.c_float * 3), ("ray_length_min", C.c_float), ("locality", C.c_float),
                ("quality", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint64),
                ("ao_intensity", C.c_float), ("ao_size", C.c_float), ("flags", C.c_void_p),
                ("solver_direct", C.c_void_p), ("solver_corner", C.c_void_p)]


def hash_u64(seed: int, stream: int, index: int) -> int:
    return int(lib().orc_hash(seed, stream, index))


def enumerate_atlas(uv_map: np.ndarray, tri_ids: np.ndarray, size: int):
    """Sub-texels of one atlas (lightmap.cpp:145-330 restated).  uv_map: (n,3,2)
    map-space corners of the atlas' triangles, tri_ids their world indices in
    visiting order.  Returns (offsets (size*size+1,) uint64, subtexels)."""
    uv_map = np.ascontiguousarray(uv_map, np.float32)
    tri_ids = np.ascontiguousarray(tri_ids, np.uint32)
    n = tri_ids.shape[0]
    counts = np.zeros(size * size, np.uint32)
    L = lib()
    total = L.orc_enumerate(_ptr(uv_map), _ptr(tri_ids), n, size, _ptr(counts), None, None)
    off = np.zeros(size * size + 1, np.uint64)
    np.cumsum(counts, out=off[1:])
    st = np.zeros(int(total), SUBTEXEL_DTYPE)
    L.orc_enumerate(_ptr(uv_map), _ptr(tri_ids), n, size, _ptr(counts), _ptr(off), _ptr(st) if total else None)
    return off, st


def texel_flags(uv_map: np.ndarray, size: int) -> np.ndarray:
    """TexelFlags of one atlas (lightmap.cpp:283-314 restated): (size*size,)
    uint8 from the atlas' triangles' map-space corners (n,3,2)."""
    uv_map = np.ascontiguousarray(uv_map, np.float32)
    flags = np.zeros(size * size, np.uint8)
    lib().orc_texel_flags(_ptr(uv_map), uv_map.shape[0], size, _ptr(flags))
    return flags


def gather_flags(gs, atlases) -> np.ndarray:
    """TexelFlags by global texel id for the given atlases of a gather scene
    (other atlases 0)."""
    S = gs.size * gs.size
    flags = np.zeros(gs.natlas * S, np.uint8)
    for a in atlases:
        ids = np.nonzero(gs.tri_atlas == a)[0]
        flags[a * S:(a + 1) * S] = texel_flags(gs.uv[ids], gs.size)
    return flags


def unwrap_seams(idx: np.ndarray, uv_map: np.ndarray) -> np.ndarray:
    """UnwrapSeams (RRBuffer.cpp:534-628 restated, vertices shared by index)
    of one object: idx (n,3) vertex indices, uv_map (n,3,2) in the object's
    triangle order -> (m, 8) float32 (edge1 from, edge1 to, edge2 from, edge2 to)."""
    idx = np.ascontiguousarray(idx, np.uint32)
    uv_map = np.ascontiguousarray(uv_map, np.float32)
    n = idx.shape[0]
    m = lib().orc_unwrap_seams(_ptr(idx), _ptr(uv_map), n, None, 0)
    out = np.zeros((max(m, 1), 8), np.float32)
    lib().orc_unwrap_seams(_ptr(idx), _ptr(uv_map), n, _ptr(out), m)
    return out[:m]


FILTER_SMOOTH, FILTER_GROW_BILINEAR, FILTER_GROW, FILTER_FILL_BACKGROUND = 1, 2, 4, 8


def lightmap_filter(rgba: np.ndarray, smoothing: float = 1.0, spread: int = 1000, background=(0, 0, 0, 0),
                    wrap: bool = False, seams: np.ndarray | None = None, stages: int = 15) -> np.ndarray:
    """The post-filters of updateLightmap (lightmap.cpp:865-874) in order on one
    lightmap (h, w, 4) float32; returns the filtered copy."""
    out = np.ascontiguousarray(rgba, np.float32).copy()
    h, w = out.shape[0], out.shape[1]
    L = lib()
    sm = np.ascontiguousarray(seams if seams is not None else np.zeros((0, 8)), np.float32)
    if stages & FILTER_SMOOTH:
        L.orc_lightmap_smooth(_ptr(out), w, h, smoothing, int(wrap), _ptr(sm) if len(sm) else None, len(sm))
    if stages & FILTER_GROW_BILINEAR:
        L.orc_lightmap_grow_bilinear(_ptr(out), w, h, int(wrap))
    if stages & FILTER_GROW:
        L.orc_lightmap_grow(_ptr(out), w, h, spread, int(wrap))
    if stages & FILTER_FILL_BACKGROUND:
        bg = np.asarray(background, np.float32)
        L.orc_lightmap_fill_background(_ptr(out), w, h, _ptr(bg))
    return out


def min_safe_distance(v: np.ndarray) -> float:
    """RRSolver::setStaticObjects: (aabb max - min).avg() * 1e-6 (RRSolver.cpp:329-334)."""
    v = np.asarray(v, np.float32)
    ext = (v.max(0) - v.min(0)).astype(np.float32)
    return float(np.float32((ext[0] + ext[1] + ext[2]) * np.float32(0.33333333333333)) * np.float32(1e-6))


class GatherOracle:
    """Plain N-bounce lightmap gather on the CPU (rr_gather.c)."""

    def __init__(self, gs, quality: int = 64, max_depth: int = 8, seed: int = 0xC2, locality: float = 100000.0,
                 bvh: "FastestOracle | None" = None, ao_intensity: float = 0.0, ao_size: float = 0.0,
                 flags: np.ndarray | None = None):
        """flags: TexelFlags by global texel id (alpha = flags/255); None: alpha 1."""
        sc = gs.scene
        self.flags = None if flags is None else np.ascontiguousarray(flags, np.uint8)
        self.fo = bvh or FastestOracle(sc.vertices, sc.indices)
        self.albedo = np.ascontiguousarray(gs.albedo, np.float32)
        L = gs.lights
        self.s = GatherScene(self.fo.v.ctypes.data, self.fo.t.ctypes.data, self.fo.t.shape[0], self.albedo.ctypes.data,
                             (C.c_float * 3)(*L["dir_direction"]), (C.c_float * 3)(*L["dir_color"]),
                             (C.c_float * 3)(*L["point_position"]), (C.c_float * 3)(*L["point_color"]),
                             min_safe_distance(sc.vertices), locality, quality, max_depth, seed, ao_intensity,
                             ao_size, None if self.flags is None else self.flags.ctypes.data)

    def bake_solver(self, rays_per_triangle: int = 0, iterations: int = 32, threads: int = 0):
        """The default bake's radiosity solver (rr_gather.c, bake section) at
        this oracle's quality and seed: per-triangle direct irradiance (first
        gather at half quality), form-factor rays (rays_per_triangle, 0 =
        the quality), Jacobi propagation, corner smoothing.  Returns
        (direct (T,3), indirect (T,3), corner (T,3,3)) and makes the later
        gathers read the solver at the first hit."""
        sc = self.s
        T = int(sc.nt)
        k = int(rays_per_triangle or sc.quality)
        L = lib()
        direct = np.zeros((T, 3), np.float32)
        L.orc_bake_direct(self.fo.h, C.byref(sc), threads, _ptr(direct))
        hits = np.zeros(T * k, np.uint32)
        L.orc_bake_factors(self.fo.h, C.byref(sc), k, threads, _ptr(hits))
        self.factor_hits = hits
        indirect = np.zeros((T, 3), np.float32)
        L.orc_bake_propagate(C.byref(sc), _ptr(direct), _ptr(hits), k, iterations, _ptr(indirect))
        group = np.zeros(3 * T, np.uint32)
        weight = np.zeros(3 * T, np.float32)
        ng = L.orc_bake_stitch(self.fo.v.ctypes.data, self.fo.t.ctypes.data, T, _ptr(group), _ptr(weight))
        corner = np.zeros((T, 3, 3), np.float32)
        L.orc_bake_smooth(T, _ptr(group), _ptr(weight), ng, _ptr(indirect), _ptr(corner))
        self.solver = (direct, corner)
        self.s.solver_direct = direct.ctypes.data
        self.s.solver_corner = corner.ctypes.data
        return direct, indirect, corner

    def gather(self, texel_ids: np.ndarray, off: np.ndarray, st: np.ndarray, threads: int = 0,
               fp64: bool = False, bent: bool = False):
        """texel_ids (n,) global ids; off (n+1,) offsets into st for these
        texels.  Returns (n,4) float32, or (that, bent normals (n,4)) with bent."""
        texel_ids = np.ascontiguousarray(texel_ids, np.uint64)
        off = np.ascontiguousarray(off, np.uint64)
        st = np.ascontiguousarray(st)
        out = np.zeros((texel_ids.shape[0], 4), np.float32)
        bn = np.zeros((texel_ids.shape[0], 4), np.float32) if bent else None
        lib().orc_gather_ex(self.fo.h, C.byref(self.s), _ptr(texel_ids), texel_ids.shape[0], _ptr(off),
                            _ptr(st) if len(st) else None, threads, int(fp64), _ptr(out),
                            _ptr(bn) if bent else None)
        return (out, bn) if bent else out

    def gather_directional(self, texel_ids: np.ndarray, off: np.ndarray, st: np.ndarray, threads: int = 0):
        """Directional mode: (LS_LIGHTMAP (n,4), LS_DIRECTION1..3 (n,3,4), bent normals (n,4))."""
        texel_ids = np.ascontiguousarray(texel_ids, np.uint64)
        off = np.ascontiguousarray(off, np.uint64)
        st = np.ascontiguousarray(st)
        n = texel_ids.shape[0]
        out = np.zeros((n, 4), np.float32)
        bn = np.zeros((n, 4), np.float32)
        dirs = np.zeros((n, 3, 4), np.float32)
        lib().orc_gather_dir(self.fo.h, C.byref(self.s), _ptr(texel_ids), n, _ptr(off), _ptr(st) if len(st) else None,
                             threads, 0, _ptr(out), _ptr(bn), _ptr(dirs))
        return out, dirs, bn


# --------------------------------------------------------------- network
def mlp_encode(p, n, alb, lo, hi) -> np.ndarray:
    """Encoded inputs (B, 64) in double (rr_mlp.c)."""
    p = np.ascontiguousarray(p, np.float32).reshape(-1, 3)
    n = np.ascontiguousarray(n, np.float32).reshape(-1, 3)
    alb = np.ascontiguousarray(alb, np.float32).reshape(-1, 3)
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    out = np.zeros((p.shape[0], 64), np.float64)
    L = lib()
    for i in range(p.shape[0]):
        L.orc_mlp_encode(_ptr(p[i]), _ptr(n[i]), _ptr(alb[i]), _ptr(lo), _ptr(hi), out[i].ctypes.data_as(C.c_void_p))
    return out


def mlp_grad(W, X, T, bf16: bool = True):
    """Mean relative-L2 loss gradient over the batch in double: (dW, loss, Y)."""
    W = np.ascontiguousarray(W, np.float32)
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    B = X.shape[0]
    dW = np.zeros(W.shape[0], np.float64)
    loss = np.zeros(1, np.float64)
    Y = np.zeros((B, 3), np.float32)
    lib().orc_mlp_grad(_ptr(W), _ptr(X), _ptr(T), B, int(bf16), _ptr(dW), _ptr(loss), _ptr(Y))
    return dW, float(loss[0]), Y


def hashgrid_res(levels: int = 16, min_res: float = 16.0, max_res: float = 1024.0) -> np.ndarray:
    """Per-level grid resolutions of the hash encoding (rr_mlp.c):
    floor(min_res * b^l), b = (max_res / min_res)^(1 / (levels - 1))."""
    b = np.exp((np.log(max_res) - np.log(min_res)) / (levels - 1))
    return np.floor(min_res * b ** np.arange(levels)).astype(np.int32)


def mlp_encode_hash(p, n, alb, lo, ie, table, res, T):
    """Hash-grid encoded inputs (B, 64) in double (rr_mlp.c)."""
    p = np.ascontiguousarray(p, np.float32).reshape(-1, 3)
    n = np.ascontiguousarray(n, np.float32).reshape(-1, 3)
    alb = np.ascontiguousarray(alb, np.float32).reshape(-1, 3)
    lo = np.ascontiguousarray(lo, np.float32)
    ie = np.ascontiguousarray(ie, np.float32)
    table = np.ascontiguousarray(table, np.float32)
    res = np.ascontiguousarray(res, np.int32)
    out = np.zeros((p.shape[0], 64), np.float64)
    L = lib()
    for i in range(p.shape[0]):
        L.orc_mlp_encode_hash(_ptr(p[i]), _ptr(n[i]), _ptr(alb[i]), _ptr(lo), _ptr(ie), _ptr(table), _ptr(res), T,
                              out[i].ctypes.data_as(C.c_void_p))
    return out


def mlp_grad_hash(W, table, res, T, lo, ie, p, n, alb, t, bf16: bool = True):
    """(dW, dTable, loss, Y) of the hash-grid network (rr_mlp.c); Y in double."""
    W = np.ascontiguousarray(W, np.float32)
    table = np.ascontiguousarray(table, np.float32)
    res = np.ascontiguousarray(res, np.int32)
    lo = np.ascontiguousarray(lo, np.float32)
    ie = np.ascontiguousarray(ie, np.float32)
    p = np.ascontiguousarray(p, np.float32)
    n = np.ascontiguousarray(n, np.float32)
    alb = np.ascontiguousarray(alb, np.float32)
    t = np.ascontiguousarray(t, np.float32)
    B = p.shape[0]
    dW = np.zeros(W.shape[0], np.float64)
    dT = np.zeros(table.shape[0], np.float64)
    loss = np.zeros(1, np.float64)
    Y = np.zeros((B, 3), np.float64)
    lib().orc_mlp_grad_hash(_ptr(W), _ptr(table), _ptr(res), T, _ptr(lo), _ptr(ie), _ptr(p), _ptr(n), _ptr(alb),
                            _ptr(t), B, int(bf16), _ptr(dW), _ptr(dT), _ptr(loss), _ptr(Y))
    return dW, dT, float(loss[0]), Y


# ------------------------------------------------------------------ scenes
def invert3x4(m: np.ndarray) -> np.ndarray:
    """RRMatrix3x4::invertedTo (RRMath.cpp:605-628) in float32, same order of
    operations: cofactors over the float determinant."""
    m = np.asarray(m, np.float32).reshape(3, 4)
    f = np.float32
    det = f(m[0, 0] * f(m[1, 1] * m[2, 2] - m[2, 1] * m[1, 2])) + f(m[0, 1] * f(m[1, 2] * m[2, 0] - m[2, 2] * m[1, 0]))
    det = f(det + f(m[0, 2] * f(m[1, 0] * m[2, 1] - m[2, 0] * m[1, 1])))
    d = np.zeros((3, 4), np.float32)
    d[0, 0] = f(m[2, 2] * m[1, 1] - m[2, 1] * m[1, 2]) / det
    d[0, 1] = -f(m[2, 2] * m[0, 1] - m[2, 1] * m[0, 2]) / det
    d[0, 2] = f(m[1, 2] * m[0, 1] - m[1, 1] * m[0, 2]) / det
    d[1, 0] = -f(m[2, 2] * m[1, 0] - m[2, 0] * m[1, 2]) / det
    d[1, 1] = f(m[2, 2] * m[0, 0] - m[2, 0] * m[0, 2]) / det
    d[1, 2] = -f(m[1, 2] * m[0, 0] - m[1, 0] * m[0, 2]) / det
    d[2, 0] = f(m[2, 1] * m[1, 0] - m[2, 0] * m[1, 1]) / det
    d[2, 1] = -f(m[2, 1] * m[0, 0] - m[2, 0] * m[0, 1]) / det
    d[2, 2] = f(m[1, 1] * m[0, 0] - m[1, 0] * m[0, 1]) / det
    for r in range(3):
        d[r, 3] = f(f(f(-m[0, 3]) * d[r, 0]) - f(m[1, 3] * d[r, 1])) - f(m[2, 3] * d[r, 2])
    return d, float(det)


def local_rays(rays: np.ndarray, inv: np.ndarray):
    """Object-space rays of RRColliderMulti::intersect (RRColliderMulti.cpp:121-131)
    in float32, one rounding per operation: (rays, scale)."""
    r = np.asarray(rays, np.float32)
    m = inv
    o, dd = r[:, 0:3], r[:, 4:7]
    out = np.empty_like(r)
    for k in range(3):
        out[:, k] = ((o[:, 0] * m[k, 0] + o[:, 1] * m[k, 1]) + o[:, 2] * m[k, 2]) + m[k, 3]
    d = np.stack([(dd[:, 0] * m[k, 0] + dd[:, 1] * m[k, 1]) + dd[:, 2] * m[k, 2] for k in range(3)], -1)
    scale = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
    out[:, 4:7] = d / scale[:, None]
    out[:, 3] = r[:, 3] * scale
    out[:, 7] = r[:, 7] * scale
    return out, scale


def scene_collide(meshes, obj_mesh, world, rays) -> tuple:
    """Closest hit over objects (meshes[i] = (v, t) local; obj_mesh; world
    (nobj, 3, 4)) as RRColliderMulti computes it, with the FASTEST oracle per
    object: the object-space hit of each object, hitDistance / scale, the
    nearest world distance (ties: the lower object), hitFrontSide flipped for a
    negative determinant.  Returns (hits dict as FastestOracle.collide, object
    per ray, 0xFFFFFFFF = none)."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    oracles = {}
    best = {"hit": np.zeros(n, bool), "tri": np.full(n, 0xFFFFFFFF, np.uint32),
            "dist": np.zeros(n, np.float32), "uv": np.zeros((n, 2), np.float32), "side": np.zeros(n, bool)}
    obj = np.full(n, 0xFFFFFFFF, np.uint32)
    for o in range(len(obj_mesh)):
        m = int(obj_mesh[o])
        if m not in oracles:
            oracles[m] = FastestOracle(*meshes[m])
        inv, det = invert3x4(np.asarray(world[o], np.float32))
        lr, scale = local_rays(rays, inv)
        h = oracles[m].collide(lr, 0)
        dw = (h["dist"] / scale).astype(np.float32)
        take = h["hit"] & (~best["hit"] | (dw < best["dist"]))
        best["hit"] |= take
        best["tri"][take] = h["tri"][take]
        best["dist"][take] = dw[take]
        best["uv"][take] = h["uv"][take]
        best["side"][take] = h["side"][take] ^ (det < 0)
        obj[take] = o
    return best, obj
