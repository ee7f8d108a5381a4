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
SRC = [os.path.join(HERE, "rr_oracle.c")]
HDR = os.path.join(HERE, "rr_oracle.h")

_lib = None


def build(force: bool = False) -> str:
    """gcc -O2 -ffp-contract=off -fopenmp: one rounding per float operation, as
    in the reference's own x86-64 build, and the same results on aarch64."""
    newest = max(os.path.getmtime(p) for p in SRC + [HDR])
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
