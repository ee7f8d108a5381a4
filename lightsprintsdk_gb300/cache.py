"""Python mirror of the learned radiance cache (include/rrgpu_cache.h) and
the learned lightmap gather (rrg_lightmap_train_samples /
rrg_lightmap_gather_learned in include/rrgpu_gather.h).

The cache has no counterpart in the reference: it replaces the bounces past
the first of the plain gather, which remains its fallback and the yardstick of
its error."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import collider as col
from . import lightmap as lm

REC_DTYPE = np.dtype([("p", "<f4", 3), ("n", "<f4", 3), ("alb", "<f4", 3), ("t", "<f4", 3)])   # 48 bytes
NPARAMS = 4 * 64 * 64 + 64 * 16

FREQUENCY, HASHGRID = 0, 1      # RRG_CACHE_*
TRAIN_RECORDS_PER_PATH = 4      # records of a training path (rrg_lightmap_train_samples)


class CacheParams(C.Structure):
    _fields_ = [("size", C.c_uint32), ("encoding", C.c_uint32), ("lo", C.c_float * 3), ("hi", C.c_float * 3),
                ("seed", C.c_uint64), ("log2_table", C.c_uint32), ("min_res", C.c_float), ("max_res", C.c_float),
                ("reserved", C.c_uint32 * 4)]


_bound = False


def _lib():
    global _bound
    L = lm._lib()
    if not _bound:
        P, U, U64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.rrg_cache_create.argtypes = [P, P, U64, C.POINTER(P)]
        L.rrg_cache_create_ex.argtypes = [C.POINTER(CacheParams), C.POINTER(P)]
        L.rrg_cache_table_floats.argtypes = [P]
        L.rrg_cache_table_floats.restype = U64
        L.rrg_cache_get_table.argtypes = [P, P]
        L.rrg_cache_set_table.argtypes = [P, P]
        L.rrg_cache_get_resolutions.argtypes = [P, P]
        L.rrg_cache_gradient_ex.argtypes = [P, P, U, P, P, P, P]
        L.rrg_cache_destroy.argtypes = [P]
        L.rrg_cache_destroy.restype = None
        L.rrg_cache_set_weights.argtypes = [P, P]
        L.rrg_cache_get_weights.argtypes = [P, P]
        L.rrg_cache_set_adam.argtypes = [P, C.c_float, C.c_float, C.c_float, C.c_float]
        L.rrg_cache_gradient.argtypes = [P, P, U, P, P, P]
        L.rrg_cache_train.argtypes = [P, P, U, U, U, P, P]
        L.rrg_cache_infer.argtypes = [P, P, U64, P, P]
        L.rrg_cache_steps.argtypes = [P]
        L.rrg_cache_steps.restype = U64
        L.rrg_cache_build_error_grid.argtypes = [P, P, U64, U, C.c_float, U, P, P]
        L.rrg_cache_build_error_grid_ex.argtypes = [P, P, U64, U, C.c_float, U, C.c_float, P, P]
        L.rrg_lightmapper_covered.argtypes = [P]
        L.rrg_lightmapper_covered.restype = U64
        L.rrg_lightmap_train_samples.argtypes = [P, C.POINTER(lm.GatherParams), U, U, P, U64, P, P]
        L.rrg_lightmap_gather_learned.argtypes = [P, P, C.POINTER(lm.GatherParams), U64, U64, P, C.c_float, P, P]
        _bound = True
    return L


def _check(st, what):
    if st:
        raise col.RRGError(st, what)


class RadianceCache:
    """encoding: FREQUENCY or HASHGRID (log2_table entries per level, grid
    resolutions min_res..max_res); see include/rrgpu_cache.h."""

    def __init__(self, lo, hi, seed: int = 1, encoding: int = FREQUENCY, log2_table: int = 19,
                 min_res: float = 16.0, max_res: float = 1024.0):
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        p = CacheParams()
        p.size = C.sizeof(CacheParams)
        p.encoding = encoding
        for k in range(3):
            p.lo[k] = float(lo[k])
            p.hi[k] = float(hi[k])
        p.seed = seed
        p.log2_table = log2_table
        p.min_res = min_res
        p.max_res = max_res
        h = C.c_void_p()
        _check(_lib().rrg_cache_create_ex(C.byref(p), C.byref(h)), "rrg_cache_create_ex")
        self._h = h
        self.lo, self.hi = lo, hi
        self.encoding = encoding

    @classmethod
    def for_scene(cls, vertices, seed: int = 1, pad: float = 1e-3, **kw):
        v = np.asarray(vertices, np.float32)
        lo, hi = v.min(0), v.max(0)
        ext = hi - lo
        return cls(lo - pad * ext, hi + pad * ext, seed, **kw)

    @property
    def inv_extent(self) -> np.ndarray:
        """1 / (hi - lo) in float32, as the library computes it."""
        return (np.float32(1.0) / (self.hi - self.lo).astype(np.float32)).astype(np.float32)

    @property
    def table_floats(self) -> int:
        return int(_lib().rrg_cache_table_floats(self._h))

    def get_table(self) -> np.ndarray:
        t = np.zeros(self.table_floats, np.float32)
        _check(_lib().rrg_cache_get_table(self._h, t.ctypes.data), "get_table")
        return t

    def set_table(self, t) -> None:
        t = np.ascontiguousarray(t, np.float32)
        assert t.shape == (self.table_floats,)
        _check(_lib().rrg_cache_set_table(self._h, t.ctypes.data), "set_table")

    def resolutions(self) -> np.ndarray:
        r = np.zeros(16, np.float32)
        _check(_lib().rrg_cache_get_resolutions(self._h, r.ctypes.data), "get_resolutions")
        return r

    def __del__(self):
        if getattr(self, "_h", None):
            _lib().rrg_cache_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def steps(self) -> int:
        return int(_lib().rrg_cache_steps(self._h))

    def get_weights(self) -> np.ndarray:
        w = np.zeros(NPARAMS, np.float32)
        _check(_lib().rrg_cache_get_weights(self._h, w.ctypes.data), "get_weights")
        return w

    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        assert w.shape == (NPARAMS,)
        _check(_lib().rrg_cache_set_weights(self._h, w.ctypes.data), "set_weights")

    def set_adam(self, lr=5e-3, beta1=0.9, beta2=0.99, eps=1e-8):
        _check(_lib().rrg_cache_set_adam(self._h, lr, beta1, beta2, eps), "set_adam")

    def gradient(self, recs: np.ndarray):
        """One forward/backward on host records (no update): (grad, loss, pred)."""
        recs = np.ascontiguousarray(recs, REC_DTYPE)
        B = recs.shape[0]
        g = np.zeros(NPARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        pred = np.zeros((B, 3), np.float32)
        _check(_lib().rrg_cache_gradient(self._h, recs.ctypes.data, B, g.ctypes.data, loss.ctypes.data,
                                         pred.ctypes.data), "rrg_cache_gradient")
        return g, float(loss[0]), pred

    def gradient_ex(self, recs: np.ndarray):
        """gradient() plus the hash table's gradient: (grad, table_grad, loss, pred)."""
        recs = np.ascontiguousarray(recs, REC_DTYPE)
        B = recs.shape[0]
        g = np.zeros(NPARAMS, np.float32)
        tg = np.zeros(self.table_floats, np.float32)
        loss = np.zeros(1, np.float32)
        pred = np.zeros((B, 3), np.float32)
        _check(_lib().rrg_cache_gradient_ex(self._h, recs.ctypes.data, B, g.ctypes.data, tg.ctypes.data,
                                            loss.ctypes.data, pred.ctypes.data), "rrg_cache_gradient_ex")
        return g, tg, float(loss[0]), pred

    def train(self, recs_ptr: int, nrec: int, batch: int = 16384, steps: int = 1, stream: int = 0) -> float:
        loss = np.zeros(1, np.float32)
        _check(_lib().rrg_cache_train(self._h, recs_ptr, nrec, batch, steps, loss.ctypes.data, stream or None),
               "rrg_cache_train")
        return float(loss[0])

    def infer(self, recs_ptr: int, n: int, out_ptr: int, stream: int = 0) -> None:
        _check(_lib().rrg_cache_infer(self._h, recs_ptr, n, out_ptr, stream or None), "rrg_cache_infer")

    def build_error_grid(self, recs_ptr: int, nrec: int, res: int = 32, rel_threshold: float = 0.25,
                         min_count: int = 32, stream: int = 0, plain_samples: float = 0.0) -> int:
        n = np.zeros(1, np.uint32)
        _check(_lib().rrg_cache_build_error_grid_ex(self._h, recs_ptr, nrec, res, rel_threshold, min_count,
                                                    plain_samples, n.ctypes.data, stream or None), "build_error_grid")
        return int(n[0])


def covered(L: lm.RRLightmapper) -> int:
    return int(_lib().rrg_lightmapper_covered(L._h))


def train_samples(L: lm.RRLightmapper, params, stride: int, paths_per_texel: int, recs_ptr: int, cap: int,
                  stream: int = 0) -> int:
    n = np.zeros(1, np.uint64)
    _check(_lib().rrg_lightmap_train_samples(L._h, C.byref(params), stride, paths_per_texel, recs_ptr, cap,
                                             n.ctypes.data, stream or None), "rrg_lightmap_train_samples")
    return int(n[0])


def gather_learned(L: lm.RRLightmapper, cache: RadianceCache, params, first: int, count: int, out_ptr: int,
                   fallback_frac: float = 0.25, stream: int = 0) -> int:
    nf = np.zeros(1, np.uint64)
    _check(_lib().rrg_lightmap_gather_learned(L._h, cache.handle, C.byref(params), first, count, out_ptr,
                                              fallback_frac, nf.ctypes.data, stream or None),
           "rrg_lightmap_gather_learned")
    return int(nf[0])


def bake_learned(L: lm.RRLightmapper, cache: RadianceCache, params, first: int, count: int, out_ptr: int,
                 stride: int = 16, paths_per_texel: int = 4, batch: int = 16384, steps: int = 300,
                 grid_res: int = 32, rel_threshold: float = 0.25, min_count: int = 32,
                 fallback_frac: float = 0.25, stream: int = 0, use_fallback: bool = True,
                 noise_aware: bool = True):
    """Online bake: training records from the gather's own paths, `steps`
    Adam steps, the error grid, then the learned gather with fallback.
    noise_aware: a cell falls back only when the cache's bias there exceeds
    the noise of the plain gather's quality-sample mean too.
    Returns a dict of counts and the last training loss."""
    import torch
    ncov = covered(L)
    npaths = (ncov + stride - 1) // stride * paths_per_texel
    cap = max(1, int(npaths * TRAIN_RECORDS_PER_PATH))
    st = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    ev[0].record(st)
    recs = torch.empty(cap * REC_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    nrec = train_samples(L, params, stride, paths_per_texel, recs.data_ptr(), cap, stream)
    ev[1].record(st)
    loss = cache.train(recs.data_ptr(), nrec, batch, steps, stream)
    ev[2].record(st)
    nrel = cache.build_error_grid(recs.data_ptr(), nrec, grid_res, rel_threshold, min_count, stream,
                                  float(params.quality) if noise_aware else 0.0) if use_fallback else 0
    ev[3].record(st)
    nfb = gather_learned(L, cache, params, first, count, out_ptr, fallback_frac if use_fallback else 2.0, stream)
    ev[4].record(st)
    ev[4].synchronize()
    ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]
    return {"train_records": nrec, "loss": loss, "reliable_cells": nrel, "fallback_texels": nfb,
            "ms": {"train_paths": ms[0], "train_steps": ms[1], "error_grid": ms[2], "learned_gather": ms[3]}}
