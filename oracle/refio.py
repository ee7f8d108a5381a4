"""Binary file formats shared by the oracle drivers, and a runner for the
reference collider built into oracle/_ref.  Test infrastructure only: tests,
fixture generators and the CPU-baseline leg of the benchmark use it as the
checker; nothing in the product imports it.

MESH "RGM1": u32 nv, u32 nt, f32 xyz[nv*3], u32 idx[nt*3]
RAYS "RGR1": u32 n, f32 [n*8] = ox oy oz tmin dx dy dz tmax
HITS "RGH1": u32 n, hit u8[n], tri u32[n], dist f32[n], uv f32[2n],
             plane f32[4n], point3d f32[3n], side u8[n]
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

# RRRay::Flags (include/Lightsprint/RRCollider.h:98-106)
FILL_DISTANCE, FILL_POINT3D, FILL_POINT2D, FILL_PLANE, FILL_TRIANGLE, FILL_SIDE = 1, 2, 4, 8, 16, 32
FILL_ALL = 63


def write_mesh(path: str, v: np.ndarray, t: np.ndarray) -> None:
    v = np.ascontiguousarray(v, np.float32)
    t = np.ascontiguousarray(t, np.uint32)
    with open(path, "wb") as f:
        f.write(b"RGM1")
        f.write(np.array([v.shape[0], t.shape[0]], np.uint32).tobytes())
        f.write(v.tobytes())
        f.write(t.tobytes())


def write_rays(path: str, rays: np.ndarray) -> None:
    rays = np.ascontiguousarray(rays, np.float32)
    with open(path, "wb") as f:
        f.write(b"RGR1")
        f.write(np.array([rays.shape[0]], np.uint32).tobytes())
        f.write(rays.tobytes())


def read_hits(path: str) -> dict:
    b = open(path, "rb").read()
    assert b[:4] == b"RGH1"
    n = int(np.frombuffer(b, np.uint32, 1, 4)[0])
    off = 8
    out = {}
    for name, dt, k in (("hit", np.uint8, 1), ("tri", np.uint32, 1), ("dist", np.float32, 1),
                        ("uv", np.float32, 2), ("plane", np.float32, 4), ("point3d", np.float32, 3),
                        ("side", np.uint8, 1)):
        cnt = n * k
        a = np.frombuffer(b, dt, cnt, off)
        off += cnt * np.dtype(dt).itemsize
        out[name] = a.reshape(n, k) if k > 1 else a.copy()
    out["hit"] = out["hit"].astype(bool)
    out["side"] = out["side"].astype(bool)
    return out


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_collide"))


def run_ref_collide(v, t, rays, technique: str = "bsp_fastest", threads: int = 0,
                    flags: int = FILL_ALL, repeat: int = 1, want_hits: bool = True):
    """Runs the reference collider; returns (timing dict, hits dict or None)."""
    exe = os.path.join(REF_DIR, "ref_collide")
    with tempfile.TemporaryDirectory() as d:
        mp, rp, hp = os.path.join(d, "m"), os.path.join(d, "r"), os.path.join(d, "h")
        write_mesh(mp, v, t)
        write_rays(rp, rays)
        res = subprocess.run([exe, mp, rp, hp if want_hits else "-", technique, str(threads), str(flags),
                              str(repeat)], capture_output=True, text=True, check=True)
        timing = json.loads(res.stdout.strip().splitlines()[-1])
        hits = read_hits(hp) if want_hits else None
    return timing, hits


# LIGHTMAP "RGL1": u32 width, u32 height, f32 rgba[width*height*4]
# UNWRAP   "RGU1": u32 nv, u32 nt, f32 xyz[3nv], f32 normal[3nv], u32 idx[3nt], f32 uv[6nt]
def write_lightmap(path: str, rgba: np.ndarray) -> None:
    rgba = np.ascontiguousarray(rgba, np.float32)
    h, w = rgba.shape[0], rgba.shape[1]
    with open(path, "wb") as f:
        f.write(b"RGL1")
        f.write(np.array([w, h], np.uint32).tobytes())
        f.write(rgba.tobytes())


def read_lightmap(path: str) -> np.ndarray:
    b = open(path, "rb").read()
    assert b[:4] == b"RGL1"
    w, h = np.frombuffer(b, np.uint32, 2, 4)
    return np.frombuffer(b, np.float32, int(w) * int(h) * 4, 12).reshape(int(h), int(w), 4).copy()


def write_unwrap(path: str, v, normals, t, uv) -> None:
    v = np.ascontiguousarray(v, np.float32)
    with open(path, "wb") as f:
        f.write(b"RGU1")
        f.write(np.array([v.shape[0], len(t)], np.uint32).tobytes())
        f.write(v.tobytes())
        f.write(np.ascontiguousarray(normals, np.float32).tobytes())
        f.write(np.ascontiguousarray(t, np.uint32).tobytes())
        f.write(np.ascontiguousarray(uv, np.float32).tobytes())


def run_ref_filter(rgba, sigma: float = 1.0, wrap: bool = False, spread: int = 1000, stages: int = 15,
                   mesh=None) -> np.ndarray:
    """The reference's lightmap filters (RRBuffer::lightmapSmooth, ...Grow...,
    lightmapFillBackground) on one (h, w, 4) lightmap; mesh = (v, normals, t,
    uv) gives lightmapSmooth an object, so it also smooths unwrap seams."""
    exe = os.path.join(REF_DIR, "ref_filter")
    with tempfile.TemporaryDirectory() as d:
        ip, op, mp = os.path.join(d, "i"), os.path.join(d, "o"), os.path.join(d, "m")
        write_lightmap(ip, rgba)
        args = [exe, ip, op, repr(float(sigma)), str(int(wrap)), str(spread), str(stages)]
        if mesh is not None:
            write_unwrap(mp, *mesh)
            args.append(mp)
        subprocess.run(args, capture_output=True, text=True, check=True)
        return read_lightmap(op)


def run_ref_enumerate(v, normals, t, uv, size: int):
    """The reference's texel enumeration (enumerateTexelsPartial) of one
    unwrapped mesh into a size x size map: returns (flags (size*size,) uint8,
    offsets (size*size+1,) uint64, sub-texels as (tri, uv (3,2), area))."""
    exe = os.path.join(REF_DIR, "ref_enumerate")
    with tempfile.TemporaryDirectory() as d:
        mp, op = os.path.join(d, "m"), os.path.join(d, "o")
        write_unwrap(mp, v, normals, t, uv)
        subprocess.run([exe, mp, str(size), op], capture_output=True, text=True, check=True)
        b = open(op, "rb").read()
    assert b[:4] == b"RGE1"
    sz, total = (int(x) for x in np.frombuffer(b, np.uint32, 2, 4))
    S = sz * sz
    flags = np.frombuffer(b, np.uint8, S, 12).copy()
    counts = np.frombuffer(b, np.uint32, S, 12 + S).astype(np.uint64)
    off = np.zeros(S + 1, np.uint64)
    np.cumsum(counts, out=off[1:])
    rec = np.dtype([("tri", "<u4"), ("uv", "<f4", (3, 2)), ("area", "<f4")])
    st = np.frombuffer(b, rec, total, 12 + 5 * S).copy()
    return flags, off, st


# SCENE  "RGS1": u32 nv, nt, natlas, size, quality, nout, seed; f32 xyz[3nv];
#                u32 idx[3nt]; f32 uv[6nt]; f32 albedo[3nt]; i32 atlas[nt];
#                f32 lights[12]; u32 out_atlas[nout]
# GATHER "RGG1": u32 nout, u32 size, f32 rgba[nout*size*size*4]
def write_gather_scene(path: str, gs, atlases, quality: int, seed: int) -> None:
    """The "RGS1" scene file of a GatherScene (format above)."""
    sc = gs.scene
    atlases = np.asarray(atlases, np.uint32)
    L = gs.lights
    lights = np.concatenate([L["dir_direction"], L["dir_color"], L["point_position"], L["point_color"]]).astype(np.float32)
    with open(path, "wb") as f:
        f.write(b"RGS1")
        f.write(np.array([sc.vertices.shape[0], sc.ntri, gs.natlas, gs.size, quality, atlases.shape[0], seed],
                         np.uint32).tobytes())
        f.write(np.ascontiguousarray(sc.vertices, np.float32).tobytes())
        f.write(np.ascontiguousarray(sc.indices, np.uint32).tobytes())
        f.write(np.ascontiguousarray(gs.uv, np.float32).tobytes())
        f.write(np.ascontiguousarray(gs.albedo, np.float32).tobytes())
        f.write(np.ascontiguousarray(gs.tri_atlas, np.int32).tobytes())
        f.write(lights.tobytes())
        f.write(atlases.tobytes())


def run_ref_gather(gs, atlases, quality: int, seed: int = 1, threads: int = 0, bake: bool = False) -> np.ndarray:
    """The reference's own processTexel over whole atlases of a GatherScene,
    with no radiosity solver (the plain N-bounce estimator, stopAtDepth 20),
    or with bake=True its whole default updateLightmaps (first gather,
    radiosity, final gather reading the solver; no smoothing or spreading).
    Returns (len(atlases), size, size, 4) float32 RGBA, alpha = flags / 255;
    with bake also the solver the final gather read, per triangle: dict of
    direct (T,3), indirect (T,3) and smoothed corner indirect (T,3,3)."""
    exe = os.path.join(REF_DIR, "ref_gather")
    atlases = np.asarray(atlases, np.uint32)
    with tempfile.TemporaryDirectory() as d:
        sp, op = os.path.join(d, "s"), os.path.join(d, "o")
        write_gather_scene(sp, gs, atlases, quality, seed)
        subprocess.run([exe, sp, op, str(threads)] + (["bake"] if bake else []), capture_output=True, text=True,
                       check=True)
        b = open(op, "rb").read()
        sb = open(op + ".solver", "rb").read() if bake else None
    assert b[:4] == b"RGG1"
    nout, size = (int(x) for x in np.frombuffer(b, np.uint32, 2, 4))
    out = np.frombuffer(b, np.float32, nout * size * size * 4, 12).reshape(nout, size, size, 4).copy()
    if not bake:
        return out
    assert sb[:4] == b"RGB1"
    nt = int(np.frombuffer(sb, np.uint32, 1, 4)[0])
    rec = np.frombuffer(sb, np.float32, nt * 15, 8).reshape(nt, 15)
    solver = {"direct": rec[:, 0:3].copy(), "indirect": rec[:, 3:6].copy(), "corner": rec[:, 6:15].reshape(nt, 3, 3).copy()}
    return out, solver


# ---------------------------------------------------------------------------
# The reference collider in-process (oracle/_ref/libref_bench.so, built from
# oracle/ref_bench.cpp): the benchmark's reference arm and CPU baseline.
IT_LINEAR, IT_BSP_COMPACT, IT_BSP_FAST, IT_BSP_FASTER, IT_BSP_FASTEST = 0, 1, 2, 3, 4
_bench_lib = None


def ref_bench_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_bench.so"))


def _ref_bench():
    global _bench_lib
    if _bench_lib is None:
        import ctypes as C
        L = C.CDLL(os.path.join(REF_DIR, "libref_bench.so"))
        P = C.c_void_p
        L.refb_create.argtypes = [P, C.c_uint, P, C.c_uint, C.c_int, C.POINTER(C.c_double)]
        L.refb_create.restype = P
        L.refb_technique.argtypes = [P]
        L.refb_technique.restype = C.c_int
        L.refb_memory.argtypes = [P]
        L.refb_memory.restype = C.c_size_t
        L.refb_trace.argtypes = [P, P, C.c_size_t, C.c_uint, C.c_int, P, P, P, P]
        L.refb_trace.restype = C.c_double
        L.refb_destroy.argtypes = [P]
        _bench_lib = L
    return _bench_lib


class RefCollider:
    """RRCollider::create(mesh, nullptr, technique) of the reference library,
    and its intersect() over ray arrays on OpenMP threads."""

    def __init__(self, v, t, technique: int = IT_BSP_FASTEST):
        import ctypes as C
        L = _ref_bench()
        self._v = np.ascontiguousarray(v, np.float32)
        self._t = np.ascontiguousarray(t, np.uint32)
        bs = C.c_double(0)
        self._h = L.refb_create(self._v.ctypes.data, self._v.shape[0], self._t.ctypes.data, self._t.shape[0],
                                technique, C.byref(bs))
        if not self._h:
            raise RuntimeError("RRCollider::create failed")
        self.build_s = bs.value
        self.technique = L.refb_technique(self._h)
        self.memory = L.refb_memory(self._h)

    def trace(self, rays, threads: int = 0, flags: int = FILL_DISTANCE | FILL_TRIANGLE | FILL_POINT2D | FILL_SIDE,
              outputs: bool = True):
        """Returns (seconds of the parallel loop, dict hit/tri/dist/uv or None)."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        L = _ref_bench()
        if outputs:
            out = {"hit": np.zeros(n, np.uint8), "tri": np.zeros(n, np.uint32), "dist": np.zeros(n, np.float32),
                   "uv": np.zeros((n, 2), np.float32)}
            s = L.refb_trace(self._h, rays.ctypes.data, n, flags, threads, out["hit"].ctypes.data,
                             out["tri"].ctypes.data, out["dist"].ctypes.data, out["uv"].ctypes.data)
            out["hit"] = out["hit"].astype(bool)
            return s, out
        s = L.refb_trace(self._h, rays.ctypes.data, n, flags, threads, None, None, None, None)
        return s, None

    def close(self):
        if self._h:
            _ref_bench().refb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
