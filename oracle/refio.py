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
