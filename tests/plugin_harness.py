"""Compiles and runs tests/cpp/plugin_check.cpp: the reference-side plugin
(include/rrgpu_rrcollider_plugin.hpp) built against the reference's headers
(as staged in oracle/_ref/src) and library (oracle/_ref), linked with
librrgpu.so; reads what its handler mode writes."""
from __future__ import annotations

import json
import os
import struct
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_INCLUDE = os.path.join(ROOT, "oracle", "_ref", "src", "include")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libLightsprintCore.a")

# pass-2 record of plugin_check's handler mode (packed)
PASS2 = np.dtype([("result", "u1"), ("tri", "<u4"), ("dist", "<f4"), ("u", "<f4"), ("v", "<f4"),
                  ("plane", "<f4", (4,)), ("point3d", "<f4", (3,)), ("side", "u1"), ("offers", "<u4")])


def available() -> bool:
    return os.path.isdir(os.path.join(REF_INCLUDE, "Lightsprint")) and os.path.exists(REF_LIB)


def build(tmp_path) -> str:
    from lightsprintsdk_gb300 import build as B
    lib = B.build()
    exe = os.path.join(str(tmp_path), "plugin_check")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-fsigned-char", "-ffp-contract=off", "-DRR_BUILD", "-w", "-include", "string",
           "-include", "climits", f"-I{REF_INCLUDE}", f"-I{os.path.join(ROOT, 'include')}",
           os.path.join(ROOT, "tests", "cpp", "plugin_check.cpp"), "-o", exe, REF_LIB, lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-lgomp", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def hello(exe: str) -> str:
    return subprocess.run([exe], capture_output=True, text=True, timeout=300, check=True).stdout


def read_log(path: str, n: int):
    """(list of per-ray offered sequences as (tri u32[], dist f32[]), pass-2
    records)."""
    b = open(path, "rb").read()
    off = 0
    seqs = []
    for _ in range(n):
        c = struct.unpack_from("<I", b, off)[0]
        off += 4
        a = np.frombuffer(b, np.dtype([("tri", "<u4"), ("dist", "<f4")]), c, off)
        off += 8 * c
        seqs.append((a["tri"].copy(), a["dist"].copy()))
    rec = np.frombuffer(b, PASS2, n, off).copy()
    return seqs, rec


def run_handler(exe: str, tmp_path, v, t, rays, accept_at: int):
    """Casts every ray through the GPU technique and IT_BSP_FASTEST with the
    logging handlers; returns (info, gpu (seqs, rec), ref (seqs, rec))."""
    from oracle import refio
    d = str(tmp_path)
    mp, rp, op = os.path.join(d, "mesh"), os.path.join(d, "rays"), os.path.join(d, "log")
    refio.write_mesh(mp, v, t)
    refio.write_rays(rp, rays)
    out = subprocess.run([exe, "handler", mp, rp, op, str(accept_at)], capture_output=True, text=True, timeout=900,
                         check=True).stdout
    info = json.loads(out.strip().splitlines()[-1])
    n = len(rays)
    return info, read_log(op + ".gpu", n), read_log(op + ".ref", n)


def compare_sequences(gpu_seqs, ref_seqs, tie_rel: float = 1e-6):
    """Per ray: 'same' (identical offered triangles in identical order),
    'tie_order' (the same triangles, differing only in the order of hits whose
    distances agree within tie_rel relative), 'ref_repeat' (the reference
    offers a triangle more than once, ours once each, otherwise the same
    set), or 'differ'.  Returns (counts, indices of 'differ')."""
    counts = {"same": 0, "tie_order": 0, "ref_repeat": 0, "differ": 0}
    bad = []
    for i, ((gt, gd), (rt, rd)) in enumerate(zip(gpu_seqs, ref_seqs)):
        if len(gt) == len(rt) and np.array_equal(gt, rt):
            counts["same"] += 1
            continue
        if len(gt) == len(rt) and sorted(gt.tolist()) == sorted(rt.tolist()):
            ok = True
            for k in range(len(gt)):
                if gt[k] != rt[k]:
                    a, b = float(gd[k]), float(rd[k])
                    if abs(a - b) > tie_rel * max(abs(a), abs(b), 1e-30):
                        ok = False
                        break
            if ok:
                counts["tie_order"] += 1
                continue
        if len(set(rt.tolist())) < len(rt):
            _, first = np.unique(rt, return_index=True)
            if np.array_equal(rt[np.sort(first)], gt):
                counts["ref_repeat"] += 1
                continue
        counts["differ"] += 1
        bad.append(i)
    return counts, bad


MULTI = np.dtype([("hit", "u1"), ("obj", "<i4"), ("tri", "<u4"), ("dist", "<f4"), ("u", "<f4"), ("v", "<f4"),
                  ("side", "u1")])
MULTI_HANDLER = np.dtype([("result", "u1"), ("obj", "<i4"), ("tri", "<u4"), ("offers", "<u4")])


def run_multi(exe: str, tmp_path, meshes, objects, rays):
    """meshes: list of (v, t); objects: list of (mesh index, enabled,
    3x4 world matrix).  Runs plugin_check's multi mode; returns (info,
    (gpu records, gpu handler records), (ref records, ref handler records))."""
    d = str(tmp_path)
    sp, rp, op = os.path.join(d, "scene"), os.path.join(d, "rays"), os.path.join(d, "mlog")
    with open(sp, "wb") as f:
        f.write(b"RGO1")
        f.write(np.array([len(meshes)], np.uint32).tobytes())
        for v, t in meshes:
            v = np.ascontiguousarray(v, np.float32)
            t = np.ascontiguousarray(t, np.uint32)
            f.write(np.array([v.shape[0], t.shape[0]], np.uint32).tobytes())
            f.write(v.tobytes())
            f.write(t.tobytes())
        f.write(np.array([len(objects)], np.uint32).tobytes())
        for m, en, w in objects:
            f.write(np.array([m, 1 if en else 0], np.uint32).tobytes())
            f.write(np.ascontiguousarray(w, np.float32).reshape(12).tobytes())
    from oracle import refio
    refio.write_rays(rp, rays)
    out = subprocess.run([exe, "multi", sp, rp, op], capture_output=True, text=True, timeout=900,
                         check=True).stdout
    info = json.loads(out.strip().splitlines()[-1])
    n = len(rays)
    res = []
    for side in ("gpu", "ref"):
        b = open(op + "." + side, "rb").read()
        a = np.frombuffer(b, MULTI, n, 0).copy()
        h = np.frombuffer(b, MULTI_HANDLER, n, MULTI.itemsize * n).copy()
        res.append((a, h))
    return info, res[0], res[1]


def run_lightmaps(exe: str, tmp_path, gs, atlases, quality: int, mode: str, seed: int):
    """plugin_check's lightmaps mode (rrgpu_plugin::updateLightmaps on a
    reference RRSolver): returns (info, (len(atlases), size, size, 4) RGBA)."""
    from oracle import refio
    d = str(tmp_path)
    sp, op = os.path.join(d, "lscene"), os.path.join(d, "lout")
    refio.write_gather_scene(sp, gs, atlases, quality, seed)
    out = subprocess.run([exe, "lightmaps", sp, op, mode, str(seed)], capture_output=True, text=True, timeout=900,
                         check=True).stdout
    info = json.loads(out.strip().splitlines()[-1])
    b = open(op, "rb").read()
    assert b[:4] == b"RGG1"
    nout, size = (int(x) for x in np.frombuffer(b, np.uint32, 2, 4))
    return info, np.frombuffer(b, np.float32, nout * size * size * 4, 12).reshape(nout, size, size, 4).copy()
