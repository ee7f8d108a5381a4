"""Shared test utilities: fixtures loading and hit comparison."""
from __future__ import annotations

import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def md5(*arrays) -> str:
    h = hashlib.md5()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def load_golden(name: str) -> dict:
    return dict(np.load(os.path.join(GOLDEN, name)))


def expand(g: dict) -> dict:
    """Compact golden (hit rays only) -> full per-ray arrays."""
    n = int(g["n"])
    out = {"hit": np.zeros(n, bool), "tri": np.full(n, 0xFFFFFFFF, np.uint32), "dist": np.zeros(n, np.float32),
           "uv": np.zeros((n, 2), np.float32), "plane": np.zeros((n, 4), np.float32), "side": np.zeros(n, bool)}
    i = g["hit_idx"]
    out["hit"][i] = True
    out["tri"][i] = g["tri"]
    out["dist"][i] = g["dist"]
    out["uv"][i] = g["uv"]
    out["plane"][i] = g["plane"]
    out["side"][i] = g["side"].astype(bool)
    return out


def exact_hit64(v, t, ray, tri):
    """Double-precision Moller-Trumbore of one ray against one triangle:
    (hit, distance)."""
    a, b, c = (v[t[tri, k]].astype(np.float64) for k in range(3))
    o = ray[0:3].astype(np.float64)
    d = ray[4:7].astype(np.float64)
    e1, e2 = b - a, c - a
    p = np.cross(d, e2)
    det = e1 @ p
    if det == 0:
        return False, np.inf
    tv = o - a
    u = (tv @ p) / det
    q = np.cross(tv, e1)
    w = (d @ q) / det
    dist = (e2 @ q) / det
    ok = 0 <= u <= 1 and 0 <= w and u + w <= 1
    return ok, dist


def classify_mismatches(v, t, rays, ref: dict, got: dict, tie_rel: float = 1e-6):
    """Hit-set and hitTriangle differences between a reference result and
    ours, each classified:
      tie      : both hit, distances equal within tie_rel (relative)
      ref_off  : the reference's (triangle, distance) is not an intersection
                 in double precision within 1e-4 relative, or a closer exact
                 intersection exists at our triangle
      other    : anything else (must be empty)"""
    n = len(ref["hit"])
    res = {"hit_mismatch": [], "tie": [], "ref_off": [], "other": []}
    for i in np.nonzero(ref["hit"] != got["hit"])[0]:
        res["hit_mismatch"].append(int(i))
        if ref["hit"][i]:
            ok, d = exact_hit64(v, t, rays[i], ref["tri"][i])
            lo, hi = rays[i, 3], rays[i, 7]
            in_range = ok and lo * (1 - 1e-6) - 1e-7 <= d <= hi * (1 + 1e-6) + 1e-7
            if not in_range:
                res["ref_off"].append(int(i))
            elif abs(d - lo) <= 1e-5 * max(1.0, abs(lo)) or abs(d - hi) <= 1e-5 * max(1.0, abs(hi)):
                res["tie"].append(int(i))      # at the range boundary
            else:
                res["other"].append(int(i))
        else:
            ok, d = exact_hit64(v, t, rays[i], got["tri"][i])
            lo, hi = rays[i, 3], rays[i, 7]
            if abs(d - lo) <= 1e-5 * max(1.0, abs(lo)) or abs(d - hi) <= 1e-5 * max(1.0, abs(hi)):
                res["tie"].append(int(i))
            else:
                res["other"].append(int(i))
    both = ref["hit"] & got["hit"]
    for i in np.nonzero(both & (ref["tri"] != got["tri"]))[0]:
        dr, dg = float(ref["dist"][i]), float(got["dist"][i])
        if abs(dr - dg) <= tie_rel * max(abs(dr), abs(dg)):
            res["tie"].append(int(i))
            continue
        okr, d_ref = exact_hit64(v, t, rays[i], ref["tri"][i])
        okg, d_got = exact_hit64(v, t, rays[i], got["tri"][i])
        if (not okr) or abs(d_ref - dr) > 1e-4 * abs(d_ref) or (okg and d_got < d_ref):
            res["ref_off"].append(int(i))
        else:
            res["other"].append(int(i))
    return res
