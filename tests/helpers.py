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


# Bounds of the statistical comparison with the reference's own gather
# (tests/golden/gather_ref.npz).  Under a correct estimator the largest |z|
# of an atlas-channel mean is about 2, the spread ratio about 1 (0.9-1.1
# over seeds) and the largest 8x8-block |z| about 3.5 (768 blocks); a gather
# cut at 3 bounces instead of 20 reaches |z| > 11.
GATHER_Z_MEAN = 4.5
GATHER_Z_BLOCK = 5.5
GATHER_SPREAD = 1.25
GATHER_REL_MEAN = 0.01


def _trimmed_mean(sq: np.ndarray, keep: float = 0.99) -> float:
    """Mean of the smallest `keep` fraction: path-traced texels have heavy
    tails (rare paths that reach the point light), which make plain mean
    squares swing from seed to seed."""
    v = np.sort(sq.ravel())
    return float(v[:max(1, int(v.shape[0] * keep))].mean())


def reference_gather_stats(g: dict, o1: np.ndarray, o2: np.ndarray) -> list[dict]:
    """Compares two independent runs (o1, o2: (natlas, size, size, 4)) of a
    gather with the two independent runs of the reference's own gather of the
    same atlases in the gather_ref fixture g, over the covered texels of each
    atlas.  With d = mean of the reference runs - mean of ours, per texel:
      z_mean    largest |mean of d| / its standard error, over RGB
      rel_mean  largest |mean of d| / the reference's mean, over RGB
      z_block   largest |z| of the mean of d over 8x8 texel blocks
      spread    (trimmed) mean square of reference run 1 - our run 1 over
                what the two sides' own noise predicts for it: half the mean
                square between the reference's runs plus half of that
                between ours.  A texel-level bias raises it; each side's
                noise is measured, not assumed equal
      alpha     our alpha equals the reference's TexelFlags / 255
      det_n, det_rel
                texels whose two reference runs agree bit for bit although
                their random numbers differ (every sample sees the same light:
                sub-texels that are wholly lit or shadowed, unoccluded
                hemispheres) and the largest relative difference of our run
                there: the sub-texel stepping, light rounds, light falloff and
                cosine then decide the value alone, so ours must match it to
                float rounding."""
    r1, r2, flags = g["rgb"].astype(np.float64), g["rgb2"].astype(np.float64), g["flags"]
    size = flags.shape[1]
    out = []
    for k in range(flags.shape[0]):
        cov = flags[k] > 0
        a, b = r1[k][cov], r2[k][cov]
        x = o1[k][cov][:, :3].astype(np.float64)
        y = o2[k][cov][:, :3].astype(np.float64)
        d = 0.5 * (a + b) - 0.5 * (x + y)
        z = d.mean(0) / (d.std(0) / np.sqrt(d.shape[0]))
        spread = _trimmed_mean((a - x) ** 2) / (0.5 * _trimmed_mean((a - b) ** 2) + 0.5 * _trimmed_mean((x - y) ** 2))
        dd = np.zeros((size, size, 3))
        dd[cov] = d
        nb = size // 8
        cb = cov.reshape(nb, 8, nb, 8).transpose(0, 2, 1, 3).reshape(nb * nb, 64)
        db = dd.reshape(nb, 8, nb, 8, 3).transpose(0, 2, 1, 3, 4).reshape(nb * nb, 64, 3)
        zb = 0.0
        for blk in range(nb * nb):
            m = cb[blk]
            if m.sum() < 16:
                continue
            v = db[blk][m]
            sd = v.std(0)
            for c in range(3):
                if sd[c] < 1e-6:   # every texel equal (unlit on both sides): the difference itself must vanish
                    zb = max(zb, 0.0 if abs(v[:, c].mean()) < 1e-5 else np.inf)
                else:
                    zb = max(zb, abs(v[:, c].mean()) / (sd[c] / np.sqrt(m.sum())))
        alpha = np.array_equal(o1[k][..., 3], flags[k].astype(np.float32) / np.float32(255))
        det = np.all(a == b, axis=1) & np.all(x == y, axis=1)
        det_rel = float((np.abs(a[det] - x[det]) / np.maximum(np.abs(a[det]), 1e-30)).max()) if det.any() else 0.0
        out.append({"z_mean": float(np.abs(z).max()), "rel_mean": float(np.abs(d.mean(0) / (0.5 * (a + b)).mean(0)).max()),
                    "spread": float(spread), "z_block": float(zb), "alpha": alpha, "det_n": int(det.sum()),
                    "det_rel": det_rel})
    return out


def reference_gather_ok(s: dict, det_rel: float = 0.0) -> bool:
    return (s["alpha"] and s["z_mean"] < GATHER_Z_MEAN and s["rel_mean"] < GATHER_REL_MEAN
            and s["spread"] < GATHER_SPREAD and s["z_block"] < GATHER_Z_BLOCK and s["det_rel"] <= det_rel)


# The reference's default bake (tests/golden/bake_ref.npz) against ours.
# Its radiosity solver stops at an accuracy target where ours iterates the
# same balance to convergence, and its photon shooting spreads the noise
# differently, so means are compared within both sides' measured scatter
# plus an allowance: 0.5 % for atlas means, 1 % for class indirect.
BAKE_Z = 4.0
BAKE_ATLAS_ALLOW = 0.005
BAKE_CLASS_ALLOW = 0.01


def room_classes(gs):
    """Triangle masks of the small room's object classes: slabs, boxes, spheres."""
    obj = gs.scene.tri_object
    return [(obj >= 0) & (obj < 9), (obj >= 9) & (obj < 19), obj >= 19]


def triangle_areas(gs):
    v = gs.scene.vertices.astype(np.float64)
    t = gs.scene.indices
    return 0.5 * np.linalg.norm(np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]]), axis=1)


def _within(ours: np.ndarray, ref: np.ndarray, allow: float) -> np.ndarray:
    """ours (n, ...) and ref (m, ...) realizations: |mean difference| over
    BAKE_Z x the combined scatter of the means plus allow x the reference
    mean; values below 1 pass."""
    mo, mr = ours.mean(0), ref.mean(0)
    so = ours.std(0, ddof=1) / np.sqrt(ours.shape[0])
    sr = ref.std(0, ddof=1) / np.sqrt(ref.shape[0])
    return np.abs(mo - mr) / (BAKE_Z * np.sqrt(so ** 2 + sr ** 2) + allow * np.abs(mr))


def reference_bake_stats(g: dict, gs, runs: list, directs: list, indirects: list) -> dict:
    """runs: our gathered atlases per run ((natlas, size, size, 4) each),
    directs / indirects: our solver's per-triangle direct and indirect
    irradiance per run.  Returns
      atlas     per atlas and channel, the mean difference over the bound
                (below 1 passes)
      cls       the same for the area-weighted indirect of each object class
      direct_z  largest |z| of the mean per-triangle direct difference per
                class (the first gather is the same estimator on both sides)
      det_n, det_rel
                texels equal in every reference run and in every run of
                ours, and the largest relative difference of ours there
      alpha     our alpha equals the reference's TexelFlags / 255."""
    flags = g["flags"]
    cov = flags > 0
    area = triangle_areas(gs)
    classes = room_classes(gs)
    ours_means = np.stack([[r[a][cov[a]][:, :3].astype(np.float64).mean(0) for a in range(flags.shape[0])]
                           for r in runs])
    ours_cls = np.stack([[(ind[m] * area[m, None]).sum(0) / area[m].sum() for m in classes] for ind in indirects])
    dz = 0.0
    for m in classes:
        for d in directs:
            for k in range(g["direct"].shape[0]):
                diff = (g["direct"][k][m] - d[m]).astype(np.float64)
                sd = diff.std(0)
                ok = sd > 0
                if ok.any():
                    dz = max(dz, float(np.abs(diff.mean(0)[ok] / (sd[ok] / np.sqrt(diff.shape[0]))).max()))
    # texels equal in every reference run and in every run of ours (as the
    # plain gather's check: on faces pressed flat against another face a
    # grazing ray may meet the coplanar face, which varies between runs)
    det_ref = g["det_mask"]
    ours_same = np.ones_like(det_ref)
    for r in runs[1:]:
        ours_same &= np.all(r[..., :3] == runs[0][..., :3], axis=-1)
    keep = ours_same[det_ref]
    det = det_ref & ours_same
    ours_det = runs[0][..., :3][det].astype(np.float64)
    ref_det = g["det_rgb"].astype(np.float64)[keep]
    det_rel = float((np.abs(ours_det - ref_det) / np.maximum(np.abs(ref_det), 1e-30)).max()) if det.any() else 0.0
    alpha = all(np.array_equal(r[..., 3], flags.astype(np.float32) / np.float32(255)) for r in runs)
    return {"atlas": _within(ours_means, g["atlas_means"].astype(np.float64), BAKE_ATLAS_ALLOW),
            "cls": _within(ours_cls, g["class_indirect"].astype(np.float64), BAKE_CLASS_ALLOW),
            "direct_z": dz, "det_n": int(det.sum()), "det_rel": det_rel, "alpha": alpha}


def reference_bake_ok(s: dict, det_rel: float = 0.0) -> bool:
    return (s["alpha"] and float(s["atlas"].max()) < 1 and float(s["cls"].max()) < 1 and s["direct_z"] < GATHER_Z_MEAN
            and s["det_rel"] <= det_rel)
