"""Generates the golden fixtures under tests/golden/ by running the reference
collider, built from the reference's own sources into oracle/_ref (see
oracle/ref.mk), on the seeded workloads of lightsprintsdk_gb300.scenes.

    make -f oracle/ref.mk -j8 && python tests/golden/make_golden.py

Each fixture stores md5 hashes of its generated inputs, so the tests also
check that the generators reproduce the same bytes on the machine they run on,
and the reference outputs of the rays that hit (ray index, hitTriangle,
hitDistance, hitPoint2d, hitPlane, hitFrontSide).  The lightmap fixture
holds the reference's texel enumeration (TexelFlags, sub-texel counts and a
hash of the sub-texels) and hashes of its post-filter outputs.  The gather
fixture holds the reference's own per-texel gather (processTexel, no
radiosity solver) of four atlases of a small room, the bake fixture summaries
of its default bake (updateLightmaps with the radiosity solver) of the same
atlases.  Test infrastructure only.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lightsprintsdk_gb300 import scenes  # noqa: E402
from oracle import refio  # noqa: E402


def md5(*arrays) -> str:
    h = hashlib.md5()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def compact(h: dict) -> dict:
    idx = np.nonzero(h["hit"])[0].astype(np.uint32)
    return {"hit_idx": idx, "tri": h["tri"][idx], "dist": h["dist"][idx], "uv": h["uv"][idx],
            "plane": h["plane"][idx], "side": h["side"][idx].astype(np.uint8), "n": np.uint32(h["hit"].shape[0])}


def save(name: str, **kw):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **kw)
    print(f"{name}: {os.path.getsize(path)} bytes")


def hello_mesh():
    """The two-triangle mesh and ray of samples/HelloCollider/HelloCollider.cpp:15-42."""
    v = np.array([[-1, 0, 0], [1, 0, 0], [0, 1, 0], [1, 0, 0], [-1, 0, 0], [0, 0, 1]], np.float32)
    t = np.arange(6, dtype=np.uint32).reshape(2, 3)
    rays = np.array([[0, -1, 0.3, 0, 0, 1, 0, 1000]], np.float32)
    return v, t, rays


def edge_mesh():
    """Small mesh with the cases the reference handles specially: degenerate
    triangles (zero area, repeated vertex; RRMesh.cpp:48-52 and
    IntersectBspFast.cpp:182-186), two coincident triangles (a distance tie),
    an axis-aligned quad, and a sliver."""
    v = np.array([
        [0, 0, 0], [1, 0, 0], [0, 1, 0],          # 0 tri in z=0
        [1, 1, 0],                                 # 3
        [0, 0, 1], [1, 0, 1], [0, 1, 1],          # 4..6 tri in z=1
        [2, 0, 0], [3, 0, 0], [4, 0, 0],          # 7..9 collinear
        [0, 0, 2], [2, 0, 2], [0, 2, 2], [2, 2, 2],  # 10..13 quad z=2
        [0.5, 0.5, 3], [0.5 + 1e-7, 0.5, 3], [0.5, 2.5, 3],  # 14..16 sliver
    ], np.float32)
    t = np.array([
        [0, 1, 2],      # 0
        [1, 3, 2],      # 1
        [4, 5, 6],      # 2
        [6, 5, 4],      # 3 coincident with 2, opposite winding: distance tie
        [7, 8, 9],      # 4 degenerate (collinear)
        [0, 0, 1],      # 5 degenerate (repeated vertex)
        [10, 11, 12],   # 6
        [11, 13, 12],   # 7
        [14, 15, 16],   # 8 sliver
    ], np.uint32)
    rng_rays = []
    # axis-aligned rays through interiors, edges and vertices
    for x, y in [(0.25, 0.25), (0.5, 0.5), (0.0, 0.0), (1.0, 0.0), (0.75, 0.75), (1.5, 1.5), (0.3, 0.6),
                 (0.5, 0.0), (0.0, 0.5), (1.0, 1.0), (2.0, 0.0)]:
        rng_rays.append([x, y, -5, 0, 0, 0, 1, 100])
        rng_rays.append([x, y, 10, 0, 0, 0, -1, 100])
    # rayLengthMin / Max clipping
    rng_rays.append([0.25, 0.25, -5, 5.5, 0, 0, 1, 100])      # starts past z=0 -> first hit z=1
    rng_rays.append([0.25, 0.25, -5, 0, 0, 0, 1, 5.5])        # ends before z=1
    rng_rays.append([0.25, 0.25, -5, 6.0, 0, 0, 1, 6.0])      # exactly at z=1 (t=6)
    rng_rays.append([0.25, 0.25, -5, 5.0, 0, 0, 1, 5.0])      # exactly at z=0 (t=5)
    # oblique rays
    d = np.array([0.3, 0.2, 1.0]); d /= np.linalg.norm(d)
    rng_rays.append([0.1, 0.1, -3, 0, *d, 100])
    d2 = np.array([1.0, 1.0, 0.0]); d2 /= np.linalg.norm(d2)
    rng_rays.append([-1, -1, 0.0, 0, *d2, 100])              # in the plane z=0
    rng_rays.append([0.6, 1.0, -1, 0, 0, 0, 1, 100])          # sliver region
    return v, t, np.array(rng_rays, np.float32)


# lightmap cases: (geodesic frequency, atlas size)
LIGHTMAP_CASES = ((4, 48), (3, 17))
# filter runs on the first case: (stages, wrap, seams); stages as RRG_FILTER_*
FILTER_RUNS = ((1, 0, 0), (1, 1, 0), (1, 0, 1), (2, 0, 0), (2, 1, 0), (4, 0, 0), (4, 1, 0), (8, 0, 0),
               (15, 0, 0), (15, 0, 1), (15, 1, 1))
# and on the second (17 x 17: growing with wrap indexes modulo 289 texels in
# unsigned arithmetic, which is not a wrap-around at the map's edges)
FILTER_RUNS_ODD = ((4, 1, 0), (15, 1, 1), (15, 0, 1))


def lightmap_case(freq: int, size: int):
    """A geodesic sphere (one vertex per position, unit normals = positions)
    with the uniform-grid unwrap into one size x size atlas."""
    v, t = scenes.geodesic_sphere_grid(freq)
    v = np.asarray(v, np.float32)
    t = np.asarray(t, np.uint32)
    nrm = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    uv = scenes.grid_unwrap(np.zeros(len(t), np.int32), 1)
    return v, nrm, t, uv


def lightmap_image(flags: np.ndarray, size: int, seed: int = 7) -> np.ndarray:
    """A lightmap as the gather leaves it: covered texels (flags != 0) random
    RGB in [0.1, 2) with alpha = flags/255, the rest 0."""
    rng = np.random.default_rng(seed)
    img = np.zeros((size * size, 4), np.float32)
    cov = flags > 0
    img[cov, :3] = rng.uniform(0.1, 2.0, (int(cov.sum()), 3)).astype(np.float32)
    img[:, 3] = flags.astype(np.float32) / np.float32(255)
    return img.reshape(size, size, 4)


def lightmaps():
    """Reference texel enumeration (flags, sub-texels) and post-filters."""
    kw = {}
    for k, (freq, size) in enumerate(LIGHTMAP_CASES):
        v, nrm, t, uv = lightmap_case(freq, size)
        flags, off, st = refio.run_ref_enumerate(v, nrm, t, uv, size)
        kw[f"case{k}_mesh_md5"] = md5(v, nrm, t, uv)
        kw[f"case{k}_flags"] = flags
        kw[f"case{k}_counts"] = np.diff(off).astype(np.uint32)
        kw[f"case{k}_st_md5"] = md5(st["tri"], st["uv"], st["area"])
        img = lightmap_image(flags, size)
        kw[f"case{k}_img_md5"] = md5(img)
        for stages, wrap, seams in (FILTER_RUNS if k == 0 else FILTER_RUNS_ODD):
            out = refio.run_ref_filter(img, 1.0, bool(wrap), 1000, stages, mesh=(v, nrm, t, uv) if seams else None)
            kw[f"case{k}_filter_{stages}_{wrap}_{seams}_md5"] = md5(out)
            if k == 0 and (stages, wrap, seams) == (15, 0, 1):
                kw["filter_all_seams"] = out
    save("lightmap_ref.npz", **kw)


# Reference gather: atlases of the small room scene (scenes.gather_room) at
# the highest quality the GPU gather takes in one call.  The texel's sub-texel
# stepping depends on the quality, so the tests run at the same one.
GATHER_ATLASES = (0, 5, 9, 13)   # floor slab, wall slab, a sphere, boxes
GATHER_QUALITY = 256
GATHER_SEEDS = (1, 2)   # two independent runs: their spread is the reference's own noise


def gather():
    """The reference's own processTexel (no radiosity solver: the plain
    N-bounce estimator, stopAtDepth 20) over whole atlases of the room, twice
    with different srand() seeds."""
    gs = scenes.gather_room()
    outs = [refio.run_ref_gather(gs, GATHER_ATLASES, GATHER_QUALITY, seed) for seed in GATHER_SEEDS]
    flags = np.rint(outs[0][..., 3] * 255).astype(np.uint8)
    for out in outs:
        assert np.array_equal(flags.astype(np.float32) / np.float32(255), out[..., 3])
    save("gather_ref.npz", scene_md5=md5(gs.scene.vertices, gs.scene.indices, gs.albedo, gs.uv, gs.tri_atlas),
         atlases=np.array(GATHER_ATLASES, np.uint32), quality=np.uint32(GATHER_QUALITY), flags=flags,
         rgb=np.ascontiguousarray(outs[0][..., :3]), rgb2=np.ascontiguousarray(outs[1][..., :3]))


# Reference bake: updateLightmaps with its radiosity solver on the same
# atlases.  Its photon shooting seeds each thread's generator with the thread
# number, so runs on different thread counts are its independent realizations.
BAKE_THREADS = (1, 2, 3, 5)


def room_classes(gs):
    """Triangle masks of the room's object classes: slabs, boxes, spheres."""
    obj = gs.scene.tri_object
    return [(obj >= 0) & (obj < 9), (obj >= 9) & (obj < 19), obj >= 19]


def triangle_areas(gs):
    v = gs.scene.vertices.astype(np.float64)
    t = gs.scene.indices
    return 0.5 * np.linalg.norm(np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]]), axis=1)


def bake():
    """The reference's default bake (first gather, radiosity, final gather
    reading the solver; no smoothing or spreading) of four atlases of the
    room, one run per thread count: per run the atlas means over covered
    texels, the area-weighted indirect irradiance of each object class and
    (first two runs) every triangle's direct irradiance; the texels equal in
    every run, with their values."""
    gs = scenes.gather_room()
    area = triangle_areas(gs)
    classes = room_classes(gs)
    outs, solvers = [], []
    for k, th in enumerate(BAKE_THREADS):
        out, sol = refio.run_ref_gather(gs, GATHER_ATLASES, GATHER_QUALITY, seed=10 + k, threads=th, bake=True)
        outs.append(out)
        solvers.append(sol)
    flags = np.rint(outs[0][..., 3] * 255).astype(np.uint8)
    cov = flags > 0
    atlas_means = np.stack([[o[a][cov[a]][:, :3].mean(0) for a in range(len(GATHER_ATLASES))] for o in outs])
    class_indirect = np.stack([[(s["indirect"][m] * area[m, None]).sum(0) / area[m].sum() for m in classes]
                               for s in solvers])
    same = cov.copy()
    for o in outs[1:]:
        same &= np.all(o[..., :3] == outs[0][..., :3], axis=-1)
    save("bake_ref.npz", scene_md5=md5(gs.scene.vertices, gs.scene.indices, gs.albedo, gs.uv, gs.tri_atlas),
         atlases=np.array(GATHER_ATLASES, np.uint32), quality=np.uint32(GATHER_QUALITY), flags=flags,
         atlas_means=atlas_means.astype(np.float32), class_indirect=class_indirect.astype(np.float32),
         direct=np.stack([solvers[0]["direct"], solvers[1]["direct"]]).astype(np.float32),
         det_mask=same, det_rgb=outs[0][..., :3][same].astype(np.float32))


def main():
    assert refio.ref_available(), "build oracle/_ref first: make -f oracle/ref.mk -j8"
    # 1. HelloCollider known answer
    v, t, r = hello_mesh()
    out = {}
    for tech in ("linear", "bsp_fastest"):
        _, h = refio.run_ref_collide(v, t, r, tech, 1)
        out[tech] = h
    save("hello_kat.npz", v=v, t=t, rays=r,
         **{f"{k}_{f}": out[k][f] for k in out for f in ("hit", "tri", "dist", "uv", "plane", "point3d", "side")})

    # 2. edge cases
    v, t, r = edge_mesh()
    kw = {"v": v, "t": t, "rays": r}
    for tech in ("linear", "bsp_fastest"):
        _, h = refio.run_ref_collide(v, t, r, tech, 1)
        for f in ("hit", "tri", "dist", "uv", "plane", "point3d", "side"):
            kw[f"{tech}_{f}"] = h[f]
    save("edge_cases.npz", **kw)

    # 3. config 0: displaced icosphere, 2^18 shell rays, IT_BSP_FASTEST
    v, t = scenes.icosphere_c0()
    n0 = 1 << 18
    r = scenes.shell_rays(n0)
    tm, h = refio.run_ref_collide(v, t, r, "bsp_fastest", 0)
    print("c0 fastest", tm)
    save("c0_fastest.npz", mesh_md5=md5(v, t), rays_md5=md5(r), **compact(h))
    # IT_LINEAR (exact Moller-Trumbore) on the first 4096 rays
    tm, h = refio.run_ref_collide(v, t, r[:4096], "linear", 0)
    print("c0 linear", tm)
    save("c0_linear.npz", rays_md5=md5(r[:4096]), **compact(h))

    # 4. config 1: interior scene, camera + surface rays (closest) and shadow rays
    sc = scenes.interior_c1()
    cam = scenes.camera_rays(cols=[0, 1024, 2048, 3072])          # 16384 rays across the image
    sur = scenes.surface_rays(sc.vertices, sc.indices, 16384)
    sha = scenes.shadow_rays(sc.vertices, sc.indices, 16384)
    rays = np.concatenate([cam, sur, sha])
    tm, h = refio.run_ref_collide(sc.vertices, sc.indices, rays, "bsp_fastest", 0)
    print("c1 fastest", tm)
    save("c1_fastest.npz", mesh_md5=md5(sc.vertices, sc.indices), rays_md5=md5(rays), n_cam=len(cam),
         n_sur=len(sur), n_sha=len(sha), **compact(h))

    # 5. lightmaps: texel enumeration and flags, post-filters
    lightmaps()

    # 6. the reference's plain per-texel gather
    gather()

    # 7. the reference's default bake (radiosity solver read at the first hit)
    bake()


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "lightmaps":
        lightmaps()
    elif len(sys.argv) > 1 and sys.argv[1] == "gather":
        gather()
    elif len(sys.argv) > 1 and sys.argv[1] == "bake":
        bake()
    else:
        main()
