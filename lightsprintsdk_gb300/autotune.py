"""Autotuner for the collider: chooses the BVH leaf size and the traversal
kernel per GPU and mesh-size bucket by timing candidates on a sample of the
caller's own rays.  Results persist in a JSON file (the package's _lib
directory, or $RRG_AUTOTUNE_CACHE) keyed by "<gpu name>|<log2 triangles>|<tag>".

Candidates: max_leaf_size in {2, 4, 8} x traversal in {if-if, while-while,
compact, root-box queue} for single colliders; for mesh batches (tune_batch) the BVH width
and leaf size x rays per warp in {32, 128} x shared-memory stack entries
per thread in {0, 8, 16} (binary trees; the 8-wide walk has its own
stack).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import build as _build
from . import collider as col

LEAF_SIZES = (2, 4, 8)
TRAVERSALS = (1, 2, 3, 4)   # RRG_TRAVERSAL_IF_IF, _WHILE_WHILE, _COMPACT, _ROOT_QUEUE


def cache_path() -> str:
    return os.environ.get("RRG_AUTOTUNE_CACHE", os.path.join(_build.OUT_DIR, "autotune.json"))


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d: dict) -> None:
    os.makedirs(os.path.dirname(cache_path()), exist_ok=True)
    tmp = cache_path() + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, cache_path())


def key(ntri: int, tag: str = "closest") -> str:
    import torch
    name = torch.cuda.get_device_name(0).replace("|", "/")
    return f"{name}|{int(math.log2(max(ntri, 1)))}|{tag}"


def tune(vertices, indices, sample_rays: np.ndarray, tag: str = "closest", repeats: int = 5,
         force: bool = False) -> dict:
    """Times every candidate on the sample (device-resident rays, CUDA
    events) and returns {"max_leaf_size", "traversal", "grays": {...}}; the
    best is remembered for the bucket."""
    import torch
    k = key(int(np.asarray(indices).reshape(-1, 3).shape[0]), tag)
    db = _load()
    if k in db and not force:
        return db[k]
    rays = torch.from_numpy(np.ascontiguousarray(sample_rays, np.float32)).cuda()
    n = rays.shape[0]
    hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    results = {}
    for leaf in LEAF_SIZES:
        c = col.RRCollider.create(vertices, indices, build_params={"max_leaf_size": leaf})
        for trav in TRAVERSALS:
            col._lib().rrg_collider_set_traversal(c.handle, trav)
            for _ in range(2):
                c.intersect_device(rays.data_ptr(), n, hits.data_ptr())
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(repeats):
                c.intersect_device(rays.data_ptr(), n, hits.data_ptr())
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / repeats
            results[f"leaf{leaf}_trav{trav}"] = n / (ms * 1e-3) / 1e9
        c.close()
    best = max(results, key=results.get)
    leaf = int(best.split("_")[0][4:])
    trav = int(best.split("_")[1][4:])
    entry = {"max_leaf_size": leaf, "traversal": trav, "grays": results, "sample_rays": int(n)}
    db[k] = entry
    _save(db)
    return entry


def create_tuned(vertices, indices, sample_rays: np.ndarray, tag: str = "closest") -> col.RRCollider:
    """A collider built and configured with the tuned choice for this bucket."""
    e = tune(vertices, indices, sample_rays, tag)
    c = col.RRCollider.create(vertices, indices, build_params={"max_leaf_size": e["max_leaf_size"],
                                                               "traversal": e["traversal"]})
    return c


BATCH_RAYS_PER_WARP = (32, 128)
BATCH_STACK_SMEM = (0, 8, 16)
# (bvh width, leaf size): the 8-wide tree takes leaves of at most 4
BATCH_TREES = ((2, 2), (2, 4), (2, 8), (8, 2), (8, 4))


def tune_batch(mb, rays_dev, ray_off_dev, repeats: int = 3, force: bool = False) -> dict:
    """BVH width and leaf size x rays per warp x shared-memory stack depth x
    root-box queue (binary trees) for a mesh batch (scenes.MeshBatch), timed
    with CUDA events on the caller's device rays (all of them: the tuner
    sees the real mix of meshes and ray sets).  Remembered per GPU and
    log2(total triangles) bucket; returns {"bvh_width", "max_leaf_size",
    "rays_per_warp", "stack_smem", "root_queue", "grays": {...}}."""
    import torch
    from . import batch as rb
    k = key(int(mb.tri_off[-1]), "batch")
    db = _load()
    if k in db and not force:
        return db[k]
    n = rays_dev.shape[0]
    hits = torch.empty((n, 4), dtype=torch.float32, device=rays_dev.device)
    results = {}
    for width, leaf in BATCH_TREES:
        b = rb.RRColliderBatch.from_meshes(mb, build_params={"max_leaf_size": leaf, "bvh_width": width})
        for rpw in BATCH_RAYS_PER_WARP:
            for sd in (BATCH_STACK_SMEM if width == 2 else (0,)):
                for q in ((0, 1) if width == 2 else (0,)):
                    b.set_rays_per_warp(rpw)
                    b.set_stack_smem(sd)
                    if width == 2:
                        b.set_root_queue(bool(q))
                    b.intersect_device(rays_dev.data_ptr(), ray_off_dev.data_ptr(), n, hits.data_ptr())
                    torch.cuda.synchronize()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    for _ in range(repeats):
                        b.intersect_device(rays_dev.data_ptr(), ray_off_dev.data_ptr(), n, hits.data_ptr())
                    e1.record()
                    torch.cuda.synchronize()
                    results[f"w{width}_leaf{leaf}_rpw{rpw}_sd{sd}_q{q}"] = (
                        n / (e0.elapsed_time(e1) / repeats * 1e-3) / 1e9)
        b.close()
    best = max(results, key=results.get)
    w, leaf, rpw, sd, q = best.split("_")
    entry = {"bvh_width": int(w[1:]), "max_leaf_size": int(leaf[4:]), "rays_per_warp": int(rpw[3:]),
             "stack_smem": int(sd[2:]), "root_queue": int(q[1:]), "grays": results, "rays": int(n)}
    db[k] = entry
    _save(db)
    return entry
