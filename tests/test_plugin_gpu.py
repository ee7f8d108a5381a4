"""The reference-side plugin on a GPU: RRCollider::create with the GPU
technique (100) and its intersect() with collision handlers, against the
reference's own IT_BSP_FASTEST collider over the same RRMesh, in one program
(tests/cpp/plugin_check.cpp) built against the reference library.

The handler contract (include/Lightsprint/RRCollider.h:39-66): init() once,
collides() for each hit, nearest first for IT_BSP techniques (:52-55), the
first accepted hit ends the query, done() is what intersect() returns.  The
reference offers kd-leaf hits sorted by distance (RayHits::getHitOrdered,
RRCollider/IntersectLinear.cpp:396-437) and BSP-plane hits in front-to-back
order (IntersectBspFast.cpp:500-515).  The plugin offers the hits of a ray
in the order (watertight t, triangle index), each once
(rrg_intersect_rrray_one_after).  Every ray is cast twice: once rejecting
every hit (the log is the whole offered sequence) and once accepting the hit
at a given position (the ray's fields are then the accepted hit's).
"""
import numpy as np
import pytest

from tests import plugin_harness as H

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not H.available(), reason="reference library (oracle/_ref) not built")]


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return H.build(tmp_path_factory.mktemp("plugin"))


def stacked_quads():
    """Eight unit quads stacked along z (two triangles each), a duplicate of
    the quad at z = 3 (coincident faces: equal distances), and the quad at
    z = 5 with reversed winding (its front side faces the other way)."""
    v, t = [], []
    for k, z in enumerate([0, 1, 2, 3, 3, 4, 5, 6, 7]):
        b = len(v)
        v += [(-1, -1, z), (1, -1, z), (1, 1, z), (-1, 1, z)]
        if k == 6:
            t += [(b, b + 2, b + 1), (b, b + 3, b + 2)]
        else:
            t += [(b, b + 1, b + 2), (b, b + 2, b + 3)]
    return np.asarray(v, np.float32), np.asarray(t, np.uint32)


def quad_rays(n=2048, seed=5):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:2] = rng.uniform(-0.7, 0.7, (n, 2))   # inside every quad along the whole ray
    r[:, 2] = -1.0
    d = np.stack([rng.uniform(-0.02, 0.02, n), rng.uniform(-0.02, 0.02, n), np.ones(n)], 1)
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3] = 0.0
    r[:, 7] = 100.0
    return r


def record(name, data):
    """Writes a JSON summary to $RRG_TEST_ARTIFACTS (an optional folder)."""
    import json
    import os
    d = os.environ.get("RRG_TEST_ARTIFACTS")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, name + ".json"), "w") as f:
            json.dump(data, f)


def check_accepted(gpu, ref, same_idx, accept_at, v, t, rays):
    """Pass 2 of the rays whose offered sequences are identical: the same
    result, offers and accepted triangle, and that triangle's hitPlane
    bit-identical.  hitDistance (and hitPoint2d, which follows from it) is
    bit-identical except where the reference took the plane of another
    triangle of a near-coplanar BSP node: there the reference is farther
    from the exact FP64 distance than we are whenever it is off by more than
    1e-5 relative, and ours stays within 2e-5.  Returns the number of
    distances that differ."""
    from tests.helpers import exact_hit64
    g, r = gpu[1][same_idx], ref[1][same_idx]
    assert np.array_equal(g["result"], r["result"])
    assert np.array_equal(g["offers"], r["offers"])
    acc = g["result"] == 1
    assert np.all(acc == (np.array([len(gpu[0][i][0]) for i in same_idx]) > accept_at))
    for f in ("tri", "plane"):
        assert np.array_equal(g[f][acc], r[f][acc]), f
    diff = acc & (g["dist"] != r["dist"])
    for k in np.nonzero(diff)[0]:
        ok, d64 = exact_hit64(v, t, rays[same_idx[k]], int(g["tri"][k]))
        assert ok
        e_ours = abs(float(g["dist"][k]) - d64) / abs(d64)
        e_ref = abs(float(r["dist"][k]) - d64) / abs(d64)
        assert e_ours < 2e-5, (k, e_ours)
        assert e_ref <= 1e-5 or e_ours < e_ref, (k, e_ours, e_ref)
    same = acc & ~diff
    for f in ("u", "v"):
        assert np.array_equal(g[f][same], r[f][same]), f
    assert np.allclose(g["point3d"][acc], r["point3d"][acc], rtol=1e-5, atol=1e-5)
    return int(diff.sum())


def test_plugin_technique_100(exe):
    out = H.hello(exe)
    assert "technique=100 hit=1 tri=1 dist=1 u=0.35 v=0.3 front=0" in out, out


def test_handler_replay_stacked_quads(exe, tmp_path):
    v, t = stacked_quads()
    rays = quad_rays()
    info, gpu, ref = H.run_handler(exe, tmp_path, v, t, rays, accept_at=4)
    assert info["gpu_technique"] == 100 and info["ref_technique"] == 4
    # every ray crosses all nine quads: nine hits, each offered once
    assert all(len(s[0]) == 9 for s in gpu[0])
    counts, bad = H.compare_sequences(gpu[0], ref[0])
    assert counts["differ"] == 0, (counts, bad[:8])
    # the coincident pair (quads 3 and 4) is the only place the order may differ
    for (gt, _), (rt, _) in zip(gpu[0], ref[0]):
        diff = np.nonzero(gt != rt)[0]
        assert np.all(np.isin(gt[diff] // 2, [3, 4]))
    same = np.asarray([i for i in range(len(rays)) if np.array_equal(gpu[0][i][0], ref[0][i][0])])
    assert len(same) > 0
    nd = check_accepted(gpu, ref, same, 4, v, t, rays)
    record("handler_stacked_quads", {"counts": counts, "dist_differs": nd})
    # the accepted hit is the fifth of the sequence: the z = 3 pair's second
    # quad or the z = 4 quad, never a farther one
    assert np.all(gpu[1]["result"] == 1) and np.all(gpu[1]["offers"] == 5)


def test_handler_replay_config0(exe, tmp_path):
    """Displaced icosphere (69,451 triangles): 2,048 shell rays that hit it,
    each through the surface and out again (and more where the displacement
    folds); the second hit is accepted."""
    from lightsprintsdk_gb300 import scenes
    from tests.helpers import load_golden
    v, t = scenes.icosphere_c0()
    g = load_golden("c0_fastest.npz")
    rays = scenes.shell_rays(int(g["n"]))[g["hit_idx"][:2048]]
    info, gpu, ref = H.run_handler(exe, tmp_path, v, t, rays, accept_at=1)
    counts, bad = H.compare_sequences(gpu[0], ref[0])
    record("handler_config0", {"counts": counts, "bad": bad[:64]})
    # (the first 69,451 faces of the subdivided sphere leave a small hole,
    # so a few rays leave it without a second hit)
    assert sum(len(s[0]) >= 2 for s in gpu[0]) >= 0.99 * len(rays)
    # observed on GB300: 2,038 identical sequences; on 10 rays the reference
    # offers one triangle twice (a triangle in two kd leaves whose ranges
    # overlap by DELTA_BSP), ours once
    assert counts["differ"] == 0 and counts["tie_order"] <= 2, (counts, bad[:8])
    assert counts["ref_repeat"] <= 12, counts
    same = np.asarray([i for i in range(len(rays)) if np.array_equal(gpu[0][i][0], ref[0][i][0])])
    assert len(same) >= len(rays) - 14
    check_accepted(gpu, ref, same, 1, v, t, rays)


def test_handler_replay_config1(exe, tmp_path):
    """The 1.2 M-triangle interior: 2,048 camera and surface rays of the
    config-1 fixture, the third hit accepted.  Abutting slabs and boxes give
    coincident faces, whose order may differ (ties)."""
    from lightsprintsdk_gb300 import scenes
    sc = scenes.interior_c1()
    cam = scenes.camera_rays(cols=[0, 1024, 2048, 3072])
    sur = scenes.surface_rays(sc.vertices, sc.indices, 16384)
    rays = np.concatenate([cam[::16], sur[::16]])
    info, gpu, ref = H.run_handler(exe, tmp_path, sc.vertices, sc.indices, rays, accept_at=2)
    counts, bad = H.compare_sequences(gpu[0], ref[0])
    record("handler_config1", {"counts": counts, "bad": bad[:64]})
    # observed on GB300: 2,018 identical, 9 tie orders (coincident faces),
    # 17 reference repeats, 4 other (rays grazing abutting slabs, where the
    # reference's plane-distance test and the watertight test disagree)
    assert counts["differ"] <= 4, (counts, bad[:8])
    assert counts["same"] >= 2010, counts
    same = np.asarray([i for i in range(len(rays)) if np.array_equal(gpu[0][i][0], ref[0][i][0])])
    check_accepted(gpu, ref, same, 2, sc.vertices, sc.indices, rays)


def test_multi_object_collider_against_rrcollidermulti(exe, tmp_path):
    """RRCollider::create(nullptr, &objects, GPU technique) against the
    reference's RRColliderMulti on the same RRObjects (each object's collider
    IT_BSP_FASTEST): the config-1 interior as a static object and 64 sphere
    instances, one of them mirrored (negative determinant) and one disabled.
    Without a handler: the same hit, hitObject and hitTriangle on all but
    near-tie rays, and where those agree the same hitFrontSide and
    hitDistance within 1e-5 relative.  With a handler (accept the second
    hit) the ray goes to the reference's own RRColliderMulti, so the results
    are identical."""
    from lightsprintsdk_gb300 import scenes
    from tests.test_scene_gpu import split_interior
    sc = scenes.interior_c1()
    static, sphere, obj_mesh, world, _ = split_interior(sc)
    world = world.copy()
    world[5, :, 0] *= -1.0            # a mirrored instance
    objects = [(int(obj_mesh[i]), i != 9, world[i]) for i in range(len(obj_mesh))]
    rays = np.concatenate([scenes.camera_rays(rows=8, cols=list(range(0, 4096, 16))),
                           scenes.surface_rays(sc.vertices, sc.indices, 8192)])
    info, (g, gh), (r, rh) = H.run_multi(exe, tmp_path, [static, sphere], objects, rays)
    assert info["gpu_technique"] == 100, info
    same = (g["hit"] == r["hit"]) & (g["obj"] == r["obj"]) & (g["tri"] == r["tri"])
    record("multi_object", {"rays": len(rays), "differ": int((~same).sum()), "hits": int(r["hit"].sum()),
                            "mirrored_hits": int(((r["obj"] == 5) & (r["hit"] == 1)).sum()),
                            "disabled_hits_gpu": int(((g["obj"] == 9) & (g["hit"] == 1)).sum())})
    assert (~same).sum() <= max(4, 2e-4 * len(rays)), np.nonzero(~same)[0][:16]
    assert not np.any((g["obj"] == 9) & (g["hit"] == 1))
    assert np.any((r["obj"] == 5) & (r["hit"] == 1))
    m = same & (r["hit"] == 1)
    np.testing.assert_array_equal(g["side"][m], r["side"][m])
    np.testing.assert_allclose(g["dist"][m], r["dist"][m], rtol=1e-5)
    for f in ("result", "obj", "tri", "offers"):
        np.testing.assert_array_equal(gh[f], rh[f], err_msg=f)


def _covered_only(runs, flags):
    """The fixture is processTexel's output, unfiltered; updateLightmaps
    then runs updateLightmap's filters, which with smoothing and spreading
    off change only texels the gather did not cover.  Those are set back to
    what the unfiltered gather leaves there (zero) before comparing."""
    out = []
    for r in runs:
        r = r.copy()
        r[flags == 0] = 0.0
        out.append(r)
    return out


def test_update_lightmaps_adapter_plain_gather(exe, tmp_path):
    """rrgpu_plugin::updateLightmaps (include/rrgpu_update_lightmaps.hpp) on
    a reference RRSolver holding the small room (its static objects' collider
    the GPU technique), with useCurrentSolution (the plain 20-bounce gather),
    against the reference's own processTexel runs of the same atlases
    (tests/golden/gather_ref.npz), by the criteria of the GPU gather's own
    reference test: texels no random number changes to 1e-6, the rest
    statistically, alpha bit-exact."""
    from lightsprintsdk_gb300 import scenes
    from tests.helpers import load_golden, reference_gather_ok, reference_gather_stats
    g = load_golden("gather_ref.npz")
    gs = scenes.gather_room()
    runs = []
    for seed in (21, 22):
        info, px = H.run_lightmaps(exe, tmp_path, gs, g["atlases"], int(g["quality"]), "plain", seed)
        assert info["updated"] == len(g["atlases"]) and info["multi_technique"] == 100, info
        runs.append(px)
    runs = _covered_only(runs, g["flags"])
    stats = reference_gather_stats(g, runs[0], runs[1])
    record("update_lightmaps_plain", {"stats": [{k: (float(v) if not isinstance(v, (bool, int)) else v)
                                                 for k, v in s.items()} for s in stats]})
    for a, s in zip(g["atlases"], stats):
        assert reference_gather_ok(s, det_rel=1e-6), (int(a), s)


def test_update_lightmaps_adapter_default_bake(exe, tmp_path):
    """The same adapter with UpdateParameters' defaults (useCurrentSolution
    false: first gather, radiosity, final gather reading the solver) against
    the reference's own updateLightmaps with its solver (tests/golden/
    bake_ref.npz, filtering with smoothing and spreading off, as here):
    each atlas's mean over its covered texels within the bound the GPU
    bake's own reference test uses, and the texels no random number changes
    to 1e-6."""
    from lightsprintsdk_gb300 import scenes
    from tests.helpers import BAKE_ATLAS_ALLOW, _within, load_golden
    g = load_golden("bake_ref.npz")
    gs = scenes.gather_room()
    runs = []
    for seed in (11, 12, 13):
        info, px = H.run_lightmaps(exe, tmp_path, gs, g["atlases"], int(g["quality"]), "bake", seed)
        assert info["updated"] == len(g["atlases"]), info
        runs.append(px)
    cov = g["flags"] > 0
    ours = np.stack([[r[a][cov[a]][:, :3].astype(np.float64).mean(0) for a in range(cov.shape[0])] for r in runs])
    within = _within(ours, g["atlas_means"].astype(np.float64), BAKE_ATLAS_ALLOW)
    det = g["det_mask"]
    same = np.all(runs[0][..., :3] == runs[1][..., :3], axis=-1) & np.all(runs[0][..., :3] == runs[2][..., :3],
                                                                       axis=-1)
    keep = same[det]
    d = det & same
    rel = np.abs(runs[0][..., :3][d].astype(np.float64) - g["det_rgb"].astype(np.float64)[keep])
    rel /= np.maximum(np.abs(g["det_rgb"].astype(np.float64)[keep]), 1e-30)
    record("update_lightmaps_bake", {"atlas_within": within.tolist(), "det_n": int(d.sum()),
                                     "det_rel": float(rel.max()) if d.any() else 0.0})
    assert float(within.max()) < 1, within
    assert d.sum() > 2000 and float(rel.max()) <= 1e-6
