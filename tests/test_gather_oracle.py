"""CPU checks of the gather oracle (oracle/rr_gather.c): the sample-stream
hash matches the Python generators, the enumeration conserves area, the
float gather agrees with its FP64-accumulated twin, and the gather matches
the reference's own per-texel gather (bit-exact where no random number
matters, statistically elsewhere)."""
import numpy as np

from lightsprintsdk_gb300 import scenes
from oracle import orc
from tests.helpers import (GATHER_Z_MEAN, load_golden, md5, reference_bake_ok, reference_bake_stats,
                           reference_gather_ok, reference_gather_stats)


def test_hash_matches_python_generators():
    for seed, stream, idx in [(0, 0, 0), (1, 2, 3), (0xC2, 61, 123456789), (2**40 + 5, 65, 2**50 + 7)]:
        assert orc.hash_u64(seed, stream, idx) == int(scenes.hash_u64(seed, stream, idx))


def test_enumeration_conserves_area():
    """Sub-texel areas sum to half the triangles' map areas (the reference
    measures sub-texels in triangle space, where a triangle has area 1/2,
    and scales by the map-space area: lightmap.cpp:313-318)."""
    gs = scenes.gather_c2()
    for a in (9, 100):
        ids = np.nonzero(gs.tri_atlas == a)[0]
        off, st = orc.enumerate_atlas(gs.uv[ids], ids, gs.size)
        uv = gs.uv[ids].astype(np.float64)
        area = 0.5 * np.abs((uv[:, 1, 0] - uv[:, 0, 0]) * (uv[:, 2, 1] - uv[:, 0, 1])
                            - (uv[:, 2, 0] - uv[:, 0, 0]) * (uv[:, 1, 1] - uv[:, 0, 1]))
        assert abs(st["area"].astype(np.float64).sum() - 0.5 * area.sum()) < 1e-3 * area.sum()
        assert np.all(np.diff(off.astype(np.int64)) >= 0)
        # each texel's list is in triangle order
        for t in np.nonzero(np.diff(off) > 1)[0][:200]:
            tri = st["tri"][off[t]:off[t + 1]]
            assert np.all(np.diff(tri.astype(np.int64)) >= 0)


def test_gather_fp32_vs_fp64_accumulation():
    gs = scenes.gather_c2()
    G = orc.GatherOracle(gs, quality=16)
    a = 9
    ids = np.nonzero(gs.tri_atlas == a)[0]
    off, st = orc.enumerate_atlas(gs.uv[ids], ids, gs.size)
    sel = np.nonzero(np.diff(off) > 0)[0][::97][:64]
    tid = (a * gs.size * gs.size + sel).astype(np.uint64)
    cnt = (off[sel + 1] - off[sel]).astype(np.uint64)
    o2 = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint64)
    sts = np.concatenate([st[off[i]:off[i + 1]] for i in sel])
    f32 = G.gather(tid, o2, sts, 0)
    f64 = G.gather(tid, o2, sts, 0, fp64=True)
    rel = np.abs(f32[:, :3] - f64[:, :3]) / np.maximum(np.abs(f64[:, :3]), 1e-9)
    assert rel.max() < 1e-5
    # at quality 16 a texel may find no light at all; nearly all do
    assert np.all(f32[:, :3] >= 0) and np.all(f32[:, :3] > 0, axis=1).sum() >= 60
    again = G.gather(tid, o2, sts, 0)
    np.testing.assert_array_equal(f32, again)


def test_directional_mode_properties():
    """Directional mode (gather.cpp:255-272, 468-486): the four outputs are
    the same samples weighted by the UE3 basis directions (gather.cpp:43-49).
    LS_LIGHTMAP's weight for a sample is its cosine to the re-normalised
    normal over its cosine to the normal, so it matches the plain mode's
    value to float rounding; the three directions are non-negative, bent
    normals are unchanged, and the weights are lower on average than 1."""
    gs = scenes.gather_c2()
    G = orc.GatherOracle(gs, quality=16)
    a = 9
    ids = np.nonzero(gs.tri_atlas == a)[0]
    off, st = orc.enumerate_atlas(gs.uv[ids], ids, gs.size)
    sel = np.nonzero(np.diff(off) > 0)[0][::131][:48]
    tid = (a * gs.size * gs.size + sel).astype(np.uint64)
    cnt = (off[sel + 1] - off[sel]).astype(np.uint64)
    o2 = np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint64)
    sts = np.concatenate([st[off[i]:off[i + 1]] for i in sel])
    plain, bent = G.gather(tid, o2, sts, 0, bent=True)
    lm, dirs, bent_d = G.gather_directional(tid, o2, sts, 0)
    np.testing.assert_allclose(lm[:, :3], plain[:, :3], rtol=1e-5, atol=1e-7)
    np.testing.assert_array_equal(bent_d, bent)
    assert np.all(dirs[..., :3] >= 0) and np.all(dirs[..., 3] == lm[:, None, 3])
    assert dirs[..., :3].sum() > 0
    assert dirs[..., :3].mean() < lm[:, :3].mean()


def _room_oracle_runs(g, quality: int, max_depth: int, seeds=(11, 12)):
    gs = scenes.gather_room()
    atl = [int(a) for a in g["atlases"]]
    S = gs.size * gs.size
    flags = orc.gather_flags(gs, atl)
    subs = []
    for a in atl:
        ids = np.nonzero(gs.tri_atlas == a)[0]
        subs.append(orc.enumerate_atlas(gs.uv[ids], ids, gs.size))
    runs = []
    for seed in seeds:
        G = orc.GatherOracle(gs, quality=quality, max_depth=max_depth, seed=seed, flags=flags)
        runs.append(np.stack([G.gather((a * S + np.arange(S)).astype(np.uint64), off, st, 0)
                              .reshape(gs.size, gs.size, 4) for a, (off, st) in zip(atl, subs)]))
    return runs


def test_oracle_gather_matches_the_reference_gather():
    """The oracle's plain N-bounce gather against the reference's own
    processTexel (gather.cpp:600-836, run with no radiosity solver so that
    its PathtracerWorker shoots shadow rays at every hit and continues by
    Russian roulette up to stopAtDepth 20; tests/golden/gather_ref.npz: two
    runs over four whole atlases of the small room at quality 256, the
    quality of the runs here, since the sub-texel stepping depends on it).
    The texels whose value no random number changes (about 2,300 on each
    slab atlas) are bit-exact; the rest use other random numbers, so they
    are compared statistically: per atlas and channel the mean difference
    within 4.5 standard errors and 1 %, every 8x8 block within 5.5, the
    texel-by-texel spread what both sides' measured noise predicts, alpha
    (TexelFlags / 255) bit-exact."""
    g = load_golden("gather_ref.npz")
    gs = scenes.gather_room()
    assert md5(gs.scene.vertices, gs.scene.indices, gs.albedo, gs.uv, gs.tri_atlas) == str(g["scene_md5"])
    o1, o2 = _room_oracle_runs(g, int(g["quality"]), 20)
    stats = reference_gather_stats(g, o1, o2)
    for a, s in zip(g["atlases"], stats):
        assert reference_gather_ok(s, det_rel=0.0), (int(a), s)
    assert stats[0]["det_n"] > 1000 and stats[1]["det_n"] > 1000, stats


def test_reference_gather_comparison_detects_missing_bounces():
    """The comparison's power, with a mistake planted in the oracle: paths
    cut at 3 bounces instead of 20 fail it on every atlas."""
    g = load_golden("gather_ref.npz")
    o1, o2 = _room_oracle_runs(g, int(g["quality"]), 3)
    for a, s in zip(g["atlases"], reference_gather_stats(g, o1, o2)):
        assert not reference_gather_ok(s), (int(a), s)
        assert s["z_mean"] > GATHER_Z_MEAN, (int(a), s)


def _room_bake_runs(g, seeds=(11, 12, 13), max_depth: int = 20):
    gs = scenes.gather_room()
    atl = [int(a) for a in g["atlases"]]
    S = gs.size * gs.size
    flags = orc.gather_flags(gs, atl)
    subs = []
    for a in atl:
        ids = np.nonzero(gs.tri_atlas == a)[0]
        subs.append(orc.enumerate_atlas(gs.uv[ids], ids, gs.size))
    runs, directs, indirects = [], [], []
    for seed in seeds:
        G = orc.GatherOracle(gs, quality=int(g["quality"]), max_depth=max_depth, seed=seed, flags=flags)
        d, ind, _ = G.bake_solver()
        runs.append(np.stack([G.gather((a * S + np.arange(S)).astype(np.uint64), off, st, 0)
                              .reshape(gs.size, gs.size, 4) for a, (off, st) in zip(atl, subs)]))
        directs.append(d)
        indirects.append(ind)
    return gs, runs, directs, indirects


def test_oracle_bake_matches_the_reference_bake():
    """The oracle's restatement of the default bake (first gather per
    triangle, radiosity, final gather reading the solver at the first hit)
    against the reference's own updateLightmaps with its radiosity solver
    (tests/golden/bake_ref.npz: four realizations, quality 256, four atlases
    of the small room).  The texels no random number changes are bit-exact;
    the per-triangle first gather agrees statistically; atlas means and the
    class indirect agree within both sides' scatter plus 0.5 % and 1 % (the
    reference stops propagating at its accuracy target, ours converges)."""
    g = load_golden("bake_ref.npz")
    gs, runs, directs, indirects = _room_bake_runs(g)
    assert md5(gs.scene.vertices, gs.scene.indices, gs.albedo, gs.uv, gs.tri_atlas) == str(g["scene_md5"])
    s = reference_bake_stats(g, gs, runs, directs, indirects)
    assert reference_bake_ok(s, det_rel=0.0), s
    assert s["det_n"] > 2000, s


def test_reference_bake_comparison_detects_a_missing_solver():
    """The comparison's power: the plain N-bounce gather cut at one bounce
    (direct light at the first hit, no radiosity) in place of the solver
    fails it."""
    g = load_golden("bake_ref.npz")
    gs = scenes.gather_room()
    atl = [int(a) for a in g["atlases"]]
    S = gs.size * gs.size
    flags = orc.gather_flags(gs, atl)
    runs, directs, indirects = [], [], []
    for seed in (11, 12, 13):
        G = orc.GatherOracle(gs, quality=int(g["quality"]), max_depth=0, seed=seed, flags=flags)
        d, ind, _ = G.bake_solver()
        G.s.solver_direct = None
        G.s.solver_corner = None
        out = []
        for a in atl:
            ids = np.nonzero(gs.tri_atlas == a)[0]
            off, st = orc.enumerate_atlas(gs.uv[ids], ids, gs.size)
            out.append(G.gather((a * S + np.arange(S)).astype(np.uint64), off, st, 0).reshape(gs.size, gs.size, 4))
        runs.append(np.stack(out))
        directs.append(d)
        indirects.append(ind)
    s = reference_bake_stats(g, gs, runs, directs, indirects)
    assert not reference_bake_ok(s), s
    assert float(s["atlas"].max()) > 2, s
