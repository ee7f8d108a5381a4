"""Parity of the CUDA collider (through the C ABI) with the reference's
outputs (golden fixtures) and with the C oracle, on the seeded workloads.

Tolerances (the benchmark spec): hitTriangle identical for >= 99.999 % of rays, any
difference only at distance ties (|d_ref - d_gpu| <= 1e-6 relative) or where
the reference's own hit is not an exact intersection; hitDistance and
hitPoint2d within 1e-5 relative (absolute floor 1e-6 for (u, v) near 0).
For the same triangle the GPU recomputes the reference's FASTEST formulas,
so against the oracle those fields are bit-exact."""
import numpy as np
import pytest

from lightsprintsdk_gb300 import collider as col
from lightsprintsdk_gb300 import scenes
from oracle import orc
from tests.helpers import classify_mismatches, expand, load_golden, md5

pytestmark = pytest.mark.gpu


def gpu_collide(v, t, rays, **kw):
    c = col.RRCollider.create(v, t, **kw)
    h = c.intersect_batch(rays)
    return c, h


def assert_fields_close(ref, got, mask, rel=1e-5, uv_abs=1e-6):
    d_ok = np.abs(got["dist"][mask] - ref["dist"][mask]) <= rel * np.abs(ref["dist"][mask])
    uv_ok = np.abs(got["uv"][mask] - ref["uv"][mask]) <= np.maximum(rel * np.abs(ref["uv"][mask]), uv_abs)
    return d_ok, uv_ok.all(axis=1)


def test_hello_collider():
    g = load_golden("hello_kat.npz")
    c, h = gpu_collide(g["v"], g["t"], g["rays"])
    assert h["hit"][0] and h["tri"][0] == 1
    assert h["dist"][0] == np.float32(1.0)
    np.testing.assert_array_equal(h["uv"][0], g["bsp_fastest_uv"][0])
    assert h["side"][0] == bool(g["bsp_fastest_side"][0])
    # the RRRay path (rrg_intersect_rrray): the reference record layout
    rr = col.make_rrrays(g["rays"])
    hit = c.intersect_rrrays(rr)
    assert hit[0]
    assert rr["hitTriangle"][0] == 1 and rr["hitDistance"][0] == np.float32(1.0)
    np.testing.assert_array_equal(rr["hitPlane"][0], g["bsp_fastest_plane"][0])
    np.testing.assert_array_equal(rr["hitPoint3d"][0], g["bsp_fastest_point3d"][0])
    assert bool(rr["hitFrontSide"][0]) == bool(g["bsp_fastest_side"][0])


def test_edge_cases():
    g = load_golden("edge_cases.npz")
    v, t, rays = g["v"], g["t"], g["rays"]
    c, h = gpu_collide(v, t, rays)
    assert c.valid_triangles == 7          # triangles 4 (collinear) and 5 (repeated vertex) are dropped
    ref = {f: g[f"bsp_fastest_{f}"] for f in ("hit", "tri", "dist", "uv", "plane", "side")}
    ref["hit"] = ref["hit"].astype(bool)
    ref["side"] = ref["side"].astype(bool)
    cls = classify_mismatches(v, t, rays, ref, h)
    assert not cls["other"], cls
    assert not cls["hit_mismatch"], cls
    same = ref["hit"] & (ref["tri"] == h["tri"])
    np.testing.assert_array_equal(h["dist"][same], ref["dist"][same])
    np.testing.assert_array_equal(h["uv"][same], ref["uv"][same])
    np.testing.assert_array_equal(h["side"][same], ref["side"][same])


@pytest.fixture(scope="module")
def c0():
    v, t = scenes.icosphere_c0()
    g = load_golden("c0_fastest.npz")
    assert md5(v, t) == str(g["mesh_md5"])
    rays = scenes.shell_rays(int(g["n"]))
    assert md5(rays) == str(g["rays_md5"])
    c = col.RRCollider.create(v, t)
    return v, t, rays, expand(g), c


def test_c0_against_reference(c0):
    v, t, rays, ref, c = c0
    h = c.intersect_batch(rays)
    cls = classify_mismatches(v, t, rays, ref, h)
    assert not cls["other"], cls
    n = len(rays)
    n_tri_diff = len(cls["tie"]) + len(cls["ref_off"])
    assert n_tri_diff <= 1e-5 * n, cls
    same = ref["hit"] & h["hit"] & (ref["tri"] == h["tri"])
    np.testing.assert_array_equal(h["side"][same], ref["side"][same])
    # hitDistance: bit-identical except where the reference took the plane of
    # another triangle of a near-coplanar BSP node (the rule of the oracle's
    # own test): wherever the reference is off the exact FP64 distance by
    # more than 1e-5 relative we are closer to it, and ours stays within
    # 2e-5 everywhere
    diff = same & (h["dist"] != ref["dist"])
    assert diff.sum() <= 0.02 * same.sum()
    tri64, d64 = orc.FastestOracle(v, t).exact64(rays, 0)
    err_ours = np.abs(h["dist"][diff] - d64[diff]) / d64[diff]
    err_ref = np.abs(ref["dist"][diff] - d64[diff]) / d64[diff]
    assert err_ours.max() <= err_ref.max()
    big = err_ref > 1e-5
    assert np.all(err_ours[big] < err_ref[big])
    assert np.max(np.abs(h["dist"][same] - d64[same]) / d64[same]) < 2e-5
    # hitPoint2d follows the distance: identical wherever the distance is
    np.testing.assert_array_equal(h["uv"][same & ~diff], ref["uv"][same & ~diff])


def test_c0_against_oracle_bit_exact(c0):
    """Same triangle => the FASTEST fields are bit-identical to the C oracle."""
    v, t, rays, _, c = c0
    o = orc.FastestOracle(v, t).collide(rays, 0)
    h = c.intersect_batch(rays)
    cls = classify_mismatches(v, t, rays, o, h)
    assert not cls["other"], cls
    same = o["hit"] & h["hit"] & (o["tri"] == h["tri"])
    assert same.sum() >= o["hit"].sum() - 2
    for f in ("dist", "uv", "side"):
        np.testing.assert_array_equal(h[f][same], o[f][same], err_msg=f)


def test_c0_full_size_vs_oracle():
    """All 2^20 config-0 rays against the oracle, plus FP64 distance error."""
    v, t = scenes.icosphere_c0()
    rays = scenes.shell_rays(1 << 20)
    c = col.RRCollider.create(v, t)
    h = c.intersect_batch(rays)
    O = orc.FastestOracle(v, t)
    o = O.collide(rays, 0)
    cls = classify_mismatches(v, t, rays, o, h)
    assert not cls["other"], cls
    assert len(cls["tie"]) + len(cls["hit_mismatch"]) <= 1e-5 * len(rays)
    tri64, d64 = O.exact64(rays, 0)
    m = h["hit"] & (tri64 == h["tri"])
    err = np.abs(h["dist"][m] - d64[m]) / d64[m]
    assert err.max() < 2e-5


# config-1 fixture (49,152 rays): differences from IT_BSP_FASTEST observed
# for the oracle (84 ties) and on GB300 (88 ties), classified by
# tests/helpers.py::classify_mismatches
C1_TIES, C1_TIES_GPU, C1_REF_OFF, C1_HIT_SET = 84, 88, 6, 1
C1_GPU_ORACLE_TIES = 28   # GB300 against the C oracle on the same rays: ties only


def test_c1_sample_against_reference():
    sc = scenes.interior_c1()
    g = load_golden("c1_fastest.npz")
    assert md5(sc.vertices, sc.indices) == str(g["mesh_md5"])
    cam = scenes.camera_rays(cols=[0, 1024, 2048, 3072])
    sur = scenes.surface_rays(sc.vertices, sc.indices, int(g["n_sur"]))
    sha = scenes.shadow_rays(sc.vertices, sc.indices, int(g["n_sha"]))
    rays = np.concatenate([cam, sur, sha])
    ref = expand(g)
    c, h = gpu_collide(sc.vertices, sc.indices, rays)
    cls = classify_mismatches(sc.vertices, sc.indices, rays, ref, h)
    assert not cls["other"], cls
    # pinned to the differences observed on GB300 (88 ties on coincident
    # faces, 6 reference non-intersections, 1 of them in the hit set): any
    # new one fails
    assert len(cls["tie"]) <= C1_TIES_GPU, cls["tie"]
    assert len(cls["ref_off"]) <= C1_REF_OFF, cls["ref_off"]
    assert len(cls["hit_mismatch"]) <= C1_HIT_SET, cls["hit_mismatch"]
    assert set(cls["hit_mismatch"]) <= set(cls["ref_off"]) | set(cls["tie"])
    ncam = int(g["n_cam"])
    assert np.array_equal(h["tri"][:ncam], ref["tri"][:ncam])
    # against the oracle (the same exact-nearest rule, evaluated with the
    # GPU's fused multiply-adds in the shear, which the C oracle does
    # without) the only differences are ties between coincident faces
    o = orc.FastestOracle(sc.vertices, sc.indices).collide(rays, 0)
    co = classify_mismatches(sc.vertices, sc.indices, rays, o, h)
    assert not co["other"] and not co["ref_off"] and not co["hit_mismatch"], co
    assert len(co["tie"]) <= C1_GPU_ORACLE_TIES, co["tie"]


def test_any_hit_matches_closest_hit_flag():
    import torch
    sc = scenes.interior_c1()
    rays = np.concatenate([scenes.surface_rays(sc.vertices, sc.indices, 1 << 18),
                           scenes.shadow_rays(sc.vertices, sc.indices, 1 << 18)])
    c = col.RRCollider.create(sc.vertices, sc.indices)
    dr = torch.from_numpy(rays).cuda()
    occ = torch.zeros(len(rays), dtype=torch.uint8, device="cuda")
    hits = torch.empty((len(rays), 4), dtype=torch.float32, device="cuda")
    c.occluded_device(dr.data_ptr(), len(rays), occ.data_ptr())
    c.intersect_device(dr.data_ptr(), len(rays), hits.data_ptr())
    torch.cuda.synchronize()
    assert c.status() == 0
    h = col.decode_hits(hits.cpu().numpy())
    np.testing.assert_array_equal(occ.cpu().numpy().astype(bool), h["hit"])
    o = orc.FastestOracle(sc.vertices, sc.indices).collide(rays, 0, any_hit=True)
    mism = np.nonzero(o["hit"] != h["hit"])[0]
    assert len(mism) <= 1e-4 * len(rays)


def test_rrray_flags_and_untouched_fields(c0):
    """rrg_intersect_rrray writes only the outputs rayFlags request (the
    reference fills them per RRRay::Flags, RRCollider.h:98-106)."""
    v, t, rays, _, c = c0
    r = rays[:4096]
    flags = col.FILL_DISTANCE | col.FILL_TRIANGLE
    rr = col.make_rrrays(r, flags)
    rr["hitPlane"] = 7.0
    rr["hitPoint2d"] = 9.0
    rr["hitFrontSide"] = 5
    hit = c.intersect_rrrays(rr)
    h = c.intersect_batch(r)
    np.testing.assert_array_equal(hit, h["hit"])
    np.testing.assert_array_equal(rr["hitTriangle"][hit], h["tri"][hit])
    np.testing.assert_array_equal(rr["hitDistance"][hit], h["dist"][hit])
    assert np.all(rr["hitPlane"] == 7.0) and np.all(rr["hitPoint2d"] == 9.0) and np.all(rr["hitFrontSide"] == 5)
    rr2 = col.make_rrrays(r, col.FILL_ALL)
    c.intersect_rrrays(rr2)
    np.testing.assert_array_equal(rr2["hitPoint2d"][hit], h["uv"][hit])
    np.testing.assert_array_equal(rr2["hitFrontSide"][hit].astype(bool), h["side"][hit])
    p3 = rr2["hitPoint3d"][hit]
    expect = (r[hit, 0:3] + r[hit, 4:7] * h["dist"][hit, None]).astype(np.float32)
    np.testing.assert_allclose(p3, expect, rtol=1e-6, atol=1e-6)


def test_deterministic_and_rebuild_independent(c0):
    v, t, rays, _, c = c0
    a = c.intersect_batch(rays)
    b = c.intersect_batch(rays)
    c2 = col.RRCollider.create(v, t, build_params={"max_leaf_size": 2})
    d = c2.intersect_batch(rays)
    for f in ("hit", "tri", "dist", "uv", "side"):
        np.testing.assert_array_equal(a[f], b[f])
        np.testing.assert_array_equal(a[f], d[f])


def test_update_rebuilds():
    v, t = scenes.icosphere_c0()
    rays = scenes.shell_rays(1 << 14)
    c = col.RRCollider.create(v, t)
    v2 = (v * np.float32(1.1)).astype(np.float32)
    c.update(v2)
    fresh = col.RRCollider.create(v2, t)
    a, b = c.intersect_batch(rays), fresh.intersect_batch(rays)
    for f in ("hit", "tri", "dist"):
        np.testing.assert_array_equal(a[f], b[f])


def test_degenerate_only_mesh_is_empty_error():
    v = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float32)
    t = np.array([[0, 1, 2]], np.uint32)
    with pytest.raises(col.RRGError) as e:
        col.RRCollider.create(v, t)
    assert e.value.status == 7


def test_nan_vertices_are_ignored_not_fatal():
    """A triangle with a NaN or infinite vertex is never hit (the reference
    drops it as degenerate, IntersectBspFast.cpp:182-186); the rest answer."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [np.nan, 0, 1], [1, 0, 1], [0, 1, 1], [np.inf, 0, 2]], np.float32)
    t = np.array([[0, 1, 2], [3, 4, 5], [6, 1, 2]], np.uint32)
    rays = np.array([[0.2, 0.2, -1, 0, 0, 0, 1, 10], [0.2, 0.2, 0.5, 0, 0, 0, 1, 10]], np.float32)
    c, h = gpu_collide(v, t, rays)
    assert c.valid_triangles == 1
    assert h["hit"][0] and h["tri"][0] == 0 and not h["hit"][1]


def test_out_of_range_index_is_invalid():
    v = np.zeros((3, 3), np.float32)
    t = np.array([[0, 1, 5]], np.uint32)
    with pytest.raises(col.RRGError) as e:
        col.RRCollider.create(v, t)
    assert e.value.status == 1


def test_traversal_variants_agree(c0):
    """The if-if, while-while and default (root-box queue) kernels return
    the same hits (ties broken by triangle index, so bit-identical)."""
    v, t, rays, _, c = c0
    c.set_traversal(1)
    a = c.intersect_batch(rays)
    for trav in (2, 0):
        c.set_traversal(trav)
        b = c.intersect_batch(rays)
        for f in ("hit", "tri", "dist", "uv", "side"):
            np.testing.assert_array_equal(a[f], b[f])


def test_launch_count_counts_device_calls(c0):
    """rrg_launch_count grows by the same positive number for each identical
    device call (the bench reports its growth over the timed region)."""
    import torch
    v, t, rays, _, c = c0
    d_rays = torch.from_numpy(np.ascontiguousarray(rays, dtype=np.float32)).cuda()
    d_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    deltas = []
    for _ in range(3):
        n0 = col.launch_count()
        c.intersect_device(d_rays.data_ptr(), rays.shape[0], d_hits.data_ptr())
        deltas.append(col.launch_count() - n0)
    torch.cuda.synchronize()
    assert deltas[0] >= 1 and deltas[0] == deltas[1] == deltas[2], deltas


def test_ray_orders_agree():
    """Binned and given ray order give bit-identical closest and any hits
    (config-1 sample of camera, surface and shadow rays)."""
    import torch
    sc = scenes.interior_c1()
    rays = np.concatenate([scenes.camera_rays(rows=32, cols=list(range(0, 4096, 16))),
                           scenes.surface_rays(sc.vertices, sc.indices, 1 << 17),
                           scenes.shadow_rays(sc.vertices, sc.indices, 1 << 17)])
    c = col.RRCollider.create(sc.vertices, sc.indices)
    d = torch.from_numpy(rays).cuda()
    n = len(rays)
    out = {}
    for order in (col.RAY_ORDER_AS_GIVEN, col.RAY_ORDER_BINNED):
        c.set_ray_order(order)
        h = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        o = torch.empty(n, dtype=torch.uint8, device="cuda")
        c.intersect_device(d.data_ptr(), n, h.data_ptr())
        c.occluded_device(d.data_ptr(), n, o.data_ptr())
        torch.cuda.synchronize()
        assert c.status() == 0
        out[order] = (h.cpu().numpy().view(np.uint32), o.cpu().numpy())
    np.testing.assert_array_equal(out[1][0], out[2][0])
    np.testing.assert_array_equal(out[1][1], out[2][1])


@pytest.mark.parametrize("n", [3 * (1 << 22) + 12345, 1000003, 70001])
def test_host_pipeline_matches_device(n):
    """rrg_intersect_host returns what rrg_intersect_device returns: above
    4 Mi rays (pipelined, binned chunks of 4 Mi rays, three staging slots
    reused); up to 4 Mi rays from page-locked
    buffers (traced in place in host memory) and from pageable ones (staged
    chunks above 256 Ki rays, below in one piece)."""
    import torch
    v, t = scenes.icosphere_c0()
    c = col.RRCollider.create(v, t)
    rng = np.random.default_rng(5)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-2.5, 2.5, (n, 3))
    d = rng.normal(size=(n, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 0.0
    rays[:, 7] = 10.0
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    for _ in range(2):
        h_hits.fill_(3.0)
        assert col._lib().rrg_intersect_host(c.handle, h_rays.data_ptr(), n, h_hits.data_ptr(), None) == 0
        d_rays = h_rays.cuda()
        d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        c.intersect_device(d_rays.data_ptr(), n, d_hits.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(h_hits.view(torch.int32), d_hits.cpu().view(torch.int32))
    if n <= 1 << 22:   # pageable buffers: the staged copy paths
        p_hits = np.full((n, 4), 3.0, np.float32)
        assert col._lib().rrg_intersect_host(c.handle, rays.ctypes.data, n, p_hits.ctypes.data, None) == 0
        assert np.array_equal(p_hits.view(np.int32), d_hits.cpu().numpy().view(np.int32))
    assert c.status() == 0


def test_wide_bvh_matches_binary():
    """The compressed 8-wide tree returns bit-identical closest and any hits
    to the binary tree (leaf sizes 1..4), on config 0 and a config-1 sample."""
    import torch
    v0, t0 = scenes.icosphere_c0()
    sc = scenes.interior_c1()
    cases = [(v0, t0, scenes.shell_rays(1 << 18)),
             (sc.vertices, sc.indices, np.concatenate([scenes.camera_rays(rows=16, cols=list(range(0, 4096, 64))),
                                                      scenes.surface_rays(sc.vertices, sc.indices, 1 << 17),
                                                      scenes.shadow_rays(sc.vertices, sc.indices, 1 << 16)]))]
    for v, t, rays in cases:
        ref = col.RRCollider.create(v, t, build_params={"bvh_width": 2})
        a = ref.intersect_batch(rays)
        d = torch.from_numpy(rays).cuda()
        occ_a = torch.empty(len(rays), dtype=torch.uint8, device="cuda")
        ref.occluded_device(d.data_ptr(), len(rays), occ_a.data_ptr())
        for leaf in (1, 2, 4):
            w = col.RRCollider.create(v, t, build_params={"bvh_width": 8, "max_leaf_size": leaf})
            b = w.intersect_batch(rays)
            assert w.status() == 0
            for f in ("hit", "tri", "dist", "uv", "side"):
                np.testing.assert_array_equal(a[f], b[f], err_msg=f"leaf {leaf} {f}")
            occ_b = torch.empty_like(occ_a)
            w.occluded_device(d.data_ptr(), len(rays), occ_b.data_ptr())
            torch.cuda.synchronize()
            assert torch.equal(occ_a, occ_b)
            np.testing.assert_array_equal(occ_a.cpu().numpy().astype(bool), a["hit"])
            w.close()
        ref.close()


def test_wide_rejects_large_leaves():
    v, t = scenes.icosphere_c0()
    with pytest.raises(col.RRGError) as e:
        col.RRCollider.create(v, t, build_params={"bvh_width": 8, "max_leaf_size": 8})
    assert e.value.status == 1


def test_autotuner_picks_a_candidate(tmp_path, monkeypatch):
    from lightsprintsdk_gb300 import autotune
    monkeypatch.setenv("RRG_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    v, t = scenes.icosphere_c0()
    rays = scenes.shell_rays(1 << 16)
    e = autotune.tune(v, t, rays)
    assert e["max_leaf_size"] in autotune.LEAF_SIZES and e["traversal"] in autotune.TRAVERSALS
    assert len(e["grays"]) == len(autotune.LEAF_SIZES) * len(autotune.TRAVERSALS)
    assert all(g > 0 for g in e["grays"].values())
    c = autotune.create_tuned(v, t, rays)
    h = c.intersect_batch(rays)
    ref = col.RRCollider.create(v, t).intersect_batch(rays)
    np.testing.assert_array_equal(h["tri"], ref["tri"])


def test_single_ray_calls_from_many_threads_are_combined():
    """RRCollider::intersect(RRRay&) is thread-safe in the reference
    (RRCollider.h:145,217-228) and its callers use it from OpenMP loops
    (RRSolver/gather.cpp:917).  16 Python threads (ctypes releases the GIL)
    each trace their share of 6,000 rays one call at a time while another
    thread runs batch calls on the same collider: every record must be
    byte-identical to a batch trace of the same rays."""
    import threading
    import time
    room = scenes.interior_c1()
    c = col.RRCollider.create(room.vertices, room.indices)
    rays = scenes.surface_rays(room.vertices, room.indices, 6000)
    want = col.make_rrrays(rays)
    want_hit = c.intersect_rrrays(want)
    got = col.make_rrrays(rays)
    got_hit = np.zeros(len(got), bool)
    other_rays = scenes.surface_rays(room.vertices, room.indices, 20000)
    other_want = col.make_rrrays(other_rays)
    c.intersect_rrrays(other_want)
    errors = []
    stop = threading.Event()

    def single(t):
        try:
            for i in range(t, len(got), 16):
                got_hit[i] = c.intersect(got, i)
        except Exception as e:   # reported below
            errors.append(e)

    def batches():
        try:
            while not stop.is_set():
                o = col.make_rrrays(other_rays)
                c.intersect_rrrays(o)
                if o.tobytes() != other_want.tobytes():
                    errors.append(AssertionError("batch call disturbed"))
        except Exception as e:
            errors.append(e)

    bt = threading.Thread(target=batches)
    bt.start()
    threads = [threading.Thread(target=single, args=(t,)) for t in range(16)]
    t0 = time.perf_counter()
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    dt = time.perf_counter() - t0
    stop.set()
    bt.join()
    assert not errors, errors[0]
    np.testing.assert_array_equal(got_hit, want_hit)
    assert got.tobytes() == want.tobytes()
    nb, nr = c.combined()
    assert nr == len(got)
    assert 0 < nb <= nr, (nb, nr)
    print(f"combined single-ray calls: {nr} rays in {nb} batches, {nr / dt:.0f} rays/s on 16 threads")
    c.close()


@pytest.mark.parametrize("threads", [1, 32])
def test_native_threads_single_ray_calls(tmp_path, threads):
    """The same from native host threads (tests/cpp/combine_threads.cpp, one
    std::thread per OpenMP-like worker): records byte-identical to a batch
    trace, and the rate printed for the record."""
    import os
    import subprocess
    from lightsprintsdk_gb300 import build as B
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = B.build()
    exe = tmp_path / "combine_threads"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{root}/include",
                    os.path.join(root, "tests", "cpp", "combine_threads.cpp"), "-o", str(exe), lib,
                    f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread"], check=True, capture_output=True, text=True)
    room = scenes.interior_c1()
    rays = scenes.surface_rays(room.vertices, room.indices, 40000)
    np.ascontiguousarray(room.vertices, np.float32).tofile(tmp_path / "xyz.f32")
    np.ascontiguousarray(room.indices, np.uint32).tofile(tmp_path / "idx.u32")
    col.make_rrrays(rays).tofile(tmp_path / "rays.rrray")
    out = subprocess.run([str(exe), str(tmp_path), str(threads)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    traced, batches, secs = out.stdout.split()
    c = col.RRCollider.create(room.vertices, room.indices)
    want = col.make_rrrays(rays)
    want_hit = c.intersect_rrrays(want)
    c.close()
    got = np.fromfile(tmp_path / "out.rrray", col.RRRAY_DTYPE)
    got_hit = np.fromfile(tmp_path / "hit.u8", np.uint8).astype(bool)
    np.testing.assert_array_equal(got_hit, want_hit)
    assert got.tobytes() == want.tobytes()
    assert int(traced) == len(rays)
    print(f"native single-ray calls, {threads} threads: {len(rays) / float(secs):.0f} rays/s, "
          f"{int(batches)} batches")


@pytest.mark.parametrize("tuning", [(16, 128, 9), (0, 32, 0), (32, 512, 9), (8, 1024, 0)])
def test_compact_traversal_is_bit_identical(tuning):
    """RRG_TRAVERSAL_COMPACT (per-lane walks over warp-claimed ray blocks,
    shared-memory stack top) against the if-if kernel on the config-1 interior: closest-hit
    records and any-hit flags bit for bit, in the given and the binned ray
    order, for several settings of its knobs."""
    import torch
    sc = scenes.interior_c1()
    rays = np.concatenate([scenes.camera_rays(rows=64), scenes.surface_rays(sc.vertices, sc.indices, 1 << 18),
                           scenes.shadow_rays(sc.vertices, sc.indices, 1 << 16)])
    n = len(rays)
    c = col.RRCollider.create(sc.vertices, sc.indices)
    dr = torch.from_numpy(rays).cuda()
    ref = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    got = torch.empty_like(ref)
    occ_ref = torch.empty(n, dtype=torch.uint8, device="cuda")
    occ = torch.empty_like(occ_ref)
    c.set_traversal(1)
    c.intersect_device(dr.data_ptr(), n, ref.data_ptr())
    c.occluded_device(dr.data_ptr(), n, occ_ref.data_ptr())
    assert c.status() == 0
    c.set_traversal(3)
    c.set_compact_tuning(*tuning)
    for order in (col.RAY_ORDER_AS_GIVEN, col.RAY_ORDER_BINNED):
        c.set_ray_order(order)
        got.fill_(7.0)
        occ.fill_(7)
        c.intersect_device(dr.data_ptr(), n, got.data_ptr())
        c.occluded_device(dr.data_ptr(), n, occ.data_ptr())
        assert c.status() == 0
        # bit patterns (a miss record holds 0xFFFFFFFF, a NaN as a float)
        assert torch.equal(got.view(torch.int32), ref.view(torch.int32)), (tuning, order)
        assert torch.equal(occ, occ_ref), (tuning, order)
    c.close()


@pytest.mark.parametrize("scene", ["c0", "c1"])
def test_root_queue_traversal_is_bit_identical(scene):
    """RRG_TRAVERSAL_ROOT_QUEUE (rays that enter neither root child box
    answered at once, the others queued per warp) against the if-if kernel:
    closest-hit records with planes and points, and any-hit flags, bit for
    bit, in the given and the binned order; on config 0's shell rays (88 %
    pass the sphere's box by) with rays of tmin > tmax and a ragged count,
    and on the config-1 interior (every ray inside the tree's box)."""
    import torch
    if scene == "c0":
        v, t = scenes.icosphere_c0()
        rays = scenes.shell_rays((1 << 18) + 77)
        rays[::101, 3] = rays[::101, 7] + 1.0   # empty interval
    else:
        sc = scenes.interior_c1()
        v, t = sc.vertices, sc.indices
        rays = np.concatenate([scenes.camera_rays(rows=64), scenes.surface_rays(v, t, 1 << 18),
                               scenes.shadow_rays(v, t, (1 << 16) + 13)])
    n = len(rays)
    c = col.RRCollider.create(v, t)
    dr = torch.from_numpy(rays).cuda()
    out = {}
    for trav in (1, 4):
        c.set_traversal(trav)
        for order in (col.RAY_ORDER_AS_GIVEN, col.RAY_ORDER_BINNED):
            c.set_ray_order(order)
            h = torch.full((n, 4), 7.0, dtype=torch.float32, device="cuda")
            pl = torch.full((n, 4), 7.0, dtype=torch.float32, device="cuda")
            pt = torch.full((n, 3), 7.0, dtype=torch.float32, device="cuda")
            occ = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
            c.intersect_device(dr.data_ptr(), n, h.data_ptr(), pl.data_ptr(), pt.data_ptr())
            c.occluded_device(dr.data_ptr(), n, occ.data_ptr())
            assert c.status() == 0
            out[trav, order] = (h.view(torch.int32), pl.view(torch.int32), pt.view(torch.int32), occ)
    for order in (col.RAY_ORDER_AS_GIVEN, col.RAY_ORDER_BINNED):
        for a, b in zip(out[1, order], out[4, order]):
            assert torch.equal(a, b), order
    if scene == "c0":
        missed = (out[1, col.RAY_ORDER_AS_GIVEN][0][:, 1] == -1).float().mean().item()
        assert missed > 0.9
    c.close()


def test_compact_tuning_rejects_bad_knobs():
    v, t = scenes.icosphere_c0()
    c = col.RRCollider.create(v, t)
    for bad in [(12, 128, 9), (16, 100, 9), (16, 2048, 9), (16, 0x7FFFFFE0, 9), (16, 128, 8)]:
        with pytest.raises(col.RRGError):
            c.set_compact_tuning(*bad)
    c.set_compact_tuning(0xFFFFFFFF, 0, 0xFFFFFFFF)
    c.close()
