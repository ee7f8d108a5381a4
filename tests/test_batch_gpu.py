"""Uneven mesh batches (include/rrgpu_batch.h) on the GPU: the multi-root
build and the persistent batch launch against per-mesh colliders (bit
exact) and the C oracle, across rays-per-warp settings and graph replays."""
import numpy as np
import pytest

from lightsprintsdk_gb300 import batch as rb
from lightsprintsdk_gb300 import collider as col
from lightsprintsdk_gb300 import scenes
from oracle import orc
from tests.helpers import classify_mismatches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch():
    """24 meshes (1k..30k triangles), plus a mesh of degenerate triangles
    only and a mesh that gets no rays; 300..20k rays per mesh."""
    import torch
    mb = scenes.batch_meshes_c3(seed=0x5C3, nmesh=24, tri_lo=1000, tri_hi=30000)
    # mesh 5 -> degenerate triangles only (no valid triangle: its rays miss)
    t0, t1 = int(mb.tri_off[5]), int(mb.tri_off[6])
    mb.indices[t0:t1] = 0
    counts = scenes.log_uniform_counts(0x5C3, 110, mb.nmesh, 300, 20000)
    counts[7] = 0
    rays, off = scenes.batch_rays(mb, counts, seed=0x5C3)
    b = rb.RRColliderBatch.from_meshes(mb)
    off_d = torch.from_numpy(off.astype(np.uint32)).cuda()
    return mb, counts, rays, off, off_d, b


def run(b, rays, off_d, k=32):
    import torch
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    b.set_rays_per_warp(k)
    b.intersect_device(rays.data_ptr(), off_d.data_ptr(), rays.shape[0], hits.data_ptr())
    torch.cuda.synchronize()
    assert b.status() == 0
    return hits.cpu().numpy()


def test_batch_equals_per_mesh_colliders(small_batch):
    mb, counts, rays, off, off_d, b = small_batch
    h = run(b, rays, off_d)
    r = rays.cpu().numpy()
    for m in range(mb.nmesh):
        a, e = int(off[m]), int(off[m + 1])
        if a == e:
            continue
        v, t = mb.mesh(m)
        if m == 5:
            assert (h[a:e, 1].view(np.uint32) == 0xFFFFFFFF).all()
            with pytest.raises(col.RRGError):
                col.RRCollider.create(v, t)
            continue
        c = col.RRCollider.create(v, t)
        got = col.decode_hits(h[a:e])
        one = c.intersect_batch(r[a:e])
        for f in ("hit", "tri", "dist", "uv", "side"):
            np.testing.assert_array_equal(got[f], one[f], err_msg=f"mesh {m} field {f}")
        c.close()


def test_batch_against_oracle(small_batch):
    mb, counts, rays, off, off_d, b = small_batch
    h = run(b, rays, off_d)
    r = rays.cpu().numpy()
    checked = 0
    for m in range(0, mb.nmesh, 3):
        a, e = int(off[m]), int(off[m + 1])
        if a == e or m == 5:
            continue
        v, t = mb.mesh(m)
        o = orc.FastestOracle(v, t).collide(r[a:e], 0)
        got = col.decode_hits(h[a:e])
        cls = classify_mismatches(v, t, r[a:e], o, got)
        assert not cls["other"], (m, cls)
        same = o["hit"] & got["hit"] & (o["tri"] == got["tri"])
        assert same.sum() >= o["hit"].sum() - 2, m
        for f in ("dist", "uv", "side"):
            np.testing.assert_array_equal(got[f][same], o[f][same], err_msg=f"mesh {m} {f}")
        checked += e - a
    assert checked > 10000


def test_rays_per_warp_and_graph_replay_agree(small_batch):
    import torch
    mb, counts, rays, off, off_d, b = small_batch
    base = run(b, rays, off_d, 32)
    for k in (64, 128, 256):
        np.testing.assert_array_equal(run(b, rays, off_d, k).view(np.uint32), base.view(np.uint32), err_msg=str(k))
    # a recapture for another output buffer, then two replays of that graph
    b.set_rays_per_warp(32)
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    for _ in range(2):
        hits.fill_(7.0)
        b.intersect_device(rays.data_ptr(), off_d.data_ptr(), rays.shape[0], hits.data_ptr())
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hits.cpu().numpy().view(np.uint32), base.view(np.uint32))


def test_leaf_sizes_agree(small_batch):
    mb, counts, rays, off, off_d, b = small_batch
    base = run(b, rays, off_d)
    for leaf in (1, 2, 8):
        b2 = rb.RRColliderBatch.from_meshes(mb, build_params={"max_leaf_size": leaf})
        np.testing.assert_array_equal(run(b2, rays, off_d).view(np.uint32), base.view(np.uint32), err_msg=str(leaf))
        b2.close()


def test_wide_batch_matches_binary(small_batch):
    mb, counts, rays, off, off_d, b = small_batch
    base = run(b, rays, off_d)
    w = rb.RRColliderBatch.from_meshes(mb, build_params={"bvh_width": 8})
    for k in (32, 128):
        np.testing.assert_array_equal(run(w, rays, off_d, k).view(np.uint32), base.view(np.uint32), err_msg=str(k))
    w.close()


def test_index_outside_its_mesh_is_invalid():
    mb = scenes.batch_meshes_c3(seed=0x5C4, nmesh=3, tri_lo=1000, tri_hi=2000)
    bad = mb.indices.copy()
    # a valid global index, but outside mesh 1's own vertices
    bad[int(mb.tri_off[1])] = int(mb.vert_off[2] - mb.vert_off[1]) + 3
    with pytest.raises(col.RRGError) as e:
        rb.RRColliderBatch.create(mb.vertices, bad, mb.vert_off, mb.tri_off)
    assert e.value.status == 1


def test_launch_count_counts_graph_replays_not_captures(small_batch):
    """rrg_launch_count: a replay of the captured batch graph adds its kernel
    nodes; the capture itself launches nothing."""
    import torch
    mb, counts, rays, off, off_d, b = small_batch
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    b.set_rays_per_warp(32)
    deltas = []
    for _ in range(3):
        torch.cuda.synchronize()
        n0 = col.launch_count()
        b.intersect_device(rays.data_ptr(), off_d.data_ptr(), rays.shape[0], hits.data_ptr())
        deltas.append(col.launch_count() - n0)
    torch.cuda.synchronize()
    assert deltas[0] >= 1 and deltas[0] == deltas[1] == deltas[2], deltas


def test_stack_depths_agree(small_batch):
    """The autotuner's stack-depth knob (shared-memory entries per thread)
    changes where the traversal stack lives, never a result."""
    mb, counts, rays, off, off_d, b = small_batch
    b.set_stack_smem(0)
    base = run(b, rays, off_d, 32)
    for sd in (8, 16, 32):
        b.set_stack_smem(sd)
        for k in (32, 128):
            np.testing.assert_array_equal(run(b, rays, off_d, k).view(np.uint32), base.view(np.uint32),
                                          err_msg=f"stack {sd} rays per warp {k}")
    with pytest.raises(col.RRGError):
        b.set_stack_smem(12)
    b.set_stack_smem(0)


def test_root_queue_agrees(small_batch):
    """The batch kernel's root-box queue (rays entering neither child box of
    their mesh's root answered at once, the rest traced 32 to a warp) gives
    the same records, bit for bit, for every stack depth and rays-per-warp
    setting, in plain launches and in the graph rebuild."""
    import torch
    mb, counts, rays, off, off_d, b = small_batch
    b.set_root_queue(False)
    b.set_stack_smem(0)
    base = run(b, rays, off_d, 32)
    b.set_root_queue(True)
    for sd in (0, 16):
        b.set_stack_smem(sd)
        for k in (32, 128):
            np.testing.assert_array_equal(run(b, rays, off_d, k).view(np.uint32), base.view(np.uint32),
                                          err_msg=f"queue, stack {sd} rays per warp {k}")
    b.set_stack_smem(0)
    n = rays.shape[0]
    hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    b.rebuild_intersect_device(rays.data_ptr(), off_d.data_ptr(), n, hits.data_ptr())
    torch.cuda.synchronize()
    assert b.status() == 0
    np.testing.assert_array_equal(hits.cpu().numpy().view(np.uint32), base.view(np.uint32))
    b.set_root_queue(False)


def test_rebuild_in_graph_equals_per_mesh_colliders(small_batch):
    """One graph replay rebuilds every mesh's tree from the batch's vertex
    positions and traces all the rays (rrg_batch_rebuild_intersect_device):
    the same hit records, bit for bit, as the batch built at create (the
    same build on the same positions), on two replays; then, with every
    vertex moved (rrg_batch_set_vertices_device), the same records as
    colliders built on the moved meshes one by one."""
    import torch
    mb, counts, rays, off, off_d, b = small_batch
    n = rays.shape[0]
    base = run(b, rays, off_d, 32)
    hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    lc0 = col.launch_count()
    for _ in range(2):
        hits.fill_(7.0)
        b.rebuild_intersect_device(rays.data_ptr(), off_d.data_ptr(), n, hits.data_ptr())
        torch.cuda.synchronize()
        assert b.status() == 0
        np.testing.assert_array_equal(hits.cpu().numpy().view(np.uint32), base.view(np.uint32))
    assert col.launch_count() - lc0 > 2 * 40   # the replayed graphs hold the build's launches
    moved = np.ascontiguousarray(mb.vertices * np.float32(1.25) + np.float32([0.5, -0.25, 0.125]), np.float32)
    xyz = torch.from_numpy(moved).cuda()
    b.set_vertices_device(xyz.data_ptr())
    hits.fill_(7.0)
    b.rebuild_intersect_device(rays.data_ptr(), off_d.data_ptr(), n, hits.data_ptr())
    torch.cuda.synchronize()
    assert b.status() == 0
    h = hits.cpu().numpy()
    r = rays.cpu().numpy()
    checked = 0
    for m in range(mb.nmesh):
        a, e = int(off[m]), int(off[m + 1])
        if a == e or m == 5:
            continue
        v, t = mb.mesh(m)
        vm = moved[int(mb.vert_off[m]):int(mb.vert_off[m + 1])]
        c = col.RRCollider.create(vm, t)
        got = col.decode_hits(h[a:e])
        one = c.intersect_batch(r[a:e])
        for f in ("hit", "tri", "dist", "uv", "side"):
            np.testing.assert_array_equal(got[f], one[f], err_msg=f"mesh {m} field {f}")
        checked += e - a
        c.close()
    assert checked > 10000
    orig = torch.from_numpy(np.ascontiguousarray(mb.vertices, np.float32)).cuda()
    b.set_vertices_device(orig.data_ptr())
    torch.cuda.synchronize()
