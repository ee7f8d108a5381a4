"""Two-level scene collider (include/rrgpu_scene.h) on the GPU: the
config-1 interior as instanced objects (one static mesh + 64 instances of
one sphere) against the RRColliderMulti oracle (object-space rays in the
reference's float arithmetic, FASTEST per object), against the flattened
scene, and under moved, mirrored and disabled objects."""
import numpy as np
import pytest

from lightsprintsdk_gb300 import batch as rb
from lightsprintsdk_gb300 import scene as rs
from lightsprintsdk_gb300 import scenes
from oracle import orc

pytestmark = pytest.mark.gpu


def split_interior(sc):
    """(static mesh, sphere mesh, object meshes, world matrices, flattened
    triangle base of each object)."""
    inst = set(int(i) for i in sc.instance_object_ids)
    static_tri = np.nonzero(~np.isin(sc.tri_object, list(inst)))[0]
    used, inv = np.unique(sc.indices[static_tri].ravel(), return_inverse=True)
    sv = sc.vertices[used]
    st = inv.reshape(-1, 3).astype(np.uint32)
    lv, lt = sc.sphere_local
    nobj = 1 + len(sc.instance_object_ids)
    world = np.zeros((nobj, 3, 4), np.float32)
    world[0, :, :3] = np.eye(3)
    world[1:] = sc.instance_matrices
    obj_mesh = np.array([0] + [1] * (nobj - 1), np.uint32)
    return (sv, st), (lv, lt), obj_mesh, world, static_tri


@pytest.fixture(scope="module")
def interior():
    sc = scenes.interior_c1()
    static, sphere, obj_mesh, world, static_tri = split_interior(sc)
    verts = np.concatenate([static[0], sphere[0]])
    idx = np.concatenate([static[1], sphere[1]])
    vo = np.array([0, static[0].shape[0], verts.shape[0]], np.uint32)
    to = np.array([0, static[1].shape[0], idx.shape[0]], np.uint32)
    b = rb.RRColliderBatch.create(verts, idx, vo, to)
    rays = np.concatenate([scenes.camera_rays(rows=16, cols=list(range(0, 4096, 32))),
                           scenes.surface_rays(sc.vertices, sc.indices, 1 << 16)])
    return sc, (static, sphere), obj_mesh, world, static_tri, b, rays


def compare(h, o, ref, ro, n):
    """Same hit set and object/triangle except for rare near-ties; where both
    agree on (object, triangle) the fields are bit-identical."""
    same = h["hit"] & ref["hit"] & (o == ro) & (h["tri"] == ref["tri"])
    differ = (h["hit"] != ref["hit"]) | (h["hit"] & ~same)
    assert differ.sum() <= max(2, 1e-4 * n), differ.sum()
    for f in ("dist", "uv", "side"):
        np.testing.assert_array_equal(h[f][same], ref[f][same], err_msg=f)
    return same


def test_instanced_interior_against_oracle(interior):
    sc, meshes, obj_mesh, world, static_tri, b, rays = interior
    s = rs.RRScene(b, obj_mesh, world)
    h, o = s.intersect(rays)
    ref, ro = orc.scene_collide(meshes, obj_mesh, world, rays)
    same = compare(h, o, ref, ro, len(rays))
    assert same.sum() > 0.5 * len(rays)
    assert (o[same] > 0).sum() > 1000          # instances are hit, not only the room


def test_instanced_matches_flattened_scene(interior):
    """Against the flattened collider of the same scene (world-space
    vertices rounded once more): same object and triangle for almost every
    ray, distances within 1e-4 relative."""
    from lightsprintsdk_gb300 import collider as col
    sc, meshes, obj_mesh, world, static_tri, b, rays = interior
    s = rs.RRScene(b, obj_mesh, world)
    h, o = s.intersect(rays)
    flat = col.RRCollider.create(sc.vertices, sc.indices).intersect_batch(rays)
    first = sc.object_first_tri
    mapped = np.full(len(rays), 0xFFFFFFFF, np.int64)
    hit0 = h["hit"] & (o == 0)
    mapped[hit0] = static_tri[h["tri"][hit0]]
    for i, oid in enumerate(sc.instance_object_ids):
        m = h["hit"] & (o == i + 1)
        mapped[m] = first[oid] + h["tri"][m].astype(np.int64)
    agree = (h["hit"] == flat["hit"]) & (~h["hit"] | (mapped == flat["tri"]))
    assert agree.mean() >= 0.999, agree.mean()
    both = h["hit"] & flat["hit"] & (mapped == flat["tri"])
    rel = np.abs(h["dist"][both] - flat["dist"][both]) / np.maximum(flat["dist"][both], 1e-6)
    assert np.quantile(rel, 0.999) < 1e-4


def test_moved_mirrored_and_disabled_objects(interior):
    sc, meshes, obj_mesh, world, static_tri, b, rays = interior
    s = rs.RRScene(b, obj_mesh, world)
    w2 = world.copy()
    w2[1::2, :, 3] += np.array([0.3, -0.2, 0.5], np.float32)     # move every other sphere
    w2[2::4, 0, :3] *= -1.0                                         # mirror some (negative determinant)
    s.set_matrices(w2)
    h, o = s.intersect(rays)
    ref, ro = orc.scene_collide(meshes, obj_mesh, w2, rays)
    compare(h, o, ref, ro, len(rays))
    en = np.ones(len(obj_mesh), np.uint8)
    en[1::3] = 0
    s.set_enabled(en)
    h, o = s.intersect(rays)
    assert not np.isin(o[h["hit"]], np.nonzero(en == 0)[0]).any()
    keep = np.nonzero(en)[0]
    ref, ro = orc.scene_collide(meshes, obj_mesh[keep], w2[keep], rays)
    ro = np.where(ro == 0xFFFFFFFF, ro, keep[np.minimum(ro, len(keep) - 1)]).astype(np.uint32)
    compare(h, o, ref, ro, len(rays))


def test_singular_matrix_is_rejected(interior):
    from lightsprintsdk_gb300 import collider as col
    sc, meshes, obj_mesh, world, static_tri, b, rays = interior
    w = world.copy()
    w[3, :, :3] = 0.0
    with pytest.raises(col.RRGError) as e:
        rs.RRScene(b, obj_mesh, w)
    assert e.value.status == 1
