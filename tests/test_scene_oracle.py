"""CPU checks of the scene oracle (oracle/orc.py scene_collide): identity
objects reduce to the single-mesh oracle, a translated and uniformly scaled
copy gives the world-space answer, a mirrored object flips hitFrontSide;
the scene C ABI rejects bad arguments before any device work."""
import ctypes as C

import numpy as np

from lightsprintsdk_gb300 import scene as rs
from lightsprintsdk_gb300 import scenes
from oracle import orc


def sphere():
    v, t = scenes.displaced_icosphere(12, 3)
    return v.astype(np.float32), t.astype(np.uint32)


def test_identity_object_equals_single_mesh_oracle():
    v, t = sphere()
    rays = scenes.shell_rays(4096)
    world = np.zeros((1, 3, 4), np.float32)
    world[0, :, :3] = np.eye(3)
    h, o = orc.scene_collide([(v, t)], [0], world, rays)
    ref = orc.FastestOracle(v, t).collide(rays, 0)
    for f in ("hit", "tri", "side"):
        np.testing.assert_array_equal(h[f], ref[f], err_msg=f)
    # the object-space direction is renormalised (RRColliderMulti.cpp:127),
    # which moves float-normalised directions by an ulp
    np.testing.assert_allclose(h["dist"], ref["dist"], rtol=1e-6)
    np.testing.assert_allclose(h["uv"], ref["uv"], atol=1e-5)
    assert (o[h["hit"]] == 0).all() and (o[~h["hit"]] == 0xFFFFFFFF).all()


def test_scaled_copy_matches_world_space_mesh():
    """A power-of-two scale keeps every coordinate exact, so the
    object-space answer is the world-space mesh's, with the distance
    divided back by the scale."""
    v, t = sphere()
    rays = scenes.shell_rays(4096, radius=2.0)
    world = np.zeros((1, 3, 4), np.float32)
    world[0, :, :3] = 2.0 * np.eye(3)
    h, o = orc.scene_collide([(v, t)], [0], world, rays)
    ref = orc.FastestOracle(v * np.float32(2.0), t).collide(rays, 0)
    np.testing.assert_array_equal(h["hit"], ref["hit"])
    np.testing.assert_array_equal(h["tri"], ref["tri"])
    np.testing.assert_allclose(h["dist"], ref["dist"], rtol=1e-6)


def test_mirrored_object_flips_front_side():
    v, t = sphere()
    rays = scenes.shell_rays(2048)
    w = np.zeros((2, 3, 4), np.float32)
    w[0, :, :3] = np.eye(3)
    w[1, :, :3] = np.diag([-1.0, 1.0, 1.0])
    a, _ = orc.scene_collide([(v, t)], [0], w[:1], rays)
    b, _ = orc.scene_collide([(v, t)], [0], w[1:], rays)
    # outside rays hit front faces of the plain sphere; the mirror image's
    # world winding is reversed, so they hit its back sides
    # (IntersectLinear.cpp:309-317 flips the object-space answer)
    assert a["side"][a["hit"]].mean() > 0.99 and b["side"][b["hit"]].mean() < 0.01


def test_scene_arguments_rejected_before_any_device_work():
    L = rs._lib()
    out = C.c_void_p()
    m = np.zeros(3, np.uint32)
    w = np.zeros(36, np.float32)
    assert L.rrg_scene_create(None, 3, m.ctypes.data, w.ctypes.data, C.byref(out)) == 1
    assert L.rrg_scene_intersect_device(None, None, 1, None, None, None) == 1
    assert L.rrg_scene_set_matrices(None, w.ctypes.data) == 1
