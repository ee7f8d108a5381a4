"""GPU lightmap post-filters (rrg_lightmap_filter) and TexelFlags.

1. On the golden sphere atlas: the GPU enumeration's flags equal the
   reference's enumerateTexelsPartial, and every filter run's output hashes
   equal the reference's RRBuffer filters (tests/golden/lightmap_ref.npz):
   GPU against the reference itself, bit-exact.
2. On the config-2 interior (several atlases per call, an offset first
   atlas): gathered lightmaps filtered on the GPU equal the oracle's filters
   applied atlas by atlas, bit-exact.
3. On a 400 x 400 sphere atlas, whose used flags exceed the seam kernel's
   shared memory: the same against the oracle."""
import numpy as np
import pytest

from lightsprintsdk_gb300 import collider as col
from lightsprintsdk_gb300 import lightmap as lm
from lightsprintsdk_gb300 import scenes
from oracle import orc
from tests.golden import make_golden as G
from tests.helpers import md5

pytestmark = pytest.mark.gpu

FIX = np.load(__file__.replace("test_filter_gpu.py", "golden/lightmap_ref.npz"))


_SPHERES = {}


def sphere(k):
    """Collider and lightmapper of golden case k (built once per module)."""
    if k not in _SPHERES:
        freq, size = G.LIGHTMAP_CASES[k]
        v, nrm, t, uv = G.lightmap_case(freq, size)
        c = col.RRCollider.create(v, t)
        L = lm.RRLightmapper(c, np.full((len(t), 3), 0.5, np.float32), np.zeros(len(t), np.int32), uv, 1, size)
        _SPHERES[k] = (c, L, size, len(t))
    return _SPHERES[k]


@pytest.mark.parametrize("k", range(len(G.LIGHTMAP_CASES)))
def test_sphere_flags_match_reference(k):
    c, L, size, nt = sphere(k)
    np.testing.assert_array_equal(L.flags(), FIX[f"case{k}_flags"])


@pytest.mark.parametrize("k,run", [(0, r) for r in G.FILTER_RUNS] + [(1, r) for r in G.FILTER_RUNS_ODD])
def test_sphere_filters_match_reference(k, run):
    import torch
    c, L, size, nt = sphere(k)
    stages, wrap, seams = run
    img = G.lightmap_image(FIX[f"case{k}_flags"], size)
    d = torch.from_numpy(img.reshape(-1, 4).copy()).cuda()
    L.filter_device(lm.filter_params(wrap=bool(wrap), seams=bool(seams), stages=stages), 0, 1, d.data_ptr())
    torch.cuda.synchronize()
    out = d.cpu().numpy().reshape(size, size, 4)
    if (k, run) == (0, (15, 0, 1)):
        np.testing.assert_array_equal(out, FIX["filter_all_seams"])
    assert md5(out) == str(FIX[f"case{k}_filter_{stages}_{wrap}_{seams}_md5"]), run
    if seams:
        assert L.nseams == nt * 3 // 2


@pytest.fixture(scope="module")
def interior():
    gs = scenes.gather_c2()
    c = col.RRCollider.create(gs.scene.vertices, gs.scene.indices)
    L = lm.RRLightmapper.from_scene(c, gs)
    return gs, c, L


@pytest.mark.parametrize("first,count,wrap", [(0, 4, False), (9, 3, True), (200, 2, False)])
def test_interior_filters_match_oracle(interior, first, count, wrap):
    import torch
    gs, c, L = interior
    S = gs.size * gs.size
    params = lm.make_params(gs.lights, quality=4, max_depth=2)
    buf = torch.zeros((gs.natlas * S, 4), dtype=torch.float32, device="cuda")
    L.gather_device(params, first * S, count * S, buf[first * S:].data_ptr())
    torch.cuda.synchronize()
    before = buf.cpu().numpy()
    L.filter_device(lm.filter_params(wrap=wrap), first, count, buf.data_ptr())
    torch.cuda.synchronize()
    after = buf.cpu().numpy()
    # atlases outside the call are untouched
    np.testing.assert_array_equal(after[:first * S], before[:first * S])
    np.testing.assert_array_equal(after[(first + count) * S:], before[(first + count) * S:])
    idx = np.asarray(gs.scene.indices, np.uint32)
    for a in range(first, first + count):
        ids = np.nonzero(gs.tri_atlas == a)[0]
        seams = orc.unwrap_seams(idx[ids], gs.uv[ids])
        img = before[a * S:(a + 1) * S].reshape(gs.size, gs.size, 4)
        want = orc.lightmap_filter(img, 1.0, 1000, (0, 0, 0, 0), wrap, seams, 15)
        got = after[a * S:(a + 1) * S].reshape(gs.size, gs.size, 4)
        bad = np.nonzero((got != want).any(-1).reshape(-1))[0]
        assert bad.size == 0, (a, bad[:10], got.reshape(-1, 4)[bad[:3]], want.reshape(-1, 4)[bad[:3]])


def test_large_atlas_seams_match_oracle():
    """Above 362^2 texels the seam kernel keeps the atlas's used flags in
    global memory and finds a seam's own earlier writes in its log instead of
    by per-texel flags: all filters with seams, bit-exact against the oracle."""
    import torch
    size = 400
    v, nrm, t, uv = G.lightmap_case(4, size)
    c = col.RRCollider.create(v, t)
    L = lm.RRLightmapper(c, np.full((len(t), 3), 0.5, np.float32), np.zeros(len(t), np.int32), uv, 1, size)
    img = G.lightmap_image(L.flags(), size, seed=11)
    d = torch.from_numpy(img.reshape(-1, 4).copy()).cuda()
    L.filter_device(lm.filter_params(), 0, 1, d.data_ptr())
    torch.cuda.synchronize()
    got = d.cpu().numpy().reshape(size, size, 4)
    want = orc.lightmap_filter(img, 1.0, 1000, (0, 0, 0, 0), False, orc.unwrap_seams(t, uv), 15)
    bad = np.nonzero((got != want).any(-1).reshape(-1))[0]
    assert bad.size == 0, (bad[:10], got.reshape(-1, 4)[bad[:3]], want.reshape(-1, 4)[bad[:3]])
