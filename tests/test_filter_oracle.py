"""The lightmap oracle's texel enumeration, TexelFlags and post-filters
(oracle/rr_gather.c, oracle/rr_filter.c) against the reference's own code,
run from its sources by tests/golden/make_golden.py (enumerateTexelsPartial,
RRBuffer::lightmapSmooth / lightmapGrowForBilinearInterpolation /
lightmapGrow / lightmapFillBackground): bit-exact, through the hashes stored
in tests/golden/lightmap_ref.npz."""
import numpy as np
import pytest

from oracle import orc
from tests.golden import make_golden as G
from tests.helpers import md5

FIX = np.load(__file__.replace("test_filter_oracle.py", "golden/lightmap_ref.npz"))


@pytest.mark.parametrize("k", range(len(G.LIGHTMAP_CASES)))
def test_enumeration_and_flags_match_reference(k):
    freq, size = G.LIGHTMAP_CASES[k]
    v, nrm, t, uv = G.lightmap_case(freq, size)
    assert md5(v, nrm, t, uv) == str(FIX[f"case{k}_mesh_md5"])
    flags = orc.texel_flags(uv, size)
    np.testing.assert_array_equal(flags, FIX[f"case{k}_flags"])
    off, st = orc.enumerate_atlas(uv, np.arange(len(t)), size)
    np.testing.assert_array_equal(np.diff(off).astype(np.uint32), FIX[f"case{k}_counts"])
    assert md5(st["tri"], st["uv"], st["area"]) == str(FIX[f"case{k}_st_md5"])


RUNS = [(0, r) for r in G.FILTER_RUNS] + [(1, r) for r in G.FILTER_RUNS_ODD]


@pytest.mark.parametrize("k,run", RUNS)
def test_filters_match_reference(k, run):
    stages, wrap, seams = run
    freq, size = G.LIGHTMAP_CASES[k]
    v, nrm, t, uv = G.lightmap_case(freq, size)
    img = G.lightmap_image(FIX[f"case{k}_flags"], size)
    assert md5(img) == str(FIX[f"case{k}_img_md5"])
    sm = orc.unwrap_seams(t, uv) if seams else None
    out = orc.lightmap_filter(img, 1.0, 1000, (0, 0, 0, 0), bool(wrap), sm, stages)
    if (k, run) == (0, (15, 0, 1)):
        np.testing.assert_array_equal(out, FIX["filter_all_seams"])
    assert md5(out) == str(FIX[f"case{k}_filter_{stages}_{wrap}_{seams}_md5"]), run


def test_unwrap_seams_small_cases():
    """Two triangles sharing edge 1-2: a seam only where their unwrap of the
    edge differs; edge1 in the first triangle's vertex order, edge2 the same
    vertices' uv in the second triangle."""
    t = np.array([[0, 1, 2], [2, 1, 3]], np.uint32)
    same = np.array([[[0, 0], [0.5, 0], [0, 0.5]], [[0, 0.5], [0.5, 0], [0.5, 0.5]]], np.float32)
    assert len(orc.unwrap_seams(t, same)) == 0
    moved = same.copy()
    moved[1] += 0.25
    s = orc.unwrap_seams(t, moved)
    assert s.shape == (1, 8)
    np.testing.assert_array_equal(s[0], [0.5, 0, 0, 0.5, 0.75, 0.25, 0.25, 0.75])


def test_filter_edge_cases():
    """smoothing 0 and fill with an empty lightmap; a single used texel grows
    over the whole map with alpha 0.001 where it was empty."""
    z = np.zeros((8, 8, 4), np.float32)
    out = orc.lightmap_filter(z, 0.0, 1000, (0.1, 0.2, 0.3, 0.4), False, None, 15)
    np.testing.assert_array_equal(out.reshape(-1, 4), np.tile(np.float32([0.1, 0.2, 0.3, 0.4]), (64, 1)))
    one = z.copy()
    one[3, 4] = [1.0, 2.0, 3.0, 1.0]
    g = orc.lightmap_filter(one, 0.0, 1000, (0, 0, 0, 0), False, None, orc.FILTER_GROW)
    np.testing.assert_allclose(g[..., :3].reshape(-1, 3), np.tile([1.0, 2.0, 3.0], (64, 1)), rtol=1e-6)
    assert g[3, 4, 3] == 1.0 and np.all(np.delete(g[..., 3].reshape(-1), 3 * 8 + 4) == np.float32(0.001))
