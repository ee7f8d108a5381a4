"""The reference-side plugin (include/rrgpu_rrcollider_plugin.hpp) compiles
against the reference's headers (staged in oracle/_ref/src), links with the
reference library (oracle/_ref) and librrgpu.so, and goes through
RRCollider::registerTechnique / create.  Without a GPU the GPU builder
returns nullptr and the reference falls back to IT_LINEAR
(RRCollider/RRCollider.cpp:236-239); tests/test_plugin_gpu.py runs the same
program on a GPU."""
import pytest

from tests import plugin_harness as H


@pytest.mark.skipif(not H.available(), reason="reference library (oracle/_ref) not built")
def test_plugin_builds_and_registers(tmp_path):
    exe = H.build(tmp_path)
    out = H.hello(exe)
    assert "hit=1 tri=1 dist=1 u=0.35 v=0.3 front=0" in out, out
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    assert ("technique=100" in out) == has_gpu, out
