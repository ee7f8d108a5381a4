"""The reference-side plugin (include/rrgpu_rrcollider_plugin.hpp) compiles
against the reference's headers, links with the reference library and
librrgpu.so, and goes through RRCollider::registerTechnique / create.  Runs
only where the reference sources and oracle/_ref exist (this is a build
check of the integration, not a GPU test)."""
import os
import subprocess

import pytest

from lightsprintsdk_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("RR_REFERENCE_DIR", "/root/reference")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libLightsprintCore.a")


@pytest.mark.skipif(not (os.path.isdir(os.path.join(REF, "include")) and os.path.exists(REF_LIB)),
                    reason="reference sources / oracle/_ref not present")
def test_plugin_builds_and_registers(tmp_path):
    lib = B.build()
    exe = tmp_path / "plugin_check"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DRR_BUILD", "-w", "-include", "string", "-include", "climits",
           f"-I{REF}/include", f"-I{ROOT}/include", os.path.join(ROOT, "tests", "cpp", "plugin_check.cpp"),
           "-o", str(exe), REF_LIB, lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-lgomp", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, check=True).stdout
    # a GPU gives technique 100; without one the reference falls back to IT_LINEAR (0)
    assert "hit=1 tri=1 dist=1 u=0.35 v=0.3 front=0" in out, out
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    assert ("technique=100" in out) == has_gpu, out
