"""The MRay-side adapter (mray_gb300/shim/AcceleratorGB300.h, a
BaseAcceleratorI over the C ABI) compiled against the MRay tree's own headers
(Source/Tracer/AcceleratorC.h and the groups it reads), host backend, with the
oracle build's shims.  Its static_asserts check that RayGMem, HitKeyPack and
MetaHit have the layouts the C ABI declares; emitting the vtable compiles
every override.  Skips where the MRay tree is absent."""
import os
import subprocess

import pytest

from oracle import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_accelerator_adapter_compiles_against_mray(tmp_path):
    src = build.reference_source_dir()
    fmt = build._fmt_include()
    if src is None or fmt is None:
        pytest.skip("the MRay source tree (and fmt headers) are not present")
    build.build_ref_pt()                      # writes the prelude and mray_cmake.h
    gen = os.path.join(build.REF_DIR, "gen")
    use = tmp_path / "use.cpp"
    use.write_text('#include "AcceleratorGB300.h"\n#include "Device/CPU/GPUSystemCPU.hpp"\n'
                   "BaseAcceleratorI* make_gb300() { return new BaseAcceleratorGB300(0); }\n")
    obj = tmp_path / "use.o"
    cmd = ["g++", "-std=c++20", "-O1", "-c", "-fPIC", "-DMRAY_GCC", "-DMRAY_LINUX", "-DMRAY_GPU_BACKEND_CPU",
           "-DFMT_HEADER_ONLY", "-DNDEBUG", "-Wno-interference-size",
           "-include", os.path.join(gen, "pack_element_prelude.h"), "-I", gen, "-I", src,
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "mray_gb300", "shim"),
           "-isystem", fmt, str(use), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    nm = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True, check=True).stdout
    assert "vtable for BaseAcceleratorGB300" in nm
    for method in ("CastRays", "CastVisibilityRays", "CastLocalRays", "Construct", "SceneAABB"):
        assert "BaseAcceleratorGB300::" + method in nm, method
