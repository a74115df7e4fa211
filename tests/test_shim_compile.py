"""The MRay-side classes compiled against the MRay tree's own headers (host
backend, with the oracle build's shims):
- mray_gb300/shim/AcceleratorGB300.h, a BaseAcceleratorI over the C ABI
  (Source/Tracer/AcceleratorC.h and the groups it reads); its static_asserts
  check that RayGMem, HitKeyPack and MetaHit have the layouts the C ABI
  declares, and emitting the vtable compiles every override;
- mray_gb300/shim/TracerGB300.h, a TracerI (Source/Core/TracerI.h) over the
  tracer C ABI with MRay's ConstructTracer / DestroyTracer entry points,
  compiled, linked with MRay's TransientPool and error sources and run by
  tests/tracer_mray_client.cpp up to the surface commit.
Skips where the MRay tree is absent."""
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


def _mray_flags():
    src = build.reference_source_dir()
    fmt = build._fmt_include()
    if src is None or fmt is None:
        pytest.skip("the MRay source tree (and fmt headers) are not present")
    build.build_ref_pt()                      # writes the prelude and mray_cmake.h
    gen = os.path.join(build.REF_DIR, "gen")
    return src, ["g++", "-std=c++20", "-O1", "-fPIC", "-DMRAY_GCC", "-DMRAY_LINUX", "-DMRAY_GPU_BACKEND_CPU",
                 "-DFMT_HEADER_ONLY", "-DNDEBUG", "-Wno-interference-size",
                 "-include", os.path.join(gen, "pack_element_prelude.h"), "-I", gen, "-I", src,
                 "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "mray_gb300", "shim"), "-isystem", fmt]


def test_tracer_adapter_compiles_against_mray(tmp_path):
    src, flags = _mray_flags()
    use = tmp_path / "use_tracer.cpp"
    use.write_text('#define MRAY_GB300_TRACER_ENTRYPOINTS\n#include "TracerGB300.h"\n')
    obj = tmp_path / "use_tracer.o"
    r = subprocess.run(flags + ["-c", str(use), "-o", str(obj)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    nm = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True, check=True).stdout
    assert "vtable for TracerGB300" in nm
    for sym in ("ConstructTracer", "DestroyTracer"):
        assert " T " + sym in nm, sym


def test_tracer_adapter_runs_with_mray_types(tmp_path, cuda_lib):
    """MRay's TransientData and MRayError through TracerGB300 over the real
    library, up to the surface commit."""
    import torch
    src, flags = _mray_flags()
    exe = str(tmp_path / "tracer_mray_client")
    r = subprocess.run(flags + [os.path.join(ROOT, "tests", "tracer_mray_client.cpp"),
                                os.path.join(src, "TransientPool", "TransientPool.cpp"),
                                os.path.join(src, "Core", "Error.cpp"), os.path.join(src, "Core", "Log.cpp"),
                                cuda_lib, "-Wl,-rpath," + os.path.dirname(cuda_lib), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "0 failures" in run.stdout
    if not torch.cuda.is_available():
        assert "commit: error" in run.stdout
