"""Build recipe for the CPU oracle (test infrastructure only).

- ``build_oracle()`` compiles the project's C restatement (mrg_oracle.c and
  the path-tracer restatement) into ``oracle/_build/libmrg_oracle.so``.
- ``build_ref()`` compiles ``ref_core_driver.cpp`` against the MRay source tree
  (its own ``Source/Core`` headers, unmodified) into
  ``oracle/_ref/libmray_ref_core.so``.  It runs only where the MRay source tree
  is present (``MRAY_REFERENCE_SRC`` or the default checkout path); elsewhere it
  is a no-op and tests that need it skip.

Both are compiled with ``-ffp-contract=off`` so that only the explicit fma()
calls of the restated algorithms are fused, matching the reference host build
(MRAY_HOST_ARCH_BASIC, no automatic contraction).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD_DIR, "libmrg_oracle.so")
REF_LIB = os.path.join(REF_DIR, "libmray_ref_core.so")

ORACLE_SOURCES = ["mrg_oracle.c", "pt_oracle.c", "zsobol_oracle.c"]


def reference_source_dir():
    d = os.environ.get("MRAY_REFERENCE_SRC", "/root/reference/Source")
    return d if os.path.isdir(os.path.join(d, "Core")) else None


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, h) for h in os.listdir(HERE) if h.endswith(".h")]
    if not force and _newer(ORACLE_LIB, deps):
        return ORACLE_LIB
    tmp = ORACLE_LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", "-Wall", "-Wno-unused-function",
           "-o", tmp] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref(force=False, verbose=False):
    src_dir = reference_source_dir()
    if src_dir is None:
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    drv = os.path.join(HERE, "ref_core_driver.cpp")
    if not force and _newer(REF_LIB, [drv]):
        return REF_LIB
    tmp = REF_LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-DMRAY_GCC", "-DMRAY_LINUX", "-I", src_dir, "-o", tmp, drv]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_LIB)
    return REF_LIB


def _mray_cmake_header(gen_dir):
    """The configure_file output the MRay sources include (mray_cmake.h.in),
    with fixed values: this recipe does not run CMake."""
    os.makedirs(gen_dir, exist_ok=True)
    h = os.path.join(gen_dir, "mray_cmake.h")
    if not os.path.exists(h):
        with open(h, "w") as f:
            f.write("#pragma once\n#include <string_view>\nusing namespace std::string_view_literals;\n"
                    "#define MRAY_VERSION_MAJOR 1\n#define MRAY_VERSION_MINOR 0\n#define MRAY_VERSION_PATCH 0\n"
                    "#define MRAY_BUILD_VISOR 0\n#define MRAY_HOST_ARCH_BASIC\n"
                    "#define MRAY_PROJECT_NAME \"MRay\"sv\n#define MRAY_PROJECT_DESCRIPTION \"\"sv\n"
                    "#define MRAY_PLATFORM_NAME \"Linux\"sv\n#define MRAY_COMPILER_NAME \"gcc\"sv\n"
                    "#define MRAY_GPU_PLATFORM_NAME \"none\"sv\n#define MRAY_GPU_COMPILER_NAME \"none\"sv\n")
    return gen_dir


def build_ref_spectra(force=False, verbose=False):
    """The reference's spectral tools, compiled from the MRay tree: the LUT
    generator (SpectraLUTGen/main.cpp) as ``oracle/_ref/spectra_lut_gen`` and
    the colour-table accessors (spectra_driver.cpp) as
    ``oracle/_ref/libmray_ref_spectra.so``.  Returns (generator, library) or
    None without the MRay tree."""
    src_dir = reference_source_dir()
    if src_dir is None:
        return None
    gen = _mray_cmake_header(os.path.join(REF_DIR, "gen"))
    color = os.path.join(src_dir, "Core", "ColorFunctions.cpp")
    flags = ["-std=c++20", "-O2", "-ffp-contract=off", "-DMRAY_GCC", "-DMRAY_LINUX", "-I", gen, "-I", src_dir]
    exe = os.path.join(REF_DIR, "spectra_lut_gen")
    lib = os.path.join(REF_DIR, "libmray_ref_spectra.so")
    drv = os.path.join(HERE, "spectra_driver.cpp")
    if force or not os.path.exists(exe):
        cmd = ["g++"] + flags + ["-pthread", "-o", exe, os.path.join(src_dir, "SpectraLUTGen", "main.cpp"), color]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    if force or not _newer(lib, [drv]):
        cmd = ["g++"] + flags + ["-fPIC", "-shared", "-o", lib, drv, color]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    return exe, lib


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
    print(build_ref(force=True, verbose=True))
