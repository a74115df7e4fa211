"""Build recipe for the CPU oracle (test infrastructure only).

- ``build_oracle()`` compiles the project's C restatement (mrg_oracle.c and
  the path-tracer restatement) into ``oracle/_build/libmrg_oracle.so``.
- ``build_ref()`` compiles ``ref_core_driver.cpp`` against the MRay source tree
  (its own ``Source/Core`` headers, unmodified) into
  ``oracle/_ref/libmray_ref_core.so``.  It runs only where the MRay source tree
  is present (``MRAY_REFERENCE_SRC``, or a checkout named ``reference`` beside
  the repository); elsewhere it is a no-op and tests that need it skip.

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

ORACLE_SOURCES = ["mrg_oracle.c", "pt_oracle.c", "zsobol_oracle.c", "guide_oracle.c"]


def reference_source_dir():
    """The MRay ``Source`` directory: ``MRAY_REFERENCE_SRC`` when set, else a
    checkout named ``reference`` beside this repository's root."""
    d = os.environ.get("MRAY_REFERENCE_SRC") or os.path.join(os.path.dirname(HERE), os.pardir, "reference", "Source")
    d = os.path.normpath(d)
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


def ref_lut(res=64):
    """MR_SPECTRA LUT for Rec.709 at resolution `res`, written by MRay's own
    SpectraLUTGen into ``oracle/_ref/lut<res>/REC_709.mrspectra`` (about
    9 MB at 64, the converter's compile-time resolution; not committed).
    None without the MRay tree."""
    tools = build_ref_spectra()
    if tools is None:
        return None
    out_dir = os.path.join(REF_DIR, "lut%d" % res)
    path = os.path.join(out_dir, "REC_709.mrspectra")
    if os.path.exists(path):
        return path
    # the generator fails when it has to create the folder itself
    # (SpectraLUTGen/main.cpp:570 treats "created" as an error)
    os.makedirs(out_dir, exist_ok=True)
    subprocess.run([tools[0], str(res), "REC_709", out_dir], check=True, capture_output=True)
    return path


# g++ 13 has no __type_pack_element builtin, and MRay's fallback
# (Core/TypePack.h:66-75) names a PackElementDetail::TypePackElementT that the
# tree does not define.  This header, force-included ahead of every source,
# defines it; no file of the MRay tree is copied or changed.
_PACK_ELEMENT_PRELUDE = """#pragma once
#include <cstddef>
namespace PackElementDetail
{
template<std::size_t I, class T0, class... Ts>
struct TypePackElementT { using Type = typename TypePackElementT<I - 1, Ts...>::Type; };
template<class T0, class... Ts>
struct TypePackElementT<0, T0, Ts...> { using Type = T0; };
}
"""

REF_PT_LIB = os.path.join(REF_DIR, "libmray_ref_pt.so")


def _fmt_include():
    """fmt headers for MRay's logging (the reference pins fmt v10, header-only
    use); torch ships a copy in its include directory."""
    try:
        import torch
        d = os.path.join(os.path.dirname(torch.__file__), "include")
    except ImportError:
        return None
    return d if os.path.exists(os.path.join(d, "fmt", "format.h")) else None


def build_ref_pt(force=False, verbose=False):
    """MRay's host-backend path-tracer building blocks (materials, lights,
    light sampler, camera, film filter, distributions, spectral converter)
    compiled from the MRay tree with the driver ``ref_pt_driver.cpp`` into
    ``oracle/_ref/libmray_ref_pt.so``.  Returns None without the MRay tree or
    the fmt headers."""
    src_dir = reference_source_dir()
    fmt = _fmt_include()
    if src_dir is None or fmt is None:
        return None
    gen = _mray_cmake_header(os.path.join(REF_DIR, "gen"))
    prelude = os.path.join(gen, "pack_element_prelude.h")
    if not os.path.exists(prelude) or open(prelude).read() != _PACK_ELEMENT_PRELUDE:
        with open(prelude, "w") as f:
            f.write(_PACK_ELEMENT_PRELUDE)
    drv = os.path.join(HERE, "ref_pt_driver.cpp")
    if not force and _newer(REF_PT_LIB, [drv, __file__]):
        return REF_PT_LIB
    tmp = REF_PT_LIB + ".tmp%d" % os.getpid()
    obj = tmp + ".o"
    # MRAY_HOST_ARCH_BASIC (no automatic FMA contraction) as in the
    # reference's host build; FTZ/DAZ is not set (no intermediate here is
    # subnormal)
    # NDEBUG as in MRay's release builds: the reference's asserts are off
    flags = ["g++", "-std=c++20", "-O2", "-fPIC", "-c", "-ffp-contract=off", "-Wno-interference-size", "-DNDEBUG",
             "-DMRAY_GCC", "-DMRAY_LINUX", "-DMRAY_GPU_BACKEND_CPU", "-DFMT_HEADER_ONLY",
             "-include", prelude, "-I", gen, "-I", src_dir, "-isystem", fmt]
    color_obj = tmp + ".color.o"
    for src, o in ((drv, obj), (os.path.join(src_dir, "Core", "ColorFunctions.cpp"), color_obj)):
        cmd = flags + ["-o", o, src]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    # The headers declare MRay's group classes (virtual bookkeeping whose
    # definitions live in the Device layer).  The driver never reaches them,
    # so their references are made weak instead of linking that layer: a
    # first link lists the unresolved, unversioned symbols, objcopy weakens
    # exactly those, and the second link yields a loadable library.
    subprocess.run(["g++", "-shared", "-o", tmp, obj, color_obj], check=True)
    nm = subprocess.run(["nm", "-D", "--undefined-only", tmp], check=True, capture_output=True, text=True)
    weak = [ln.split()[-1] for ln in nm.stdout.splitlines()
            if ln.strip() and "@" not in ln and not ln.split()[-1].startswith(("_ITM", "__gmon", "_Jv"))]
    lst = tmp + ".weak"
    with open(lst, "w") as f:
        f.write("\n".join(weak) + "\n")
    subprocess.run(["objcopy", "--weaken-symbols=" + lst, obj], check=True)
    subprocess.run(["g++", "-shared", "-o", tmp, obj, color_obj], check=True)
    for p in (obj, color_obj, lst):
        os.remove(p)
    os.replace(tmp, REF_PT_LIB)
    return REF_PT_LIB


if __name__ == "__main__":
    print(build_oracle(force=True, verbose=True))
    print(build_ref(force=True, verbose=True))
    print(build_ref_pt(force=True, verbose=True))
