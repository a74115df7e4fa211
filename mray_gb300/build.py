"""Compile the CUDA library libmray_gb300.so in-tree for sm_103a.

Translation units are compiled in parallel: CUDA sources with nvcc
(-gencode arch=compute_103a,code=sm_103a), host C++ with g++ and
-ffp-contract=off (the host restatement of MRay's Matrix3x4::Inverse must not
fuse operations the reference host build does not fuse).  The CUDA runtime is
linked statically so the library loads beside any PyTorch build.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmray_gb300.so")
SCENES_LIB = os.path.join(PKG, "libmrg_scenes.so")
INCLUDE = os.path.join(ROOT, "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdr.append(os.path.join(INCLUDE, "mray_gb300.h"))
    return cu, cpp, hdr


def _compile(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build_scenes(force=False, verbose=False):
    """Seeded scene / ray generators (plain C, no CUDA)."""
    src = os.path.join(CSRC, "scenes.c")
    if not force and os.path.exists(SCENES_LIB) and \
            os.path.getmtime(SCENES_LIB) >= max(os.path.getmtime(src), os.path.getmtime(__file__)):
        return SCENES_LIB
    tmp = SCENES_LIB + ".tmp%d" % os.getpid()
    _compile(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
              "-fno-fast-math", "-Wall", "-o", tmp, src, "-lm"], verbose)
    os.replace(tmp, SCENES_LIB)
    return SCENES_LIB


def build(force=False, verbose=False, ptxas_verbose=False, defines=None, lib_path=None,
          obj_dir=None):
    """Builds the library.  ``defines`` (e.g. ``{"MRG_TRACE_STEP_BUDGET": 8}``)
    override the kernels' compile-time tuning knobs; ``lib_path`` / ``obj_dir``
    place such a variant elsewhere (the default library is untouched)."""
    build_scenes(force=force, verbose=verbose)
    lib_out = lib_path or LIB
    obj = obj_dir or OBJ
    dflags = ["-D%s=%s" % (k, v) for k, v in sorted((defines or {}).items())]
    cu, cpp, hdr = _sources()
    srcs = [os.path.join(CSRC, f) for f in cu + cpp]
    newest = max(os.path.getmtime(p) for p in srcs + hdr + [__file__])
    if not force and os.path.exists(lib_out) and os.path.getmtime(lib_out) >= newest:
        return lib_out
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(obj, exist_ok=True)
    jobs = []
    for f in cu:
        o = os.path.join(obj, f + ".o")
        cmd = [nvcc] + GENCODE + dflags + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                  "-I", CSRC, "-I", INCLUDE, "-c", os.path.join(CSRC, f), "-o", o]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, o))
    for f in cpp:
        o = os.path.join(obj, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"] + dflags + [
               "-I", CSRC, "-I", INCLUDE, "-I", os.path.join(home, "include"),
               "-c", os.path.join(CSRC, f), "-o", o]
        jobs.append((cmd, o))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        futs = [ex.submit(_compile, cmd, verbose) for cmd, _ in jobs]
        for fu in futs:
            logs.append(fu.result())
    tmp = lib_out + ".tmp%d" % os.getpid()
    link = [nvcc] + GENCODE + ["-shared", "-cudart", "static", "-o", tmp] + [o for _, o in jobs]
    _compile(link, verbose)
    os.replace(tmp, lib_out)
    if ptxas_verbose:
        sys.stderr.write("".join(logs))
    return lib_out


if __name__ == "__main__":
    build(force=True, verbose=True, ptxas_verbose="-v" in sys.argv)
