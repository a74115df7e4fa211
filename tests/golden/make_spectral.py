"""Writes the spectral fixtures from the MRay tree's own tools (run where the
MRay source tree is present; the outputs are committed):

  REC_709_r32.mrspectra   Jakob-Hanika RGB -> spectrum coefficient LUT at
                          resolution 32, written by MRay's SpectraLUTGen
                          (Source/SpectraLUTGen/main.cpp) in its own
                          MR_SPECTRA format
  spectral_rec709.npz     CIE 1931 observer (471 x 3, 360-830 nm), its
                          integrals, the Rec.709 standard illuminant SPD (D65)
                          and its normalisation factor, RGB <-> XYZ matrices,
                          read through oracle/spectra_driver.cpp from
                          Source/Core/ColorFunctions.{h,cpp}

Usage: python tests/golden/make_spectral.py
"""
import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build  # noqa: E402

RES = 32


def main():
    tools = build.build_ref_spectra()
    if tools is None:
        sys.exit("the MRay source tree is needed (MRAY_REFERENCE_SRC)")
    exe, lib = tools
    out_dir = os.path.join(build.REF_DIR, "lut_out")
    if os.path.isdir(out_dir):
        shutil.rmtree(out_dir)
    # the generator reports an error when it has to create the folder itself
    # (main.cpp:570 treats create_directories' "created" as a failure)
    os.makedirs(out_dir)
    subprocess.run([exe, str(RES), "REC_709", out_dir], check=True)
    shutil.copyfile(os.path.join(out_dir, "REC_709.mrspectra"), os.path.join(HERE, "REC_709_r%d.mrspectra" % RES))

    L = C.CDLL(lib)
    L.ref_cie_count.restype = C.c_uint32
    L.ref_cie_start.restype = C.c_uint32
    n = L.ref_cie_count()
    vp = C.c_void_p
    xyz = np.zeros((n, 3), np.float32)
    L.ref_cie_xyz(vp(xyz.ctypes.data))
    integ = np.zeros(3, np.float32)
    L.ref_cie_integrals(vp(integ.ctypes.data))
    spd = np.zeros(n, np.float32)
    norm = np.zeros(1, np.float32)
    L.ref_illuminant_spd(vp(spd.ctypes.data), vp(norm.ctypes.data))
    r2x = np.zeros(9, np.float32)
    x2r = np.zeros(9, np.float32)
    L.ref_rgb_xyz_matrices(vp(r2x.ctypes.data), vp(x2r.ctypes.data))
    np.savez(os.path.join(HERE, "spectral_rec709.npz"), cie_start=np.uint32(L.ref_cie_start()), cie_xyz=xyz,
             cie_integrals=integ, illuminant=spd, illuminant_norm=norm, rgb_to_xyz=r2x, xyz_to_rgb=x2r)
    print("wrote", RES, n)


if __name__ == "__main__":
    main()
