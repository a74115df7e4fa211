"""Spectral inputs of the path tracer: MRay's MR_SPECTRA coefficient LUT
files (written by its SpectraLUTGen, Source/SpectraLUTGen/main.cpp:596-606)
and its colour tables (CIE 1931 observer, illuminant SPD, XYZ -> RGB)."""
import numpy as np

MAGIC = b"MR_SPECTRA"


def read_mrspectra(path):
    """Returns (resolution, float32 array of 9 * res^3): the ten characters
    MR_SPECTRA, uint32 resolution, uint32 mode (1 = float), then the data."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:len(MAGIC)] != MAGIC:
        raise ValueError("%s: not an MR_SPECTRA file" % path)
    res, mode = np.frombuffer(raw[10:18], np.uint32)
    if mode != 1:
        raise ValueError("%s: only float (mode 1) LUTs are supported" % path)
    lut = np.frombuffer(raw[18:], np.float32)
    if lut.size != 9 * int(res) ** 3:
        raise ValueError("%s: %d floats for resolution %d" % (path, lut.size, res))
    return int(res), np.ascontiguousarray(lut)


def load_tables(path):
    """Colour tables as a dict: cie_xyz (n, 3), cie_integrals (3,),
    illuminant (n,), illuminant_norm, xyz_to_rgb (9,)."""
    t = np.load(path)
    return {k: t[k] for k in t.files}
