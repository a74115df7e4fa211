"""ctypes bindings of ``oracle/_ref/libmray_ref_pt.so``: MRay's own
path-tracer building blocks compiled from the MRay tree (see
``ref_pt_driver.cpp``).  Test infrastructure only; ``load()`` returns None
where the MRay tree is absent.

The record dtypes below are shared with the project's restatement
(``oracle.fx_*``), which takes the same records.
"""
import ctypes as C

import numpy as np

from . import build as _build

MAT_IN = np.dtype([("albedo", "<f4", 3), ("rough", "<f4"), ("metal", "<f4"), ("spec", "<f4"), ("iorF", "<f4"),
                   ("iorB", "<f4"), ("backSide", "<u4"), ("pos", "<f4", 3), ("wo", "<f4", 3),
                   ("wiEval", "<f4", 3), ("xi", "<u4", 3)])
MAT_OUT = np.dtype([("wi", "<f4", 3), ("wiPos", "<f4", 3), ("pdf", "<f4"), ("refl", "<f4", 4), ("passed", "<u4"),
                    ("evalRefl", "<f4", 4), ("evalPdf", "<f4"), ("specularity", "<f4")])
LIGHT_IN = np.dtype([("m", "<f4", 12), ("v9", "<f4", 9), ("twoSided", "<u4"), ("radiance", "<f4", 3),
                     ("distant", "<f4", 3), ("xi", "<u4", 2), ("hit", "<f4", 2), ("dir", "<f4", 3),
                     ("wo", "<f4", 3)])
LIGHT_OUT = np.dtype([("point", "<f4", 3), ("samplePdf", "<f4"), ("pdfSolidAngle", "<f4"), ("emitHit", "<f4", 4),
                      ("emitPoint", "<f4", 4), ("area", "<f4")])
assert MAT_IN.itemsize == 84 and MAT_OUT.itemsize == 72
assert LIGHT_IN.itemsize == 152 and LIGHT_OUT.itemsize == 56

MATERIALS = {"lambert": 0, "reflect": 1, "refract": 2, "unreal": 3}

_lib = None


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def load():
    global _lib
    if _lib is None:
        path = _build.build_ref_pt()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_spec_create.restype = C.c_void_p
        L.ref_spec_create.argtypes = [C.c_void_p, C.c_uint32]
        L.ref_spec_destroy.argtypes = [C.c_void_p]
        L.ref_spec_convert.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 3 + [C.c_uint32]
        L.ref_spec_to_rgb.argtypes = [C.c_void_p] + [C.c_void_p] * 4 + [C.c_uint32]
        _lib = L
    return _lib


def material(kind, rec):
    out = np.zeros(rec.shape[0], MAT_OUT)
    load().ref_material(C.c_int(MATERIALS[kind]), _p(rec), _p(out), C.c_uint32(rec.shape[0]))
    return out


def _rows(fn, inp, width_out, dtype=np.float32):
    inp = np.ascontiguousarray(inp, dtype)
    out = np.zeros((inp.shape[0], width_out), np.float32)
    fn(_p(inp), _p(out), C.c_uint32(inp.shape[0]))
    return out


def fresnel_dielectric(in3):
    return _rows(load().ref_fresnel_dielectric, in3, 1)[:, 0]


def vndf_sample(in6):
    return _rows(load().ref_vndf_sample, in6, 4)


def cos_sample(in2):
    return _rows(load().ref_cos_sample, in2, 4)


def russian_roulette(in6):
    return _rows(load().ref_russian_roulette, in6, 5)


def balance_cancelled(in4):
    return _rows(load().ref_balance_cancelled, in4, 1)[:, 0]


def nudge(in6):
    return _rows(load().ref_nudge, in6, 3)


def gaussian_filter(in3):
    return _rows(load().ref_gaussian_filter, in3, 5)


def spherical_coords(in6):
    return _rows(load().ref_spherical_coords, in6, 7)


def tri_light(rec):
    out = np.zeros(rec.shape[0], LIGHT_OUT)
    load().ref_tri_light(_p(rec), _p(out), C.c_uint32(rec.shape[0]))
    return out


def pwc2d(cdfx, cdfy, xi2, uvq2):
    h, w = cdfx.shape
    cdfx = np.ascontiguousarray(cdfx, np.float32)
    cdfy = np.ascontiguousarray(cdfy, np.float32)
    xi2 = np.ascontiguousarray(xi2, np.float32)
    uvq2 = np.ascontiguousarray(uvq2, np.float32)
    n = xi2.shape[0]
    out = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    load().ref_pwc2d(_p(cdfx), _p(cdfy), C.c_uint32(w), C.c_uint32(h), _p(xi2), _p(out), _p(uvq2), _p(pdf),
                     C.c_uint32(n))
    return out, pdf


def camera(cam13, res, pix, off4):
    cam13 = np.ascontiguousarray(cam13, np.float32)
    res = np.ascontiguousarray(res, np.uint32)
    pix = np.ascontiguousarray(pix, np.uint32)
    off4 = np.ascontiguousarray(off4, np.float32)
    out = np.zeros((pix.shape[0], 6), np.float32)
    load().ref_camera(_p(cam13), _p(res), _p(pix), _p(off4), _p(out), C.c_uint32(pix.shape[0]))
    return out


def sample_waves(mode, xi):
    xi = np.ascontiguousarray(xi, np.uint32)
    w = np.zeros((xi.shape[0], 4), np.float32)
    p = np.zeros((xi.shape[0], 4), np.float32)
    load().ref_spec_sample_waves(C.c_int(mode), _p(xi), _p(w), _p(p), C.c_uint32(xi.shape[0]))
    return w, p


def zsobol(in8):
    """in8 rows: px, py, seed, sampleIndex, initialMaxSPP, resMaxBits, dim,
    size -> up to 3 uint32 numbers (ZSobol::Next / Next2D / Next3D)."""
    in8 = np.ascontiguousarray(in8, np.uint32)
    out = np.zeros((in8.shape[0], 3), np.uint32)
    load().ref_zsobol(_p(in8), _p(out), C.c_uint32(in8.shape[0]))
    return out


def zsobol_seeds(seed, count):
    out = np.zeros(count, np.uint32)
    load().ref_zsobol_seeds(C.c_uint64(seed), C.c_uint32(count), _p(out))
    return out


def pcg32_jump(seeds, delta):
    """MRay's PermutedCG32: the number after Advance(delta[i]) of the stream
    GenerateState(seeds[i]) starts."""
    sd = np.ascontiguousarray(seeds, np.uint32)
    dl = np.ascontiguousarray(np.broadcast_to(np.asarray(delta, np.uint32), sd.shape))
    out = np.zeros(sd.shape, np.uint32)
    load().ref_pcg32_jump(_p(sd), _p(dl), C.c_uint32(sd.size), _p(out))
    return out


def pcg32_seq(seed, n):
    """The first n numbers (successive Next calls) of the stream
    GenerateState(seed) starts."""
    out = np.zeros(n, np.uint32)
    load().ref_pcg32_seq(C.c_uint32(seed), C.c_uint32(n), _p(out))
    return out


def guide_lobe(in7, w3):
    a = np.ascontiguousarray(in7, np.float32)
    w = np.ascontiguousarray(w3, np.float32)
    out = np.zeros((a.shape[0], 8), np.float32)
    load().ref_guide_lobe(_p(a), _p(w), _p(out), C.c_uint32(a.shape[0]))
    return out


def conc_octa(dirs, sts):
    d = np.ascontiguousarray(dirs, np.float32)
    s = np.ascontiguousarray(sts, np.float32)
    st2 = np.zeros((d.shape[0], 2), np.float32)
    dout = np.zeros((s.shape[0], 3), np.float32)
    load().ref_conc_octa(_p(d), _p(st2), _p(s), _p(dout), C.c_uint32(d.shape[0]))
    return st2, dout


def guide_codes(view15, in6, rng):
    v = np.ascontiguousarray(view15, np.float32)
    q = np.ascontiguousarray(in6, np.float32)
    r = np.array(rng, np.uint32, copy=True)
    out = np.zeros((q.shape[0], 2), np.uint64)
    load().ref_guide_codes(_p(v), _p(q), _p(r), _p(out), C.c_uint32(q.shape[0]))
    return out, r


def cone(in20):
    """RayCone Advance / Project, RefractRayCone and ConeAfterScatter
    (record layout of ref_cone in ref_pt_driver.cpp)."""
    return _rows(load().ref_cone, in20, 12)


def pixel_indices(in6):
    return _rows(load().ref_pixel_indices, in6, 2)


def guide_table(codes, probe, size):
    c = np.ascontiguousarray(codes, np.uint64)
    p = np.ascontiguousarray(probe, np.uint64)
    slots = np.zeros(c.size, np.uint32)
    found = np.zeros(p.size, np.uint32)
    load().ref_guide_table(_p(c), C.c_uint32(c.size), _p(p), C.c_uint32(p.size), C.c_uint32(size), _p(slots), _p(found))
    return slots, found


class Spectral:
    """MRay's Jakob 2019 converter over a resolution-64 LUT (the converter's
    compile-time resolution)."""

    def __init__(self, lut, res):
        self._lut = np.ascontiguousarray(lut, np.float32)
        self.h = load().ref_spec_create(_p(self._lut), C.c_uint32(res))
        if not self.h:
            raise ValueError("MRay's converter needs a resolution-64 LUT")

    def convert(self, rgb, waves, radiance=False):
        rgb = np.ascontiguousarray(rgb, np.float32)
        waves = np.ascontiguousarray(waves, np.float32)
        out = np.zeros((rgb.shape[0], 4), np.float32)
        load().ref_spec_convert(self.h, 1 if radiance else 0, _p(rgb), _p(waves), _p(out), rgb.shape[0])
        return out

    def to_rgb(self, value, waves, pdf):
        value, waves, pdf = (np.ascontiguousarray(a, np.float32) for a in (value, waves, pdf))
        out = np.zeros((value.shape[0], 3), np.float32)
        load().ref_spec_to_rgb(self.h, _p(value), _p(waves), _p(pdf), _p(out), value.shape[0])
        return out

    def close(self):
        if self.h:
            load().ref_spec_destroy(self.h)
            self.h = None
