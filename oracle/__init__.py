"""CPU oracle for the mray_gb300 hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` (as the checker) and bench.py's CPU
baseline / reference arm may import this package.  The product (mray_gb300)
never does.

``Scene`` wraps the C restatement of MRay's host-backend LBVH path
(mrg_oracle.c); ``RefCore`` wraps the reference's own compiled core math
(oracle/_ref/libmray_ref_core.so, built from the MRay source tree where it is
present).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

vp = C.c_void_p
u32 = C.c_uint32


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_intersect_triangle.argtypes = [vp] * 5 + [C.c_int, vp, vp, vp]
        L.orc_intersect_triangle.restype = C.c_int
        L.orc_intersect_aabb.argtypes = [vp] * 6
        L.orc_intersect_aabb.restype = C.c_int
        L.orc_mat34_inverse.argtypes = [vp, vp]
        L.orc_transform_ray.argtypes = [vp] * 5
        L.orc_transform_aabb.argtypes = [vp] * 5
        L.orc_morton3d_u64.argtypes = [u32, u32, u32]
        L.orc_morton3d_u64.restype = C.c_uint64
        L.orc_nudge.argtypes = [vp, vp, vp]
        L.orc_scene_set_watertight.argtypes = [vp, C.c_int]
        L.orc_intersect_triangle_wt.argtypes = [vp] * 5 + [C.c_int, vp, vp, vp]
        L.orc_intersect_triangle_wt.restype = C.c_int
        L.orc_scene_create.restype = vp
        L.orc_scene_destroy.argtypes = [vp]
        L.orc_scene_add_mesh.argtypes = [vp, vp, u32, vp, u32, u32]
        L.orc_scene_add_mesh.restype = C.c_int
        L.orc_scene_add_instance.argtypes = [vp, u32, vp, u32, u32, u32, u32]
        L.orc_mat34_inverse_corrected.argtypes = [vp, vp]
        L.orc_scene_add_instance.restype = C.c_int
        L.orc_scene_build.argtypes = [vp]
        L.orc_scene_build.restype = C.c_int
        L.orc_scene_instance_inverse.argtypes = [vp, u32, vp]
        for f in ("orc_cast_closest", "orc_cast_closest_linear"):
            getattr(L, f).argtypes = [vp, vp, vp, u32, vp, vp, vp, C.c_int]
        L.orc_cast_visibility.argtypes = [vp, vp, vp, u32, vp, C.c_int]
        L.orc_cast_local.argtypes = [vp, vp, vp, vp, u32, vp, vp, C.c_int]
        L.orc_scene_stats.argtypes = [vp, vp]
        L.orc_pt_render.argtypes = [vp, vp, vp, vp, u32, vp, vp, vp, C.c_int]
        L.orc_spec_prepare.argtypes = [vp, vp, vp, C.c_float, u32, vp, vp]
        L.orc_spec_sample_waves.argtypes = [C.c_float, vp, vp]
        L.orc_spec_convert_albedo.argtypes = [vp, vp, vp, vp]
        L.orc_spec_convert_radiance.argtypes = [vp, vp, vp, vp]
        L.orc_spec_to_rgb.argtypes = [vp, vp, vp, vp, vp]
        L.orc_scene_aabb.argtypes = [vp, vp]
        L.orc_scene_diameter.argtypes = [vp]
        L.orc_scene_diameter.restype = C.c_float
        L.orc_pwc2d_build.argtypes = [vp, u32, u32, vp, vp]
        L.orc_pwc2d_sample_uv.argtypes = [vp, vp, u32, u32, vp, vp, vp]
        L.orc_pwc2d_pdf_uv.argtypes = [vp, vp, u32, u32, vp]
        L.orc_pwc2d_pdf_uv.restype = C.c_float
        L.orc_env_luminance.argtypes = [vp, u32, u32, vp]
        L.orc_env_read.argtypes = [vp, u32, u32, vp, vp]
        L.orc_env_dir_to_uv.argtypes = [vp, vp]
        L.orc_env_uv_to_dir.argtypes = [vp, vp]
        L.orc_tex_read.argtypes = [vp, u32, u32, u32, vp, vp]
        L.orc_pt_adjoint.argtypes = [vp, vp, vp, vp, u32, vp, vp, u32, u32, vp, vp, vp, u32, C.c_int]
        L.orc_pt_adjoint.restype = C.c_int
        L.orc_zs_tables.argtypes = [vp, vp]
        L.orc_mt19937.argtypes = [u32, u32, vp]
        L.orc_zs_res_max_bits.argtypes = [u32, u32]
        L.orc_zs_res_max_bits.restype = u32
        L.orc_zs_seeds.argtypes = [u32, u32, C.c_uint64, vp]
        L.orc_zs_generate.argtypes = [u32, u32, vp, u32, u32, u32, C.c_uint64, u32, vp]
        L.orc_zs_generate.restype = C.c_int
        L.orc_zs_number.argtypes = [u32, u32, u32, u32, u32, u32, u32, u32, u32, C.c_int]
        L.orc_zs_number.restype = u32
        L.orc_pcg32_numbers.argtypes = [vp, vp, u32, vp]
        L.orc_guide_lobe_batch.argtypes = [vp, vp, vp, u32]
        L.orc_conc_octa_batch.argtypes = [vp, vp, vp, vp, u32]
        L.orc_guide_codes_batch.argtypes = [vp, vp, vp, vp, u32]
        L.orc_guide_table_batch.argtypes = [vp, u32, vp, u32, u32, vp, vp]
        L.orc_guide_new.argtypes = [vp, u32, u32, u32, u32, C.c_float, C.c_float, C.c_int]
        L.orc_guide_new.restype = vp
        L.orc_guide_delete.argtypes = [vp]
        L.orc_guide_clear.argtypes = [vp]
        L.orc_guide_table_size.argtypes = [vp]
        L.orc_guide_table_size.restype = u32
        L.orc_guide_used.argtypes = [vp]
        L.orc_guide_used.restype = u32
        L.orc_guide_snapshot.argtypes = [vp, vp, vp, vp]
        L.orc_pt_render_guided.argtypes = [vp, vp, vp, vp, u32, vp, vp, vp, u32, vp]
        L.orc_pt_render_guided.restype = C.c_int
        L.orc_gen_mips.argtypes = [vp, u32, u32, u32, C.c_float, vp]
        L.orc_gen_mips.restype = u32
        L.orc_gen_mips_levels.argtypes = [vp, u32, u32, u32, C.c_float, u32, u32, vp]
        L.orc_gen_mips_levels.restype = u32
        L.orc_pt_render.restype = C.c_int
        L.orc_pt_camera_frame.argtypes = [vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]
        L.orc_pt_make_light.argtypes = [vp, vp, vp, C.c_int, vp]
        _lib = L
    return _lib


def default_threads():
    return max(1, os.cpu_count() or 1)


class Scene:
    """Two-level LBVH scene with MRay host-backend semantics."""

    def __init__(self, watertight=False):
        """watertight: the restatement's watertight triangle test instead of
        MRay's Moller-Trumbore test for every mesh."""
        self._L = lib()
        self._h = self._L.orc_scene_create()
        self._keep = []
        if watertight:
            self._L.orc_scene_set_watertight(self._h, 1)

    def __del__(self):
        try:
            if self._h:
                self._L.orc_scene_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def add_mesh(self, pos, idx, prim_key_base=0):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
        r = self._L.orc_scene_add_mesh(self._h, _vp(pos), pos.shape[0], _vp(idx), idx.shape[0],
                                       prim_key_base)
        if r < 0:
            raise ValueError("oracle: bad mesh")
        return r

    def add_instance(self, mesh, m34, cull=True, lm_key=0, trans_key=0, accel_key=0,
                     corrected_inverse=False):
        m = np.ascontiguousarray(m34, np.float32).reshape(12)
        flags = (1 if cull else 0) | (2 if corrected_inverse else 0)
        r = self._L.orc_scene_add_instance(self._h, mesh, _vp(m), flags, lm_key,
                                           trans_key, accel_key)
        if r < 0:
            raise ValueError("oracle: bad instance")
        return r

    def build(self):
        if self._L.orc_scene_build(self._h) != 0:
            raise RuntimeError("oracle build failed")

    def instance_inverse(self, i):
        out = np.empty(12, np.float32)
        self._L.orc_scene_instance_inverse(self._h, i, _vp(out))
        return out

    def cast_closest(self, rays, ray_idx=None, hits=None, meta=None, linear=False, threads=None):
        """Returns (rays (tMax updated), hits [N,4] u32, meta [N,2] f32, inst [N] u32)."""
        rays = np.array(rays, np.float32, copy=True, order="C")
        n_total = rays.shape[0]
        hits = np.zeros((n_total, 4), np.uint32) if hits is None else np.array(hits, np.uint32, copy=True)
        meta = np.zeros((n_total, 2), np.float32) if meta is None else np.array(meta, np.float32, copy=True)
        inst = np.full(n_total, 0xFFFFFFFF, np.uint32)
        ridx = None if ray_idx is None else np.ascontiguousarray(ray_idx, np.uint32)
        n = n_total if ridx is None else ridx.shape[0]
        f = self._L.orc_cast_closest_linear if linear else self._L.orc_cast_closest
        f(self._h, _vp(rays), _vp(ridx), n, _vp(hits), _vp(meta), _vp(inst),
          threads or default_threads())
        return rays, hits, meta, inst

    def cast_local(self, rays, inst_ids, ray_idx=None, hits=None, meta=None, threads=None):
        """CastLocalRays: listed ray i against instance inst_ids[i] only.
        Returns (rays (tMax updated), hits [N,4] u32, meta [N,2] f32)."""
        rays = np.array(rays, np.float32, copy=True, order="C")
        n_total = rays.shape[0]
        hits = np.zeros((n_total, 4), np.uint32) if hits is None else np.array(hits, np.uint32, copy=True)
        meta = np.zeros((n_total, 2), np.float32) if meta is None else np.array(meta, np.float32, copy=True)
        ridx = None if ray_idx is None else np.ascontiguousarray(ray_idx, np.uint32)
        ids = np.ascontiguousarray(inst_ids, np.uint32)
        n = n_total if ridx is None else ridx.shape[0]
        assert ids.shape[0] == n
        self._L.orc_cast_local(self._h, _vp(rays), _vp(ridx), _vp(ids), n, _vp(hits), _vp(meta),
                               threads or default_threads())
        return rays, hits, meta

    def cast_visibility(self, rays, ray_idx=None, bits=None, threads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n_total = rays.shape[0]
        words = (n_total + 31) // 32
        bits = np.zeros(words, np.uint32) if bits is None else np.array(bits, np.uint32, copy=True)
        ridx = None if ray_idx is None else np.ascontiguousarray(ray_idx, np.uint32)
        n = n_total if ridx is None else ridx.shape[0]
        self._L.orc_cast_visibility(self._h, _vp(rays), _vp(ridx), n, _vp(bits),
                                    threads or default_threads())
        return bits

    def stats(self):
        out = np.zeros(4, np.uint64)
        self._L.orc_scene_stats(self._h, _vp(out))
        return out


def intersect_triangle(dir, pos, v0, v1, v2, cull):
    L = lib()
    a = [np.ascontiguousarray(x, np.float32) for x in (dir, pos, v0, v1, v2)]
    bary = np.zeros(3, np.float32)
    t = np.zeros(1, np.float32)
    bf = np.zeros(1, np.int32)
    hit = L.orc_intersect_triangle(*[_vp(x) for x in a], 1 if cull else 0, _vp(bary), _vp(t), _vp(bf))
    return bool(hit), bary, float(t[0]), bool(bf[0])


class RefCore:
    """The reference's own compiled core math (oracle/_ref), when built."""

    def __init__(self):
        global _ref
        if _ref is None:
            path = _build.build_ref()
            if path is None or not os.path.exists(path):
                raise FileNotFoundError("reference core library unavailable (MRay source tree absent)")
            R = C.CDLL(path)
            R.ref_intersect_triangles.argtypes = [u32, vp, vp, C.c_int, vp, vp, vp]
            R.ref_intersect_aabbs.argtypes = [u32, vp, vp, vp, vp, vp]
            R.ref_mat34_inverse.argtypes = [vp, vp]
            R.ref_transform_rays.argtypes = [u32, vp, vp, vp]
            R.ref_transform_aabb.argtypes = [vp, vp, vp]
            R.ref_morton3d_u64.argtypes = [u32, vp, vp]
            R.ref_nudge.argtypes = [u32, vp, vp, vp]
            _ref = R
        self.R = _ref

    def intersect_triangles(self, rays6, tris9, cull):
        n = rays6.shape[0]
        rays6 = np.ascontiguousarray(rays6, np.float32)
        tris9 = np.ascontiguousarray(tris9, np.float32)
        hit = np.zeros(n, np.uint32)
        bary = np.zeros((n, 3), np.float32)
        t = np.zeros(n, np.float32)
        self.R.ref_intersect_triangles(n, _vp(rays6), _vp(tris9), 1 if cull else 0, _vp(hit),
                                       _vp(bary), _vp(t))
        return hit, bary, t

    def intersect_aabbs(self, rays6, boxes6, tmm2):
        n = rays6.shape[0]
        hit = np.zeros(n, np.uint32)
        tout = np.zeros((n, 2), np.float32)
        self.R.ref_intersect_aabbs(n, _vp(np.ascontiguousarray(rays6, np.float32)),
                                   _vp(np.ascontiguousarray(boxes6, np.float32)),
                                   _vp(np.ascontiguousarray(tmm2, np.float32)), _vp(hit), _vp(tout))
        return hit, tout

    def mat34_inverse(self, m):
        out = np.zeros(12, np.float32)
        self.R.ref_mat34_inverse(_vp(np.ascontiguousarray(m, np.float32)), _vp(out))
        return out

    def transform_rays(self, m, rays6):
        out = np.zeros_like(rays6, dtype=np.float32)
        self.R.ref_transform_rays(rays6.shape[0], _vp(np.ascontiguousarray(m, np.float32)),
                                  _vp(np.ascontiguousarray(rays6, np.float32)), _vp(out))
        return out

    def transform_aabb(self, m, box6):
        out = np.zeros(6, np.float32)
        self.R.ref_transform_aabb(_vp(np.ascontiguousarray(m, np.float32)),
                                  _vp(np.ascontiguousarray(box6, np.float32)), _vp(out))
        return out

    def morton3d(self, xyz):
        xyz = np.ascontiguousarray(xyz, np.uint32)
        out = np.zeros(xyz.shape[0], np.uint64)
        self.R.ref_morton3d_u64(xyz.shape[0], _vp(xyz), _vp(out))
        return out

    def nudge(self, pos, dirs):
        pos = np.ascontiguousarray(pos, np.float32)
        out = np.zeros_like(pos)
        self.R.ref_nudge(pos.shape[0], _vp(pos), _vp(np.ascontiguousarray(dirs, np.float32)), _vp(out))
        return out


# ---------------------------------------------------------------------------
# path-tracer oracle
# ---------------------------------------------------------------------------
PT_PURE, PT_NEE, PT_NEE_MIS = 0, 1, 2


class PtParams(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("spp", u32), ("sampleStart", u32),
                ("rrStart", u32), ("maxDepth", u32), ("sampleMode", u32), ("seed", u32),
                ("filterRadius", C.c_float), ("camPos", C.c_float * 3),
                ("camBottomLeft", C.c_float * 3), ("camRight", C.c_float * 3),
                ("camUp", C.c_float * 3), ("planeSize", C.c_float * 2),
                ("nearT", C.c_float), ("farT", C.c_float), ("sampler", u32), ("samplerMaxSpp", u32),
                ("coneAperture", C.c_float)]


class PtTex(C.Structure):
    _fields_ = [("texels", vp), ("w", u32), ("h", u32), ("format", u32), ("mips", vp), ("mipCount", u32)]


class PtSurface(C.Structure):
    _fields_ = [("isLight", C.c_int), ("albedo", C.c_float * 3), ("matType", C.c_int),
                ("roughness", C.c_float), ("metallic", C.c_float), ("specular", C.c_float),
                ("iorFront", C.c_float), ("iorBack", C.c_float), ("lightBase", u32),
                ("primKeyBase", u32), ("triangles", vp), ("m", C.c_float * 12),
                ("inv", C.c_float * 12), ("texels", vp), ("texW", u32), ("texH", u32),
                ("texFormat", u32), ("uvs", vp), ("mips", vp), ("mipCount", u32), ("param", PtTex * 3)]


class PtLightTri(C.Structure):
    _fields_ = [("p0", C.c_float * 3), ("p1", C.c_float * 3), ("p2", C.c_float * 3),
                ("n", C.c_float * 3), ("area", C.c_float), ("radiance", C.c_float * 3),
                ("twoSided", C.c_int), ("instance", C.c_uint32)]


class PtEnv(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("texels", C.c_void_p),
                ("cdfX", C.c_void_p), ("cdfY", C.c_void_p), ("m", C.c_float * 12),
                ("inv", C.c_float * 12), ("sceneDiameter", C.c_float)]


class Pwc2D:
    """Piecewise-constant 2D distribution over a (h, w) function."""

    def __init__(self, func):
        func = np.ascontiguousarray(func, np.float32)
        self.h, self.w = func.shape
        self.cdf_x = np.zeros((self.h, self.w), np.float32)
        self.cdf_y = np.zeros(self.h, np.float32)
        lib().orc_pwc2d_build(_vp(func), self.w, self.h, _vp(self.cdf_x), _vp(self.cdf_y))

    def sample_uv(self, xi):
        xi = np.ascontiguousarray(xi, np.float32).reshape(-1, 2)
        uv = np.zeros_like(xi)
        pdf = np.zeros(xi.shape[0], np.float32)
        L = lib()
        for i in range(xi.shape[0]):
            L.orc_pwc2d_sample_uv(_vp(self.cdf_x), _vp(self.cdf_y), self.w, self.h,
                                  _vp(xi[i]), _vp(uv[i]), _vp(pdf[i:i + 1]))
        return uv, pdf

    def pdf_uv(self, uv):
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        L = lib()
        return np.array([L.orc_pwc2d_pdf_uv(_vp(self.cdf_x), _vp(self.cdf_y), self.w, self.h, _vp(uv[i]))
                         for i in range(uv.shape[0])], np.float32)


def env_luminance(texels):
    t = np.ascontiguousarray(texels, np.float32)
    out = np.zeros(t.shape[:2], np.float32)
    lib().orc_env_luminance(_vp(t), t.shape[1], t.shape[0], _vp(out))
    return out


def env_read(texels, uv):
    t = np.ascontiguousarray(texels, np.float32)
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((uv.shape[0], 3), np.float32)
    for i in range(uv.shape[0]):
        lib().orc_env_read(_vp(t), t.shape[1], t.shape[0], _vp(uv[i]), _vp(out[i]))
    return out


def env_dir_to_uv(d):
    d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
    out = np.zeros((d.shape[0], 2), np.float32)
    for i in range(d.shape[0]):
        lib().orc_env_dir_to_uv(_vp(d[i]), _vp(out[i]))
    return out


def env_uv_to_dir(uv):
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    out = np.zeros((uv.shape[0], 3), np.float32)
    for i in range(uv.shape[0]):
        lib().orc_env_uv_to_dir(_vp(uv[i]), _vp(out[i]))
    return out


class OrcSpectral(C.Structure):
    _fields_ = [("lutRes", C.c_uint32), ("lut", C.c_void_p), ("cieCount", C.c_uint32),
                ("observer", C.c_void_p), ("illuminant", C.c_void_p), ("xyzToRgb", C.c_float * 9)]


def read_mrspectra(path):
    """MRay's MR_SPECTRA LUT file (SpectraLUTGen/main.cpp:596-606): the ten
    characters MR_SPECTRA, uint32 resolution, uint32 mode (1 = float), then
    9 * res^3 floats."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:10] != b"MR_SPECTRA":
        raise ValueError("not an MR_SPECTRA file")
    res, mode = np.frombuffer(raw[10:18], np.uint32)
    if mode != 1:
        raise ValueError("only float MR_SPECTRA files are supported")
    lut = np.frombuffer(raw[18:], np.float32)
    if lut.size != 9 * int(res) ** 3:
        raise ValueError("truncated MR_SPECTRA file")
    return int(res), lut.copy()


class Spectral:
    """Spectral context of the oracle from a LUT file and the colour tables
    (tests/golden fixtures written from the MRay tree)."""

    def __init__(self, lut_path, tables_path):
        self.res, self.lut = read_mrspectra(lut_path)
        t = np.load(tables_path)
        n = int(t["cie_xyz"].shape[0])
        self.raw = {k: t[k] for k in t.files}
        self.observer = np.zeros((n, 3), np.float32)
        self.illuminant = np.zeros(n, np.float32)
        lib().orc_spec_prepare(_vp(np.ascontiguousarray(t["cie_xyz"], np.float32)),
                               _vp(np.ascontiguousarray(t["cie_integrals"], np.float32)),
                               _vp(np.ascontiguousarray(t["illuminant"], np.float32)),
                               float(t["illuminant_norm"][0]), n, _vp(self.observer), _vp(self.illuminant))
        c = OrcSpectral()
        c.lutRes, c.lut, c.cieCount = self.res, self.lut.ctypes.data, n
        c.observer, c.illuminant = self.observer.ctypes.data, self.illuminant.ctypes.data
        c.xyzToRgb[:] = [float(x) for x in t["xyz_to_rgb"]]
        self.c = c

    def sample_waves(self, xi0):
        w = np.zeros(4, np.float32)
        p = np.zeros(4, np.float32)
        lib().orc_spec_sample_waves(float(xi0), _vp(w), _vp(p))
        return w, p

    def convert_albedo(self, rgb, waves):
        out = np.zeros(4, np.float32)
        lib().orc_spec_convert_albedo(C.byref(self.c), _vp(np.ascontiguousarray(rgb, np.float32)),
                                      _vp(np.ascontiguousarray(waves, np.float32)), _vp(out))
        return out

    def convert_radiance(self, rgb, waves):
        out = np.zeros(4, np.float32)
        lib().orc_spec_convert_radiance(C.byref(self.c), _vp(np.ascontiguousarray(rgb, np.float32)),
                                        _vp(np.ascontiguousarray(waves, np.float32)), _vp(out))
        return out

    def to_rgb(self, value, waves, pdf):
        out = np.zeros(3, np.float32)
        lib().orc_spec_to_rgb(C.byref(self.c), _vp(np.ascontiguousarray(value, np.float32)),
                              _vp(np.ascontiguousarray(waves, np.float32)),
                              _vp(np.ascontiguousarray(pdf, np.float32)), _vp(out))
        return out


# ---- per-function entry points (records of oracle.ref_pt) ---------------

def fx_material(kind, rec):
    from . import ref_pt
    rec = np.ascontiguousarray(rec, ref_pt.MAT_IN)
    out = np.zeros(rec.shape[0], ref_pt.MAT_OUT)
    lib().orc_fx_material(C.c_int(ref_pt.MATERIALS[kind]), _vp(rec), _vp(out), C.c_uint32(rec.shape[0]))
    return out


def _fx_rows(fn, inp, width_out, dtype=np.float32):
    inp = np.ascontiguousarray(inp, dtype)
    out = np.zeros((inp.shape[0], width_out), np.float32)
    fn(_vp(inp), _vp(out), C.c_uint32(inp.shape[0]))
    return out


def fx_fresnel_dielectric(in3):
    return _fx_rows(lib().orc_fx_fresnel_dielectric, in3, 1)[:, 0]


def fx_vndf_sample(in6):
    return _fx_rows(lib().orc_fx_vndf_sample, in6, 4)


def fx_russian_roulette(in6):
    return _fx_rows(lib().orc_fx_russian_roulette, in6, 5)


def fx_gaussian_filter(in3):
    return _fx_rows(lib().orc_fx_gaussian_filter, in3, 5)


def fx_sample_waves(xi):
    xi = np.ascontiguousarray(xi, np.uint32)
    w = np.zeros((xi.shape[0], 4), np.float32)
    p = np.zeros((xi.shape[0], 4), np.float32)
    lib().orc_fx_sample_waves(_vp(xi), _vp(w), _vp(p), C.c_uint32(xi.shape[0]))
    return w, p


def fx_cone(in20):
    return _fx_rows(lib().orc_fx_cone, in20, 12)


def fx_pixel_indices(in6):
    return _fx_rows(lib().orc_fx_pixel_indices, in6, 2)


def fx_spherical_coords(in6):
    return _fx_rows(lib().orc_fx_spherical_coords, in6, 7)


def fx_tri_light(rec):
    from . import ref_pt
    rec = np.ascontiguousarray(rec, ref_pt.LIGHT_IN)
    out = np.zeros(rec.shape[0], ref_pt.LIGHT_OUT)
    lib().orc_fx_tri_light(_vp(rec), _vp(out), C.c_uint32(rec.shape[0]))
    return out


def fx_camera(cam13, res, pix, off4):
    cam13 = np.ascontiguousarray(cam13, np.float32)
    res = np.ascontiguousarray(res, np.uint32)
    pix = np.ascontiguousarray(pix, np.uint32)
    off4 = np.ascontiguousarray(off4, np.float32)
    out = np.zeros((pix.shape[0], 6), np.float32)
    lib().orc_fx_camera(_vp(cam13), _vp(res), _vp(pix), _vp(off4), _vp(out), C.c_uint32(pix.shape[0]))
    return out


class PtScene:
    """The CPU path-tracer oracle over a list of surfaces (dicts with pos,
    idx, m34, kind, albedo / radiance), keyed like mray_gb300.pt.PathTracer:
    dense primitive keys, instance id = surface index."""

    def __init__(self, surfaces, cull=True, env=None, spectral=None):
        self.L = lib()
        self.spectral = spectral
        self.S = Scene()
        self._keep = []
        prim = 0
        lights = []
        surf = (PtSurface * len(surfaces))()
        for k, s in enumerate(surfaces):
            pos = np.ascontiguousarray(s["pos"], np.float32)
            idx = np.ascontiguousarray(s["idx"], np.uint32)
            mid = self.S.add_mesh(pos, idx, prim_key_base=prim)
            lm = (0x80000000 | k) if s["kind"] == "light" else k
            self.S.add_instance(mid, s["m34"], cull=s.get("cull", cull), lm_key=lm, trans_key=k,
                                accel_key=k)
            tri = np.ascontiguousarray(pos[idx].reshape(-1, 9), np.float32)
            self._keep.append(tri)
            sf = surf[k]
            sf.isLight = 1 if s["kind"] == "light" else 0
            sf.albedo[:] = [float(x) for x in s.get("albedo", (0, 0, 0))]
            sf.matType = {"lambert": 0, "reflect": 1, "refract": 2, "unreal": 3}[s.get("material", "lambert")]
            sf.roughness = float(s.get("roughness", 0.0))
            sf.metallic = float(s.get("metallic", 0.0))
            sf.specular = float(s.get("specular", 0.5))
            ior = s.get("ior", (1.0, 1.5))
            sf.iorFront, sf.iorBack = float(ior[0]), float(ior[1])
            sf.lightBase = len(lights)
            sf.primKeyBase = prim
            sf.triangles = tri.ctypes.data_as(vp)
            sf.m[:] = [float(x) for x in np.asarray(s["m34"], np.float32).reshape(12)]
            if s.get("texture") is not None:
                tex = np.ascontiguousarray(s["texture"])
                if tex.dtype not in (np.uint8, np.float32) or tex.ndim != 3 or tex.shape[2] != 4:
                    raise ValueError("texture must be (h, w, 4) uint8 or float32")
                uv = np.ascontiguousarray(s["uv"], np.float32).reshape(-1, 2)
                uvp = np.ascontiguousarray(uv[idx].reshape(-1, 6), np.float32)
                self._keep += [tex, uvp]
                sf.texels = tex.ctypes.data
                sf.texH, sf.texW = tex.shape[0], tex.shape[1]
                sf.texFormat = 0 if tex.dtype == np.uint8 else 1
                sf.uvs = uvp.ctypes.data
                sf.mipCount = 1
                if s.get("mip_radius") or s.get("mips_given"):
                    key = (id(s["texture"]), float(s.get("mip_radius") or 0.0), id(s.get("mips_given")))
                    mips = getattr(self, "_mips", {})
                    if key not in mips:
                        mips[key] = gen_mips(tex, float(s.get("mip_radius") or 0.0), s.get("mips_given"))
                    self._mips = mips
                    chain, count = mips[key]
                    sf.mips = chain.ctypes.data
                    sf.mipCount = count
            params = [s.get(k + "_texture") for k in ("roughness", "metallic", "specular")]
            if any(t is not None for t in params):
                uv = np.ascontiguousarray(s["uv"], np.float32).reshape(-1, 2)
                uvp = np.ascontiguousarray(uv[idx].reshape(-1, 6), np.float32)
                self._keep.append(uvp)
                sf.uvs = uvp.ctypes.data
                for j, t in enumerate(params):
                    if t is None:
                        continue
                    t = np.ascontiguousarray(t)
                    if t.dtype not in (np.uint8, np.float32) or t.ndim != 3 or t.shape[2] != 4:
                        raise ValueError("texture must be (h, w, 4) uint8 or float32")
                    self._keep.append(t)
                    pt_ = sf.param[j]
                    pt_.texels = t.ctypes.data
                    pt_.h, pt_.w = t.shape[0], t.shape[1]
                    pt_.format = 0 if t.dtype == np.uint8 else 1
                    pt_.mipCount = 1
                    if s.get("mip_radius"):
                        chain, count = gen_mips(t, float(s["mip_radius"]))
                        self._keep.append(chain)
                        pt_.mips = chain.ctypes.data
                        pt_.mipCount = count
            if s["kind"] == "light":
                rad = (C.c_float * 3)(*[float(x) for x in s["radiance"]])
                m = np.ascontiguousarray(s["m34"], np.float32).reshape(12)
                for t in range(tri.shape[0]):
                    lt = PtLightTri()
                    self.L.orc_pt_make_light(_vp(m), _vp(tri[t]), rad, 0, C.byref(lt))
                    lt.instance = k
                    lights.append(lt)
            prim += idx.shape[0]
        self.S.build()
        for k in range(len(surfaces)):
            surf[k].inv[:] = [float(x) for x in self.S.instance_inverse(k)]
        self.surf = surf
        self.lights = (PtLightTri * max(1, len(lights)))(*lights)
        self.n_lights = len(lights)
        self.env = None
        if env is not None:
            # env: {"texels": (h, w, 4) f32, "m34": optional rotation}
            tex = np.ascontiguousarray(env["texels"], np.float32)
            h, w = tex.shape[:2]
            self._env_tex = tex
            self._env_dist = Pwc2D(env_luminance(tex))
            E = PtEnv()
            E.width, E.height = w, h
            E.texels = tex.ctypes.data
            E.cdfX = self._env_dist.cdf_x.ctypes.data
            E.cdfY = self._env_dist.cdf_y.ctypes.data
            m = np.asarray(env.get("m34", np.eye(3, 4)), np.float32).reshape(3, 4)
            E.m[:] = [float(x) for x in m.reshape(12)]
            inv = np.zeros(12, np.float32)
            self.L.orc_mat34_inverse_corrected(_vp(np.ascontiguousarray(m.reshape(12))), _vp(inv))
            E.inv[:] = [float(x) for x in inv]
            E.sceneDiameter = self.L.orc_scene_diameter(self.S._h)
            self.env = E

    def adjoint(self, p, surface, delta, threads=None, emission=False):
        """FP64 path-replay gradient of sum(delta * image) with respect to the
        RGB texels of the albedo texture of surface index `surface` (every
        surface sharing that texture array contributes; None: no texture).
        With emission=True returns (texture gradient or None, (n_surfaces, 4)
        gradient by each area light's radiance)."""
        d = np.ascontiguousarray(delta, np.float32)
        grad, texels, tw, th = None, None, 0, 0
        if surface is not None:
            sf = self.surf[surface]
            if not sf.texels:
                raise ValueError("surface has no texture")
            grad = np.zeros((sf.texH, sf.texW, 4), np.float64)
            texels, tw, th = C.c_void_p(sf.texels), sf.texW, sf.texH
        n = len(self.surf)
        ge = np.zeros((n, 4), np.float64) if emission else None
        rc = self.L.orc_pt_adjoint(self.S._h, C.byref(p), self.surf, self.lights, self.n_lights,
                                   C.byref(self.env) if self.env is not None else None,
                                   texels, tw, th, _vp(d), None if grad is None else _vp(grad),
                                   None if ge is None else _vp(ge), n, threads or default_threads())
        if rc != 0:
            raise RuntimeError("oracle adjoint failed")
        return (grad, ge) if emission else grad

    def scene_aabb(self):
        out = np.zeros(6, np.float32)
        self.L.orc_scene_aabb(self.S._h, _vp(out))
        return out

    @staticmethod
    def params(width, height, spp, camera, max_depth=8, rr_start=3, sample_mode=PT_NEE_MIS, seed=0,
               filter_radius=1.0, sample_start=0, sampler=0, sampler_max_spp=0):
        p = PtParams()
        p.sampler, p.samplerMaxSpp = sampler, sampler_max_spp
        p.width, p.height, p.spp, p.sampleStart = width, height, spp, sample_start
        p.rrStart, p.maxDepth, p.sampleMode, p.seed = rr_start, max_depth, sample_mode, seed
        p.filterRadius = filter_radius
        pos = (C.c_float * 3)(*camera["pos"])
        gaze = (C.c_float * 3)(*camera["gaze"])
        up = (C.c_float * 3)(*camera["up"])
        lib().orc_pt_camera_frame(pos, gaze, up, float(camera["fov"][0]), float(camera["fov"][1]),
                                  float(camera["near_far"][0]), float(camera["near_far"][1]), C.byref(p))
        return p

    def guide(self, entry_limit=2000000, pos_bits=14, normal_bits=2, max_level_offset=3, cone_aperture=0.6,
              lobe_probability=0.75, fix_zero_weight=False):
        """A guided path tracer's state (hash grid, chains, irradiance) over
        this scene (GuidedPTRenderer options, as mray_gb300.pt.PathTracer.guide_create)."""
        return GuideState(self, entry_limit, pos_bits, normal_bits, max_level_offset, cone_aperture,
                          lobe_probability, fix_zero_weight)

    def render_guided(self, p, guide, samples_per_pass, image=None):
        """Guided samples (single-threaded wavefront) added to image."""
        img = np.zeros((p.height, p.width, 4), np.float32) if image is None else image
        rc = self.L.orc_pt_render_guided(self.S._h, C.byref(p), self.surf, self.lights, self.n_lights,
                                         C.byref(self.env) if self.env is not None else None,
                                         C.byref(self.spectral.c) if self.spectral is not None else None,
                                         guide._h, samples_per_pass, _vp(img))
        if rc != 0:
            raise RuntimeError("oracle guided render failed (%d)" % rc)
        return img

    def render(self, p, image=None, threads=None):
        img = np.zeros((p.height, p.width, 4), np.float32) if image is None else image
        self.L.orc_pt_render(self.S._h, C.byref(p), self.surf, self.lights, self.n_lights,
                             C.byref(self.env) if self.env is not None else None,
                             C.byref(self.spectral.c) if self.spectral is not None else None,
                             _vp(img), threads or default_threads())
        return img


def mip_chain_texels(w, h, levels=None):
    """Texels of levels 1 .. levels - 1 (all of a full chain by default)."""
    n, m = 0, 1
    while ((w >> (m - 1)) > 1 or (h >> (m - 1)) > 1) and (levels is None or m < levels):
        n += max(w >> m, 1) * max(h >> m, 1)
        m += 1
    return n


def gen_mips(tex, radius, given=None):
    """Levels 1.. of a (h, w, 4) uint8 / float32 texture, one after another
    in a flat array of its dtype; returns (array, level count).  given maps
    levels to caller texels that are kept (their children filtered from
    them); with radius 0 the chain ends at the last given level
    (orc_gen_mips_levels)."""
    t = np.ascontiguousarray(tex)
    h, w = t.shape[:2]
    given = given or {}
    full = max(w, h).bit_length()
    if radius > 0:
        levels = full
    else:
        levels = max(given) + 1 if given else 1
        missing = [m for m in range(1, levels) if m not in given]
        if missing:
            raise ValueError("mip levels %s have no data and no generation filter" % missing)
    out = np.zeros(mip_chain_texels(w, h, levels) * 4, t.dtype)
    valid = 0
    for m, texels in given.items():
        if not 1 <= m < full:
            raise ValueError("mip level %d out of range" % m)
        o = mip_chain_texels(w, h, m) * 4
        a = np.ascontiguousarray(texels, t.dtype).ravel()
        if a.size != max(w >> m, 1) * max(h >> m, 1) * 4:
            raise ValueError("mip level %d has the wrong size" % m)
        out[o:o + a.size] = a
        valid |= 1 << m
    if radius > 0:
        lib().orc_gen_mips_levels(_vp(t), w, h, 0 if t.dtype == np.uint8 else 1, radius, levels, valid,
                                  _vp(out) if out.size else None)
    return out, levels


class GuideState:
    """orc_guide_state: the oracle's guiding grid, chains, irradiance
    averages and backup streams."""

    def __init__(self, scene, entry_limit, pos_bits, normal_bits, max_level_offset, cone_aperture, lobe_probability,
                 fix_zero_weight=False):
        self.L = lib()
        self._h = self.L.orc_guide_new(scene.S._h, entry_limit, pos_bits, normal_bits, max_level_offset,
                                       cone_aperture, lobe_probability, 1 if fix_zero_weight else 0)
        if not self._h:
            raise MemoryError("orc_guide_new")

    def clear(self):
        self.L.orc_guide_clear(self._h)

    def stats(self):
        return self.L.orc_guide_used(self._h), self.L.orc_guide_table_size(self._h)

    def read(self):
        n = self.L.orc_guide_table_size(self._h)
        codes = np.empty(n, np.uint64)
        chain = np.empty((n, 6), np.float32)
        irr = np.empty((n, 2), np.float32)
        self.L.orc_guide_snapshot(self._h, _vp(codes), _vp(chain), _vp(irr))
        return codes, chain, irr

    def __del__(self):
        if getattr(self, "_h", None):
            self.L.orc_guide_delete(self._h)
            self._h = None


def multi_partition(keys, indices=None, key_data_bits=(0, 0), key_batch_bits=(0, 32),
                    only_sort_for_batches=False):
    """RayPartitioner::MultiPartition (Source/Tracer/RayPartitioner.cu:263-411):
    stable radix sort of (key, index) by the data bits then the batch bits
    (one sort over the joined range when they are contiguous; the batch bits
    alone when only_sort_for_batches), then KCFindSplits (:19-49) marks where
    the batch portion changes and KCFindBinMatIds (:51-75) gathers each run's
    start offset and key.  Returns (count, offsets[count + 1], keys[count],
    sorted indices, sorted keys)."""
    k = np.asarray(keys, np.uint64).ravel()
    n = k.shape[0]
    idx = np.arange(n, dtype=np.uint64) if indices is None else np.asarray(indices, np.uint64).ravel()

    def bits(v, r):
        w = r[1] - r[0]
        return (v >> np.uint64(r[0])) & np.uint64((1 << w) - 1)

    comp = bits(k, key_batch_bits)
    if not only_sort_for_batches:
        comp = (comp << np.uint64(key_data_bits[1] - key_data_bits[0])) | bits(k, key_data_bits)
    order = np.argsort(comp, kind="stable")
    sk, si = k[order], idx[order]
    if n == 0:
        return 0, np.zeros(1, np.uint32), np.zeros(0, np.uint32), si.astype(np.uint32), sk.astype(np.uint32)
    b = bits(sk, key_batch_bits)
    starts = np.concatenate([[0], np.nonzero(b[1:] != b[:-1])[0] + 1]).astype(np.uint32)
    offsets = np.concatenate([starts, [n]]).astype(np.uint32)
    return (len(starts), offsets, sk[starts].astype(np.uint32), si.astype(np.uint32), sk.astype(np.uint32))


# ---- ZSobol random-number group (zsobol_oracle.c) ----------------------------
def zsobol_tables():
    """(3 x 52 uint32 Sobol matrices, 24 x 4 uint8 digit permutations)."""
    m = np.zeros((3, 52), np.uint32)
    p = np.zeros((24, 4), np.uint8)
    lib().orc_zs_tables(_vp(m), _vp(p))
    return m, p


def mt19937(seed, count):
    out = np.zeros(count, np.uint32)
    lib().orc_mt19937(seed, count, _vp(out))
    return out


def zsobol_seeds(width, height, seed):
    out = np.zeros(width * height, np.uint32)
    lib().orc_zs_seeds(width, height, seed, _vp(out))
    return out


def pcg32_numbers(seeds, delta):
    """Number delta[i] of MRay's PermutedCG32 stream seeded (GenerateState)
    by seeds[i]."""
    sd = np.ascontiguousarray(seeds, np.uint32)
    dl = np.ascontiguousarray(np.broadcast_to(np.asarray(delta, np.uint32), sd.shape))
    out = np.zeros(sd.shape, np.uint32)
    lib().orc_pcg32_numbers(_vp(sd), _vp(dl), sd.size, _vp(out))
    return out


def guide_lobe(in7, w3):
    """Gaussian (vMF) lobe records (dir, kappa, xi0, xi1, -) and a direction
    each -> (alpha, sample dir, pdf of the sample, pdf of w, XOverExp1M,
    XOverExp1MRecip of -2 kappa)."""
    a = np.ascontiguousarray(in7, np.float32)
    w = np.ascontiguousarray(w3, np.float32)
    out = np.zeros((a.shape[0], 8), np.float32)
    lib().orc_guide_lobe_batch(_vp(a), _vp(w), _vp(out), a.shape[0])
    return out


def conc_octa(dirs, sts):
    d = np.ascontiguousarray(dirs, np.float32)
    s = np.ascontiguousarray(sts, np.float32)
    st2 = np.zeros((d.shape[0], 2), np.float32)
    dout = np.zeros((s.shape[0], 3), np.float32)
    lib().orc_conc_octa_batch(_vp(d), _vp(st2), _vp(s), _vp(dout), d.shape[0])
    return st2, dout


def guide_codes(view15, in6, rng):
    """(GenCode, GenCodeStochastic) per record; rng: PCG32 states (a copy is
    advanced)."""
    v = np.ascontiguousarray(view15, np.float32)
    q = np.ascontiguousarray(in6, np.float32)
    r = np.array(rng, np.uint32, copy=True)
    out = np.zeros((q.shape[0], 2), np.uint64)
    lib().orc_guide_codes_batch(_vp(v), _vp(q), _vp(r), _vp(out), q.shape[0])
    return out, r


def guide_table(codes, probe, size):
    c = np.ascontiguousarray(codes, np.uint64)
    p = np.ascontiguousarray(probe, np.uint64)
    slots = np.zeros(c.size, np.uint32)
    found = np.zeros(p.size, np.uint32)
    lib().orc_guide_table_batch(_vp(c), c.size, _vp(p), p.size, size, _vp(slots), _vp(found))
    return slots, found


def zsobol_generate(width, height, seeds, initial_max_spp, sample_index, dim_start, requests):
    """requests: list of request sizes (1..3).  Returns (numbers, width*height)
    uint32 in MRay's strided order (number k of pixel i at [k, i])."""
    enc = 0
    for r, d in enumerate(requests):
        enc |= int(d) << (2 * r)
    total = int(sum(requests))
    out = np.zeros((total, width * height), np.uint32)
    sd = np.ascontiguousarray(seeds, np.uint32)
    rc = lib().orc_zs_generate(width, height, _vp(sd), initial_max_spp, sample_index, dim_start, enc,
                               len(requests), _vp(out))
    if rc != 0:
        raise ValueError("zsobol_generate: bad arguments")
    return out


def zsobol_number(px, py, seed, sample_index, initial_max_spp, res_max_bits, dim, size, comp, owen=False):
    """One ZSobol number (component comp of a size-number request)."""
    return int(lib().orc_zs_number(px, py, seed, sample_index, initial_max_spp, res_max_bits, dim, size, comp,
                                   1 if owen else 0))
