"""Host-side mirror of MRay's path-tracer renderer over the C ABI.

``PathTracer`` wraps ``mrg_pt_*``: surfaces get a Lambert material or an
area light (MRay's primitive-backed lights: every triangle of a light surface
is one light), ``params`` mirrors the renderer attributes (totalSPP,
russianRouletteRange, sampleMode, film filter radius, pinhole camera) and
``render`` accumulates samples into a device film of (R, G, B, weight).
"""
import ctypes as C

import numpy as np

from . import _native as N
from .accel import Accelerator, _stream_ptr


class PathTracer:
    def __init__(self, device=0):
        self.acc = Accelerator(device)
        self.device = device
        self.n_instances = 0
        self._prim_base = 0

    def add_surface(self, pos, idx, m34, cull=True, uv=None):
        """Adds a mesh instance with dense primitive keys and trans_key =
        instance id (what the renderer's shading looks up); uv: optional
        per-vertex texture coordinates."""
        nt = int(np.asarray(idx).reshape(-1, 3).shape[0])
        mesh = self.acc.upload_mesh(pos, idx, prim_key_base=self._prim_base)
        if uv is not None:
            u = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
            N.check(N.lib().mrg_upload_mesh_uv(self.acc._h, mesh, u.ctypes.data, u.shape[0]))
        inst = self.n_instances
        self.acc.add_instance(mesh, m34, cull=cull, trans_key=inst, accel_key=inst)
        self._prim_base += nt
        self.n_instances += 1
        return inst

    def add_texture(self, texels):
        """An albedo texture: a (h, w, 4) uint8 / float32 numpy array (copied)
        or a float32 CUDA tensor (borrowed: rewrites show in later renders).
        Returns its id."""
        out = C.c_uint32()
        if hasattr(texels, "data_ptr"):
            if texels.dtype.__str__() != "torch.float32" or texels.dim() != 3 or texels.shape[2] != 4:
                raise ValueError("device textures are (h, w, 4) float32")
            if not texels.is_contiguous():
                raise ValueError("device textures must be contiguous")
            self._tex_keep = getattr(self, "_tex_keep", []) + [texels]
            N.check(N.lib().mrg_pt_add_texture(self.acc._h, texels.shape[1], texels.shape[0], 1,
                                               C.c_void_p(texels.data_ptr()), 1, C.byref(out)))
            self._tex_shapes = getattr(self, "_tex_shapes", {})
            self._tex_shapes[out.value] = (texels.shape[0], texels.shape[1], np.float32)
            return out.value
        t = np.ascontiguousarray(texels)
        if t.ndim != 3 or t.shape[2] != 4 or t.dtype not in (np.uint8, np.float32):
            raise ValueError("textures are (h, w, 4) uint8 or float32")
        N.check(N.lib().mrg_pt_add_texture(self.acc._h, t.shape[1], t.shape[0], 0 if t.dtype == np.uint8 else 1,
                                           t.ctypes.data, 0, C.byref(out)))
        self._tex_shapes = getattr(self, "_tex_shapes", {})
        self._tex_shapes[out.value] = (t.shape[0], t.shape[1], t.dtype.type)
        return out.value

    def render_cached(self, p, image=None, train_paths=32768, stream=None, loss=False):
        """One cache-assisted frame (see mrg_pt_render_cached); needs a
        RadianceCache created on this tracer.  Returns (image, loss or None)."""
        import torch
        if image is None:
            image = torch.zeros((p.height, p.width, 4), dtype=torch.float32, device="cuda:%d" % self.acc.device)
        l = C.c_float(0.0)
        N.check(N.lib().mrg_pt_render_cached(self.acc._h, C.byref(p), C.c_void_p(image.data_ptr()), train_paths,
                                             C.byref(l) if loss else None, _stream_ptr(stream)))
        return image, (l.value if loss else None)

    def adjoint(self, p, tex_id, image_adjoint, grad=None, image=None, stream=None, grad_emission=None):
        """Path-replay adjoint (see mrg_pt_adjoint): image_adjoint is a
        (h, w, 4) float32 CUDA tensor of dLoss/dPixel; returns grad, a
        (texH, texW, 4) float32 CUDA tensor the texture gradient is added to
        (None when tex_id is None: emission only).  grad_emission, a
        (n_instances, 4) float32 CUDA tensor, receives dLoss / d(radiance)
        of every area-light instance when given."""
        import torch
        dev = "cuda:%d" % self.acc.device
        if grad_emission is not None and (tuple(grad_emission.shape) != (self.n_instances, 4) or
                                          grad_emission.dtype != torch.float32 or
                                          not grad_emission.is_cuda or not grad_emission.is_contiguous()):
            raise ValueError("grad_emission must be a contiguous (n_instances, 4) float32 CUDA tensor")
        if tex_id is not None and grad is None:
            t = self._tex_shape(tex_id)
            grad = torch.zeros((t[0], t[1], 4), dtype=torch.float32, device=dev)
        N.check(N.lib().mrg_pt_adjoint(self.acc._h, C.byref(p), 0xFFFFFFFF if tex_id is None else tex_id,
                                       C.c_void_p(image_adjoint.data_ptr()),
                                       None if grad is None else C.c_void_p(grad.data_ptr()),
                                       None if grad_emission is None else C.c_void_p(grad_emission.data_ptr()),
                                       None if image is None else C.c_void_p(image.data_ptr()),
                                       _stream_ptr(stream)))
        return grad

    def _tex_shape(self, tex_id):
        return self._tex_shapes[tex_id]

    def generate_mips(self, tex_id, filter_radius=2.0):
        """A mip chain for the texture (see mrg_pt_generate_mips); 0 drops it."""
        N.check(N.lib().mrg_pt_generate_mips(self.acc._h, tex_id, float(filter_radius)))

    def set_texture_mip(self, tex_id, level, texels):
        """Given texels of one mip level (see mrg_pt_set_texture_mip): a
        (max(h >> level, 1), max(w >> level, 1), 4) array in the texture's
        format."""
        a = np.ascontiguousarray(texels)
        h, w, dt = getattr(self, "_tex_shapes", {}).get(tex_id, (None, None, None))
        if h is None or level < 1:
            raise ValueError("unknown texture or level < 1")
        if a.shape != (max(h >> level, 1), max(w >> level, 1), 4) or a.dtype != dt:
            raise ValueError("mip level %d of a %d x %d texture is (%d, %d, 4) %s"
                             % (level, w, h, max(h >> level, 1), max(w >> level, 1), np.dtype(dt).name))
        N.check(N.lib().mrg_pt_set_texture_mip(self.acc._h, tex_id, level, a.ctypes.data_as(C.c_void_p)))

    def set_unreal_textures(self, inst, roughness=None, metallic=None, specular=None):
        """Textured roughness / metallic / specular of an Unreal instance
        (texture ids; None keeps the constant)."""
        ids = [0xFFFFFFFF if t is None else t for t in (roughness, metallic, specular)]
        N.check(N.lib().mrg_pt_set_unreal_textures(self.acc._h, inst, *ids))

    def set_albedo_texture(self, inst, tex_id):
        N.check(N.lib().mrg_pt_set_albedo_texture(self.acc._h, inst, 0xFFFFFFFF if tex_id is None else tex_id))

    def set_lambert(self, inst, albedo):
        a = (C.c_float * 3)(*[float(x) for x in albedo])
        N.check(N.lib().mrg_pt_set_lambert(self.acc._h, inst, a))

    _MAT = {"lambert": N.MRG_MAT_LAMBERT, "reflect": N.MRG_MAT_REFLECT,
            "refract": N.MRG_MAT_REFRACT, "unreal": N.MRG_MAT_UNREAL}

    def set_material(self, inst, kind, albedo=(0.0, 0.0, 0.0), roughness=0.0, metallic=0.0,
                     specular=0.5, ior=(1.0, 1.5)):
        m = N.MrgPtMaterial()
        m.type = self._MAT[kind]
        m.albedo[:] = [float(x) for x in albedo]
        m.roughness, m.metallic, m.specular = float(roughness), float(metallic), float(specular)
        m.iorFront, m.iorBack = float(ior[0]), float(ior[1])
        N.check(N.lib().mrg_pt_set_material(self.acc._h, inst, C.byref(m)))

    def set_area_light(self, inst, radiance, two_sided=False):
        r = (C.c_float * 3)(*[float(x) for x in radiance])
        N.check(N.lib().mrg_pt_set_area_light(self.acc._h, inst, r, 1 if two_sided else 0))

    def set_env(self, texels, m34=None):
        """Skysphere radiance map, (h, w, 4) float32 RGBA (row 0 at v = 0);
        None removes it."""
        if texels is None:
            N.check(N.lib().mrg_pt_set_env(self.acc._h, 0, 0, None, None))
            return
        t = np.ascontiguousarray(texels, np.float32)
        if t.ndim != 3 or t.shape[2] != 4:
            raise ValueError("skysphere texels must be (height, width, 4)")
        m = None if m34 is None else np.ascontiguousarray(m34, np.float32).reshape(12)
        N.check(N.lib().mrg_pt_set_env(self.acc._h, t.shape[1], t.shape[0], t.ctypes.data,
                                       None if m is None else m.ctypes.data))

    def set_spectral(self, lut_res, lut, tables):
        """4-wavelength spectral rendering with an MR_SPECTRA LUT and MRay's
        colour tables (see mray_gb300.spectral); lut_res = 0 returns to RGB."""
        if not lut_res:
            N.check(N.lib().mrg_pt_set_spectral(self.acc._h, 0, None, 0, None, None, None, 0.0, None))
            return
        self._spec_keep = [np.ascontiguousarray(lut, np.float32),
                           np.ascontiguousarray(tables["cie_xyz"], np.float32),
                           np.ascontiguousarray(tables["cie_integrals"], np.float32),
                           np.ascontiguousarray(tables["illuminant"], np.float32),
                           np.ascontiguousarray(tables["xyz_to_rgb"], np.float32)]
        k = self._spec_keep
        N.check(N.lib().mrg_pt_set_spectral(self.acc._h, lut_res, k[0].ctypes.data, k[1].shape[0], k[1].ctypes.data,
                                            k[2].ctypes.data, k[3].ctypes.data,
                                            float(np.asarray(tables["illuminant_norm"]).ravel()[0]),
                                            k[4].ctypes.data))

    def build(self):
        self.acc.construct()

    @staticmethod
    def params(width, height, spp, camera, max_depth=8, rr_start=3, sample_mode=N.MRG_PT_NEE_MIS,
               seed=0, filter_radius=1.0, samples_per_pass=0, sample_start=0, partition="auto",
               sampler="independent", sampler_max_spp=0):
        p = N.MrgPtParams()
        p.sampler = {"independent": 0, "zsobol": 1, "zsobol-owen": 2, "pcg32": 3}[sampler]
        p.samplerMaxSpp = sampler_max_spp
        p.width, p.height, p.spp = width, height, spp
        p.samplesPerPass = samples_per_pass
        p.rrStart, p.maxDepth = rr_start, max_depth
        p.sampleMode, p.seed = sample_mode, seed
        p.filterRadius = filter_radius
        p.partitionByMaterial = 2 if partition == "auto" else (1 if partition else 0)
        p.camPos[:] = [float(x) for x in camera["pos"]]
        p.camGaze[:] = [float(x) for x in camera["gaze"]]
        p.camUp[:] = [float(x) for x in camera["up"]]
        p.fov[:] = [float(x) for x in camera["fov"]]
        p.nearFar[:] = [float(x) for x in camera["near_far"]]
        p.sampleStart = sample_start
        return p

    @staticmethod
    def camera_frame(p):
        out = (C.c_float * 16)()
        N.check(N.lib().mrg_pt_camera_frame(C.byref(p), out))
        return np.array(out[:], np.float32)

    def render(self, p, image=None, stream=None):
        """Adds p.spp samples per pixel to `image` (a device float32 tensor
        [H, W, 4], created zeroed when None) and returns it."""
        import torch
        if image is None:
            image = torch.zeros((p.height, p.width, 4), dtype=torch.float32, device="cuda")
        N.check(N.lib().mrg_pt_render(self.acc._h, C.byref(p), C.c_void_p(image.data_ptr()),
                                      _stream_ptr(stream)))
        return image

    # ---- guided path tracing (GuidedPTRenderer) ----
    def guide_create(self, entry_limit=2000000, pos_bits=14, normal_bits=2, max_level_offset=3,
                     cone_aperture=0.6, lobe_probability=0.75, fix_zero_weight=False):
        """Allocates the guiding hash grid over the built scene's box with
        GuidedPTRenderer's options (cacheEntryLimit, cachePosBits,
        cacheNormalBits, cacheMaxLvlOffset, cacheConeAperture in degrees,
        lobeProbablity)."""
        g = N.MrgGuideParams()
        N.check(N.lib().mrg_guide_defaults(C.byref(g)))
        g.entryLimit, g.posBits, g.normalBits = entry_limit, pos_bits, normal_bits
        g.maxLevelOffset, g.coneAperture, g.lobeProbability = max_level_offset, cone_aperture, lobe_probability
        g.fixZeroWeight = 1 if fix_zero_weight else 0
        N.check(N.lib().mrg_guide_create(self.acc._h, C.byref(g)))

    def guide_clear(self):
        N.check(N.lib().mrg_guide_clear(self.acc._h))

    def guide_stats(self):
        """(entries in use, table size)"""
        used, size = C.c_uint32(), C.c_uint32()
        N.check(N.lib().mrg_guide_stats(self.acc._h, C.byref(used), C.byref(size)))
        return used.value, size.value

    def guide_read(self):
        """The table: codes (uint64, ~0 empty), chains (n, 6: target xyz,
        cosine, weight, count), irradiance (n, 2: value, count)."""
        _, size = self.guide_stats()
        codes = np.empty(size, np.uint64)
        chain = np.empty((size, 6), np.float32)
        irr = np.empty((size, 2), np.float32)
        N.check(N.lib().mrg_guide_read(self.acc._h, codes.ctypes.data, chain.ctypes.data, irr.ctypes.data))
        return codes, chain, irr

    def render_guided(self, p, image=None, stream=None):
        """Adds p.spp guided samples per pixel to `image` (see
        mrg_pt_render_guided) and returns it."""
        import torch
        if image is None:
            image = torch.zeros((p.height, p.width, 4), dtype=torch.float32, device="cuda")
        N.check(N.lib().mrg_pt_render_guided(self.acc._h, C.byref(p), C.c_void_p(image.data_ptr()),
                                             _stream_ptr(stream)))
        return image

    def close(self):
        self.acc.close()


def load_box_scene(pt, seed=0):
    """Adds the box scene's surfaces (or a given surface list) to a
    PathTracer; returns the surface list."""
    from . import scenes
    surf = scenes.box_scene(seed) if isinstance(seed, int) else seed
    textures = {}
    for s in surf:
        inst = pt.add_surface(s["pos"], s["idx"], s["m34"], cull=s.get("cull", True), uv=s.get("uv"))
        if s["kind"] == "light":
            pt.set_area_light(inst, s["radiance"])
        else:
            pt.set_material(inst, s.get("material", "lambert"), s["albedo"],
                            roughness=s.get("roughness", 0.0), metallic=s.get("metallic", 0.0),
                            specular=s.get("specular", 0.5), ior=s.get("ior", (1.0, 1.5)))
            if s.get("texture") is not None:
                key = id(s["texture"])
                if key not in textures:
                    textures[key] = pt.add_texture(s["texture"])
                    if s.get("mip_radius"):
                        pt.generate_mips(textures[key], s["mip_radius"])
                    for lv, texels in sorted(s.get("mips_given", {}).items()):
                        pt.set_texture_mip(textures[key], lv, texels)
                pt.set_albedo_texture(inst, textures[key])
            params = [s.get(k + "_texture") for k in ("roughness", "metallic", "specular")]
            if any(t is not None for t in params):
                ids = []
                for t in params:
                    if t is None:
                        ids.append(None)
                        continue
                    if id(t) not in textures:
                        textures[id(t)] = pt.add_texture(t)
                        if s.get("mip_radius"):
                            pt.generate_mips(textures[id(t)], s["mip_radius"])
                    ids.append(textures[id(t)])
                pt.set_unreal_textures(inst, *ids)
    pt.build()
    return surf
