"""Host-side mirror of MRay's TracerI (Source/Core/TracerI.h:150-376) over
the C ABI of include/mray_gb300_tracer.h.

Method names follow TracerI (CreatePrimitiveGroup -> create_primitive_group
and so on); ids are MRay's keys as the library returns them; attribute data
is passed as numpy arrays of the attribute's element type; errors raise
``MRGError`` carrying the message where MRay throws ``MRayError``.
"""
import ctypes as C

import numpy as np

from . import _native as N

KIND = {"prim": N.MRG_KIND_PRIM, "material": N.MRG_KIND_MATERIAL, "transform": N.MRG_KIND_TRANSFORM,
        "camera": N.MRG_KIND_CAMERA, "medium": N.MRG_KIND_MEDIUM, "light": N.MRG_KIND_LIGHT,
        "renderer": N.MRG_KIND_RENDERER}
PIXEL = {"rgba8_unorm": N.MRG_PIX_RGBA8_UNORM, "rgb_float": N.MRG_PIX_RGB_FLOAT, "rgba_float": N.MRG_PIX_RGBA_FLOAT,
         "r8_unorm": N.MRG_PIX_R8_UNORM, "r_float": N.MRG_PIX_R_FLOAT}
SAMPLER = {"independent": N.MRG_TRACER_SAMPLER_INDEPENDENT, "zsobol": N.MRG_TRACER_SAMPLER_ZSOBOL}

# (P)Triangle attribute indices (PrimitiveDefaultTriangle.cu:169-184)
POSITION, NORMAL, UV0, INDEX = 0, 1, 2, 3


def _u32s(v):
    return np.ascontiguousarray(np.asarray(v, np.uint32).ravel())


class Tracer:
    def __init__(self, seed=0, device=0, sampler="independent", film_filter_radius=0.0, watertight=False,
                 gen_mips=False, mip_filter_radius=0.0):
        p = N.MrgTracerParams()
        p.seed = int(seed)
        p.device = int(device)
        p.samplerType = SAMPLER[sampler]
        p.filmFilterRadius = float(film_filter_radius)
        p.triangleTest = N.MRG_TRI_WATERTIGHT if watertight else N.MRG_TRI_MOLLER_TRUMBORE
        p.genMips = 1 if gen_mips else 0
        p.mipGenFilterRadius = float(mip_filter_radius)
        self._h = C.c_void_p()
        self._L = N.lib()
        N.check(self._L.mrg_tracer_create(C.byref(p), C.byref(self._h)))
        self._film_shape = None

    def close(self):
        if self._h:
            self._L.mrg_tracer_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        N.check(getattr(self._L, name)(self._h, *args))

    def _id(self, name, *args):
        out = C.c_uint32()
        self._call(name, *args, C.byref(out))
        return out.value

    # ---- generic ----
    def parameters(self):
        p = N.MrgTracerParams()
        self._call("mrg_tracer_parameters", C.byref(p))
        return p

    def type_names(self, kind):
        need = C.c_size_t()
        self._call("mrg_tracer_type_names", KIND[kind], None, 0, C.byref(need))
        buf = C.create_string_buffer(need.value)
        self._call("mrg_tracer_type_names", KIND[kind], buf, need.value, None)
        return [n for n in buf.value.decode().split("\n") if n]

    def primitive_groups(self): return self.type_names("prim")
    def material_groups(self): return self.type_names("material")
    def transform_groups(self): return self.type_names("transform")
    def camera_groups(self): return self.type_names("camera")
    def medium_groups(self): return self.type_names("medium")
    def light_groups(self): return self.type_names("light")
    def renderers(self): return self.type_names("renderer")

    def attribute_info(self, kind, type_name):
        """[{name, data_type, element_bytes, optional, texturable, is_color}]"""
        n = C.c_uint32()
        self._call("mrg_tracer_attribute_info", KIND[kind], type_name.encode(), 0, None, C.byref(n))
        out = []
        for i in range(n.value):
            a = N.MrgTracerAttribInfo()
            self._call("mrg_tracer_attribute_info", KIND[kind], type_name.encode(), i, C.byref(a), None)
            out.append(dict(name=a.name.decode(), data_type=N.MRG_DT_NAMES[a.dataType], element_bytes=a.elementBytes,
                            optional=bool(a.optional), texturable=a.texturable, is_color=bool(a.isColor)))
        return out

    def type_name(self, kind, group_id):
        buf = C.create_string_buffer(64)
        self._call("mrg_tracer_group_type_name", KIND[kind], group_id, buf, 64)
        return buf.value.decode()

    # ---- primitives ----
    def create_primitive_group(self, type_name):
        return self._id("mrg_tracer_create_prim_group", type_name.encode())

    def reserve_primitive_batches(self, group_id, counts):
        """counts: [(primCount, attributeCount)] -> batch ids"""
        c = _u32s(counts)
        ids = np.zeros(len(counts), np.uint32)
        self._call("mrg_tracer_reserve_prim_batches", group_id, c.ctypes.data, len(counts), ids.ctypes.data)
        return [int(x) for x in ids]

    def reserve_primitive_batch(self, group_id, prim_count, attribute_count):
        return self.reserve_primitive_batches(group_id, [(prim_count, attribute_count)])[0]

    def commit_prim_reservations(self, group_id):
        self._call("mrg_tracer_commit_prim_reservations", group_id)

    def is_prim_committed(self, group_id):
        return bool(self._id("mrg_tracer_is_prim_committed", group_id))

    def push_prim_attribute(self, group_id, batch_id, attribute_index, data, sub_range=None):
        dt = np.uint32 if attribute_index == INDEX else np.float32
        a = np.ascontiguousarray(data, dt)
        b, e = (0, 0) if sub_range is None else sub_range
        self._call("mrg_tracer_push_prim_attribute", group_id, batch_id, attribute_index, b, e, a.ctypes.data, a.nbytes)

    def transform_primitives(self, group_id, batch_ids, matrices):
        b = _u32s(batch_ids)
        m = np.ascontiguousarray(np.asarray(matrices, np.float32).reshape(len(batch_ids), 12))
        self._call("mrg_tracer_transform_primitives", group_id, b.ctypes.data, m.ctypes.data, len(batch_ids))

    # ---- groups of materials, transforms, lights, cameras ----
    def create_material_group(self, type_name):
        return self._id("mrg_tracer_create_mat_group", type_name.encode())

    def create_transform_group(self, type_name):
        return self._id("mrg_tracer_create_trans_group", type_name.encode())

    def create_camera_group(self, type_name):
        return self._id("mrg_tracer_create_camera_group", type_name.encode())

    def create_light_group(self, type_name, prim_group_id=0):
        return self._id("mrg_tracer_create_light_group", type_name.encode(), prim_group_id)

    def _reserve(self, fn, group_id, n):
        ids = np.zeros(n, np.uint32)
        self._call(fn, group_id, n, ids.ctypes.data)
        return [int(x) for x in ids]

    def reserve_materials(self, group_id, n):
        return self._reserve("mrg_tracer_reserve_materials", group_id, n)

    def reserve_transformations(self, group_id, n):
        return self._reserve("mrg_tracer_reserve_transforms", group_id, n)

    def reserve_cameras(self, group_id, n):
        return self._reserve("mrg_tracer_reserve_cameras", group_id, n)

    def reserve_lights(self, group_id, n, prim_batches=None):
        ids = np.zeros(n, np.uint32)
        pb = None if prim_batches is None else _u32s(prim_batches)
        self._call("mrg_tracer_reserve_lights", group_id, n, None if pb is None else pb.ctypes.data, ids.ctypes.data)
        return [int(x) for x in ids]

    def commit_mat_reservations(self, group_id): self._call("mrg_tracer_commit_mat_reservations", group_id)
    def commit_trans_reservations(self, group_id): self._call("mrg_tracer_commit_trans_reservations", group_id)
    def commit_light_reservations(self, group_id): self._call("mrg_tracer_commit_light_reservations", group_id)
    def commit_cam_reservations(self, group_id): self._call("mrg_tracer_commit_cam_reservations", group_id)
    def is_mat_committed(self, group_id): return bool(self._id("mrg_tracer_is_mat_committed", group_id))
    def is_trans_committed(self, group_id): return bool(self._id("mrg_tracer_is_trans_committed", group_id))
    def is_light_committed(self, group_id): return bool(self._id("mrg_tracer_is_light_committed", group_id))
    def is_cam_committed(self, group_id): return bool(self._id("mrg_tracer_is_cam_committed", group_id))

    @staticmethod
    def _data(data, dtype):
        if data is None:
            return None, 0, None
        a = np.ascontiguousarray(data, dtype)
        return a.ctypes.data, a.nbytes, a

    def _push_tex(self, fn, group_id, id_range, attribute_index, data, textures, dtype):
        p, nb, keep = self._data(data, dtype)
        t = None if textures is None else _u32s([0 if x is None else x for x in textures])
        self._call(fn, group_id, id_range[0], id_range[1], attribute_index, p, nb,
                   None if t is None else t.ctypes.data)

    def push_mat_attribute(self, group_id, id_range, attribute_index, data=None, textures=None):
        """id_range: (first, last) ids, inclusive; textures: per item a
        texture id or None (the constant)."""
        self._push_tex("mrg_tracer_push_mat_attribute", group_id, id_range, attribute_index, data, textures, np.float32)

    def push_light_attribute(self, group_id, id_range, attribute_index, data=None, textures=None, dtype=np.float32):
        self._push_tex("mrg_tracer_push_light_attribute", group_id, id_range, attribute_index, data, textures, dtype)

    def push_trans_attribute(self, group_id, id_range, attribute_index, data):
        p, nb, keep = self._data(data, np.float32)
        self._call("mrg_tracer_push_trans_attribute", group_id, id_range[0], id_range[1], attribute_index, p, nb)

    def push_cam_attribute(self, group_id, id_range, attribute_index, data):
        p, nb, keep = self._data(data, np.float32)
        self._call("mrg_tracer_push_cam_attribute", group_id, id_range[0], id_range[1], attribute_index, p, nb)

    # ---- textures ----
    def create_texture_2d(self, width, height, mip_count=1, pixel_type="rgba_float"):
        return self._id("mrg_tracer_create_texture2d", width, height, mip_count, PIXEL[pixel_type])

    def commit_textures(self):
        self._call("mrg_tracer_commit_textures")

    def push_texture_data(self, texture_id, mip_level, data):
        a = np.ascontiguousarray(data)
        self._call("mrg_tracer_push_texture_data", texture_id, mip_level, a.ctypes.data, a.nbytes)

    # ---- surfaces ----
    def create_surface(self, prim_batches, materials, transform_id=0, cull_face=None, alpha_maps=None):
        s = N.MrgTracerSurface()
        n = len(prim_batches)
        s.count = n                         # the library rejects more than 8
        for i in range(min(n, 8)):
            s.primBatches[i] = prim_batches[i]
            s.materials[i] = materials[i]
            s.cullFace[i] = 1 if cull_face is None else int(bool(cull_face[i]))
            s.alphaMaps[i] = 0 if alpha_maps is None or alpha_maps[i] is None else alpha_maps[i]
        s.transformId = transform_id
        return self._id("mrg_tracer_create_surface", C.byref(s))

    def set_boundary_surface(self, light_id, transform_id=0):
        return self._id("mrg_tracer_set_boundary_surface", light_id, transform_id)

    def create_light_surface(self, light_id, transform_id=0):
        return self._id("mrg_tracer_create_light_surface", light_id, transform_id)

    def create_camera_surface(self, camera_id, transform_id=0):
        return self._id("mrg_tracer_create_camera_surface", camera_id, transform_id)

    def commit_surfaces(self):
        r = N.MrgTracerCommitResult()
        self._call("mrg_tracer_commit_surfaces", C.byref(r))
        return dict(aabb=tuple(r.aabb), instance_count=r.instanceCount, accelerator_count=r.acceleratorCount)

    def get_cam_transform(self, cam_surface_id):
        out = (C.c_float * 9)()
        self._call("mrg_tracer_get_cam_transform", cam_surface_id, out)
        return np.array(out[:], np.float32)

    def set_spectral_data(self, lut_res, lut, tables):
        k = [np.ascontiguousarray(lut, np.float32), np.ascontiguousarray(tables["cie_xyz"], np.float32),
             np.ascontiguousarray(tables["cie_integrals"], np.float32),
             np.ascontiguousarray(tables["illuminant"], np.float32),
             np.ascontiguousarray(tables["xyz_to_rgb"], np.float32)]
        self._call("mrg_tracer_set_spectral_data", lut_res, k[0].ctypes.data, k[1].shape[0], k[1].ctypes.data,
                   k[2].ctypes.data, k[3].ctypes.data, float(np.asarray(tables["illuminant_norm"]).ravel()[0]),
                   k[4].ctypes.data)

    # ---- renderers ----
    def create_renderer(self, type_name):
        return self._id("mrg_tracer_create_renderer", type_name.encode())

    def destroy_renderer(self, renderer_id):
        self._call("mrg_tracer_destroy_renderer", renderer_id)

    def push_renderer_attribute(self, renderer_id, attribute_index, value):
        """value: an int (totalSPP, burstSize, the guided renderer's cache
        options), a float (cacheConeAperture, lobeProbability), a str
        (renderMode, sampleMode, neeSamplerType, lightSampler, displayMode) or
        a pair of ints (rrRange)."""
        if isinstance(value, str):
            b = value.encode()
            self._call("mrg_tracer_push_renderer_attribute", renderer_id, attribute_index, b, len(b))
            return
        a = np.ascontiguousarray([value], np.float32) if isinstance(value, float) else _u32s(value)
        self._call("mrg_tracer_push_renderer_attribute", renderer_id, attribute_index, a.ctypes.data, a.nbytes)

    def start_render(self, renderer_id, cam_surface_id, width, height, region=None):
        info = N.MrgTracerRenderInfo()
        rmin, rmax = (None, None) if region is None else (_u32s(region[0]), _u32s(region[1]))
        self._call("mrg_tracer_start_render", renderer_id, cam_surface_id, width, height,
                   None if rmin is None else rmin.ctypes.data, None if rmax is None else rmax.ctypes.data,
                   C.byref(info))
        self._film_shape = (height, width, 4)
        return dict(width=info.width, height=info.height, total_spp=info.totalSpp, d_film=info.d_film)

    def set_camera_transform(self, renderer_id, cam):
        c = (C.c_float * 9)(*[float(x) for x in np.asarray(cam).ravel()])
        self._call("mrg_tracer_set_camera_transform", renderer_id, c)

    def do_render_work(self):
        o = N.MrgTracerRenderOutput()
        self._call("mrg_tracer_do_render_work", C.byref(o))
        return dict(samples_done=o.samplesDone, total_spp=o.totalSpp, finished=bool(o.finished),
                    work_ms=o.workMs, paths_per_second=o.pathsPerSecond)

    def read_film(self):
        if self._film_shape is None:
            raise N.MRGError(N.MRG_ERR_INVALID_ARG, "no render in progress")
        out = np.zeros(self._film_shape, np.float32)
        self._call("mrg_tracer_read_film", out.ctypes.data, out.nbytes)
        return out

    def stop_render(self):
        self._call("mrg_tracer_stop_render")

    def clear_all(self):
        self._call("mrg_tracer_clear_all")

    def flush(self):
        self._call("mrg_tracer_flush")

    def device_memory(self):
        t, u = C.c_uint64(), C.c_uint64()
        self._call("mrg_tracer_device_memory", C.byref(t), C.byref(u))
        return t.value, u.value

    def context(self):
        return self._L.mrg_tracer_context(self._h)
