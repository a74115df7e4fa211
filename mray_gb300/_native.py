"""ctypes bindings of the C ABI declared in include/mray_gb300.h.

The library is built in-tree by ``mray_gb300.build.build()`` (or
``__graft_entry__.build()``).  Loading fails loudly when it is missing: there
is no CPU fallback for any entry point.
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
# MRAY_GB300_LIB selects another build of the library (e.g. a tuning variant).
LIB_PATH = os.environ.get("MRAY_GB300_LIB") or os.path.join(_PKG, "libmray_gb300.so")
SCENES_PATH = os.path.join(_PKG, "libmrg_scenes.so")

MRG_OK = 0
MRG_ERR_INVALID_ARG = 1
MRG_ERR_CUDA = 2
MRG_ERR_OUT_OF_MEMORY = 3
MRG_ERR_NOT_BUILT = 4
MRG_ERR_LIMIT = 5
MRG_ERR_TRAVERSAL = 6

MRG_INSTANCE_CULL_BACKFACE = 0x1
MRG_INSTANCE_CORRECTED_INVERSE = 0x2

#: every function declared in include/mray_gb300.h
EXPORTED = [
    "mrg_create", "mrg_destroy", "mrg_last_error", "mrg_status_string",
    "mrg_upload_mesh", "mrg_add_instance", "mrg_build", "mrg_cast_closest", "mrg_cast_local",
    "mrg_cast_visibility", "mrg_cast_closest_host", "mrg_scene_aabb", "mrg_get_stats",
    "mrg_sync_status", "mrg_cast_closest_stats", "mrg_cast_closest_host_noalloc",
    "mrg_pt_set_lambert", "mrg_pt_set_area_light", "mrg_pt_camera_frame", "mrg_pt_render",
    "mrg_pt_set_material", "mrg_pt_set_env", "mrg_multi_partition", "mrg_pt_set_spectral",
    "mrg_upload_mesh_uv", "mrg_pt_add_texture", "mrg_pt_set_albedo_texture", "mrg_pt_adjoint",
    "mrg_zsobol_seeds", "mrg_zsobol_generate",
    "mrg_cache_create", "mrg_cache_query", "mrg_cache_train", "mrg_cache_get_params", "mrg_cache_set_params",
    "mrg_cache_gradients", "mrg_pt_render_cached",
    "mrg_guide_defaults", "mrg_guide_create", "mrg_guide_clear", "mrg_guide_destroy", "mrg_guide_stats",
    "mrg_guide_read", "mrg_pt_render_guided", "mrg_pt_generate_mips", "mrg_pt_set_texture_mip", "mrg_pt_set_unreal_textures",
]

MRG_MAT_LAMBERT, MRG_MAT_REFLECT, MRG_MAT_REFRACT, MRG_MAT_UNREAL = 0, 1, 2, 3


class MrgPtMaterial(C.Structure):
    _fields_ = [("type", C.c_uint32), ("albedo", C.c_float * 3), ("roughness", C.c_float),
                ("metallic", C.c_float), ("specular", C.c_float), ("iorFront", C.c_float),
                ("iorBack", C.c_float)]

MRG_PT_PURE = 0
MRG_PT_NEE = 1
MRG_PT_NEE_MIS = 2


class MrgPtParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("samplesPerPass", C.c_uint32), ("rrStart", C.c_uint32), ("maxDepth", C.c_uint32),
                ("sampleMode", C.c_uint32), ("seed", C.c_uint32), ("filterRadius", C.c_float),
                ("camPos", C.c_float * 3), ("camGaze", C.c_float * 3), ("camUp", C.c_float * 3),
                ("fov", C.c_float * 2), ("nearFar", C.c_float * 2), ("sampleStart", C.c_uint32),
                ("partitionByMaterial", C.c_uint32), ("sampler", C.c_uint32), ("samplerMaxSpp", C.c_uint32)]

#: capacity of mrg_cast_closest_host_noalloc (rays per call)
MRG_NOALLOC_MAX_RAYS = 262144


class MrgCacheParams(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("log2_table_size", C.c_uint32), ("base_resolution", C.c_uint32),
                ("max_resolution", C.c_uint32), ("learning_rate", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("epsilon", C.c_float), ("seed", C.c_uint32), ("max_batch", C.c_uint32),
                ("aabb", C.c_float * 6)]


MRG_TRI_MOLLER_TRUMBORE = 0
MRG_TRI_WATERTIGHT = 1


class MrgParams(C.Structure):
    _fields_ = [("device", C.c_int), ("triangle_test", C.c_uint32), ("reserved", C.c_uint32 * 6)]


class MrgAccelStats(C.Structure):
    _fields_ = [("blasNodes", C.c_uint64), ("blasTriangles", C.c_uint64),
                ("tlasNodes", C.c_uint64), ("instances", C.c_uint64),
                ("deviceBytes", C.c_uint64), ("buildMs", C.c_double), ("accelerators", C.c_uint64)]


# ---- include/mray_gb300_tracer.h ----
TRACER_EXPORTED = [
    "mrg_tracer_create", "mrg_tracer_destroy", "mrg_tracer_parameters", "mrg_tracer_type_names",
    "mrg_tracer_attribute_info", "mrg_tracer_group_type_name",
    "mrg_tracer_create_prim_group", "mrg_tracer_reserve_prim_batches", "mrg_tracer_commit_prim_reservations",
    "mrg_tracer_is_prim_committed", "mrg_tracer_push_prim_attribute", "mrg_tracer_transform_primitives",
    "mrg_tracer_create_mat_group", "mrg_tracer_reserve_materials", "mrg_tracer_commit_mat_reservations",
    "mrg_tracer_is_mat_committed", "mrg_tracer_push_mat_attribute",
    "mrg_tracer_create_trans_group", "mrg_tracer_reserve_transforms", "mrg_tracer_commit_trans_reservations",
    "mrg_tracer_is_trans_committed", "mrg_tracer_push_trans_attribute",
    "mrg_tracer_create_light_group", "mrg_tracer_reserve_lights", "mrg_tracer_commit_light_reservations",
    "mrg_tracer_is_light_committed", "mrg_tracer_push_light_attribute",
    "mrg_tracer_create_camera_group", "mrg_tracer_reserve_cameras", "mrg_tracer_commit_cam_reservations",
    "mrg_tracer_is_cam_committed", "mrg_tracer_push_cam_attribute",
    "mrg_tracer_create_texture2d", "mrg_tracer_commit_textures", "mrg_tracer_push_texture_data",
    "mrg_tracer_create_surface", "mrg_tracer_set_boundary_surface", "mrg_tracer_create_light_surface",
    "mrg_tracer_create_camera_surface", "mrg_tracer_commit_surfaces", "mrg_tracer_get_cam_transform",
    "mrg_tracer_set_spectral_data", "mrg_tracer_create_renderer", "mrg_tracer_destroy_renderer",
    "mrg_tracer_push_renderer_attribute", "mrg_tracer_start_render", "mrg_tracer_set_camera_transform",
    "mrg_tracer_do_render_work", "mrg_tracer_read_film", "mrg_tracer_stop_render", "mrg_tracer_clear_all",
    "mrg_tracer_flush", "mrg_tracer_device_memory", "mrg_tracer_context",
]

MRG_KIND_PRIM, MRG_KIND_MATERIAL, MRG_KIND_TRANSFORM, MRG_KIND_CAMERA = 0, 1, 2, 3
MRG_KIND_MEDIUM, MRG_KIND_LIGHT, MRG_KIND_RENDERER = 4, 5, 6
MRG_TRACER_SAMPLER_INDEPENDENT, MRG_TRACER_SAMPLER_ZSOBOL = 0, 1
MRG_PIX_RGBA8_UNORM, MRG_PIX_RGB_FLOAT, MRG_PIX_RGBA_FLOAT, MRG_PIX_R8_UNORM, MRG_PIX_R_FLOAT = 0, 1, 2, 3, 4
MRG_ATTR_CONSTANT_ONLY, MRG_ATTR_TEXTURE_OR_CONSTANT, MRG_ATTR_TEXTURE_ONLY = 0, 1, 2
MRG_DT_NAMES = ["FLOAT", "VECTOR_2", "VECTOR_3", "VECTOR_4", "QUATERNION", "MATRIX_4x4", "UINT32", "VECTOR_2UI",
                "VECTOR_3UI", "BOOL", "STRING"]


class MrgTracerParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("device", C.c_int), ("samplerType", C.c_uint32),
                ("filmFilterRadius", C.c_float), ("triangleTest", C.c_uint32), ("genMips", C.c_uint32),
                ("mipGenFilterRadius", C.c_float), ("reserved", C.c_uint32 * 2)]


class MrgTracerAttribInfo(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("dataType", C.c_uint32), ("elementBytes", C.c_uint32),
                ("optional", C.c_uint32), ("texturable", C.c_uint32), ("isColor", C.c_uint32)]


class MrgTracerSurface(C.Structure):
    _fields_ = [("count", C.c_uint32), ("primBatches", C.c_uint32 * 8), ("materials", C.c_uint32 * 8),
                ("alphaMaps", C.c_uint32 * 8), ("cullFace", C.c_uint32 * 8), ("transformId", C.c_uint32)]


class MrgTracerCommitResult(C.Structure):
    _fields_ = [("aabb", C.c_float * 6), ("instanceCount", C.c_uint64), ("acceleratorCount", C.c_uint64)]


class MrgTracerRenderInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("totalSpp", C.c_uint32),
                ("channels", C.c_uint32), ("d_film", C.c_void_p)]


class MrgGuideParams(C.Structure):
    _fields_ = [("entryLimit", C.c_uint32), ("posBits", C.c_uint32), ("normalBits", C.c_uint32),
                ("maxLevelOffset", C.c_uint32), ("coneAperture", C.c_float), ("lobeProbability", C.c_float),
                ("fixZeroWeight", C.c_uint32), ("reserved", C.c_uint32)]


class MrgTracerRenderOutput(C.Structure):
    _fields_ = [("samplesDone", C.c_uint32), ("totalSpp", C.c_uint32), ("finished", C.c_uint32),
                ("workMs", C.c_float), ("pathsPerSecond", C.c_double)]


class MRGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("mrg status %d: %s" % (status, msg))
        self.status = status


_lib = None
_scenes = None

vp = C.c_void_p
u32 = C.c_uint32
u32p = C.POINTER(C.c_uint32)
fp = C.POINTER(C.c_float)


def _declare(lib):
    sig = {
        "mrg_create": (C.c_int, [C.POINTER(MrgParams), C.POINTER(vp)]),
        "mrg_destroy": (C.c_int, [vp]),
        "mrg_last_error": (C.c_char_p, []),
        "mrg_status_string": (C.c_char_p, [C.c_int]),
        "mrg_upload_mesh": (C.c_int, [vp, vp, u32, vp, u32, u32, u32p]),
        "mrg_add_instance": (C.c_int, [vp, u32, fp, u32, u32, u32, u32, u32p]),
        "mrg_build": (C.c_int, [vp]),
        "mrg_cast_closest": (C.c_int, [vp, vp, vp, u32, vp, vp, vp]),
        "mrg_cast_local": (C.c_int, [vp, vp, vp, vp, u32, vp, vp, vp]),
        "mrg_cast_visibility": (C.c_int, [vp, vp, vp, vp, u32, vp]),
        "mrg_cast_closest_host": (C.c_int, [vp, vp, u32, vp, vp]),
        "mrg_cast_closest_host_noalloc": (C.c_int, [vp, vp, u32, vp, vp]),
        "mrg_scene_aabb": (C.c_int, [vp, fp]),
        "mrg_get_stats": (C.c_int, [vp, C.POINTER(MrgAccelStats)]),
        "mrg_sync_status": (C.c_int, [vp, vp]),
        "mrg_cast_closest_stats": (C.c_int, [vp, vp, u32, C.POINTER(C.c_uint64), vp]),
        "mrg_pt_set_lambert": (C.c_int, [vp, u32, fp]),
        "mrg_pt_set_material": (C.c_int, [vp, u32, C.POINTER(MrgPtMaterial)]),
        "mrg_pt_set_area_light": (C.c_int, [vp, u32, fp, u32]),
        "mrg_pt_set_env": (C.c_int, [vp, u32, u32, vp, vp]),
        "mrg_pt_set_spectral": (C.c_int, [vp, u32, vp, u32, vp, vp, vp, C.c_float, vp]),
        "mrg_upload_mesh_uv": (C.c_int, [vp, u32, vp, u32]),
        "mrg_pt_add_texture": (C.c_int, [vp, u32, u32, u32, vp, u32, C.POINTER(u32)]),
        "mrg_pt_set_albedo_texture": (C.c_int, [vp, u32, u32]),
        "mrg_pt_generate_mips": (C.c_int, [vp, u32, C.c_float]),
        "mrg_pt_set_texture_mip": (C.c_int, [vp, u32, u32, vp]),
        "mrg_pt_set_unreal_textures": (C.c_int, [vp, u32, u32, u32, u32]),
        "mrg_pt_adjoint": (C.c_int, [vp, C.POINTER(MrgPtParams), u32, vp, vp, vp, vp, vp]),
        "mrg_zsobol_seeds": (C.c_int, [u32, u32, C.c_uint64, vp]),
        "mrg_zsobol_generate": (C.c_int, [u32, u32, vp, u32, u32, u32, C.c_uint64, u32, vp, vp]),
        "mrg_cache_create": (C.c_int, [vp, C.POINTER(MrgCacheParams)]),
        "mrg_cache_query": (C.c_int, [vp, vp, u32, vp, vp]),
        "mrg_cache_train": (C.c_int, [vp, vp, vp, u32, fp, vp]),
        "mrg_cache_get_params": (C.c_int, [vp, fp, fp]),
        "mrg_cache_set_params": (C.c_int, [vp, fp, fp]),
        "mrg_cache_gradients": (C.c_int, [vp, vp, vp, u32, fp, fp, fp]),
        "mrg_pt_render_cached": (C.c_int, [vp, C.POINTER(MrgPtParams), vp, u32, fp, vp]),
        "mrg_multi_partition": (C.c_int, [vp, vp, vp, u32, vp, vp, u32, vp, vp, vp, vp, vp, u32, vp]),
        "mrg_pt_camera_frame": (C.c_int, [C.POINTER(MrgPtParams), fp]),
        "mrg_pt_render": (C.c_int, [vp, C.POINTER(MrgPtParams), vp, vp]),
        "mrg_guide_defaults": (C.c_int, [C.POINTER(MrgGuideParams)]),
        "mrg_guide_create": (C.c_int, [vp, C.POINTER(MrgGuideParams)]),
        "mrg_guide_clear": (C.c_int, [vp]),
        "mrg_guide_destroy": (C.c_int, [vp]),
        "mrg_guide_stats": (C.c_int, [vp, u32p, u32p]),
        "mrg_guide_read": (C.c_int, [vp, vp, vp, vp]),
        "mrg_pt_render_guided": (C.c_int, [vp, C.POINTER(MrgPtParams), vp, vp]),
    }
    sz = C.c_size_t
    sig.update({
        "mrg_tracer_create": (C.c_int, [C.POINTER(MrgTracerParams), C.POINTER(vp)]),
        "mrg_tracer_destroy": (C.c_int, [vp]),
        "mrg_tracer_parameters": (C.c_int, [vp, C.POINTER(MrgTracerParams)]),
        "mrg_tracer_type_names": (C.c_int, [vp, u32, C.c_char_p, sz, C.POINTER(sz)]),
        "mrg_tracer_attribute_info": (C.c_int, [vp, u32, C.c_char_p, u32, C.POINTER(MrgTracerAttribInfo), u32p]),
        "mrg_tracer_group_type_name": (C.c_int, [vp, u32, u32, C.c_char_p, sz]),
        "mrg_tracer_create_prim_group": (C.c_int, [vp, C.c_char_p, u32p]),
        "mrg_tracer_reserve_prim_batches": (C.c_int, [vp, u32, vp, u32, vp]),
        "mrg_tracer_commit_prim_reservations": (C.c_int, [vp, u32]),
        "mrg_tracer_is_prim_committed": (C.c_int, [vp, u32, u32p]),
        "mrg_tracer_push_prim_attribute": (C.c_int, [vp, u32, u32, u32, u32, u32, vp, sz]),
        "mrg_tracer_transform_primitives": (C.c_int, [vp, u32, vp, vp, u32]),
        "mrg_tracer_set_boundary_surface": (C.c_int, [vp, u32, u32, u32p]),
        "mrg_tracer_create_light_surface": (C.c_int, [vp, u32, u32, u32p]),
        "mrg_tracer_create_camera_surface": (C.c_int, [vp, u32, u32, u32p]),
        "mrg_tracer_create_surface": (C.c_int, [vp, C.POINTER(MrgTracerSurface), u32p]),
        "mrg_tracer_commit_surfaces": (C.c_int, [vp, C.POINTER(MrgTracerCommitResult)]),
        "mrg_tracer_get_cam_transform": (C.c_int, [vp, u32, fp]),
        "mrg_tracer_set_spectral_data": (C.c_int, [vp, u32, vp, u32, vp, vp, vp, C.c_float, vp]),
        "mrg_tracer_create_renderer": (C.c_int, [vp, C.c_char_p, u32p]),
        "mrg_tracer_destroy_renderer": (C.c_int, [vp, u32]),
        "mrg_tracer_push_renderer_attribute": (C.c_int, [vp, u32, u32, vp, sz]),
        "mrg_tracer_start_render": (C.c_int, [vp, u32, u32, u32, u32, vp, vp, C.POINTER(MrgTracerRenderInfo)]),
        "mrg_tracer_set_camera_transform": (C.c_int, [vp, u32, fp]),
        "mrg_tracer_do_render_work": (C.c_int, [vp, C.POINTER(MrgTracerRenderOutput)]),
        "mrg_tracer_read_film": (C.c_int, [vp, vp, sz]),
        "mrg_tracer_stop_render": (C.c_int, [vp]),
        "mrg_tracer_clear_all": (C.c_int, [vp]),
        "mrg_tracer_flush": (C.c_int, [vp]),
        "mrg_tracer_device_memory": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "mrg_tracer_context": (vp, [vp]),
        "mrg_tracer_commit_textures": (C.c_int, [vp]),
        "mrg_tracer_create_texture2d": (C.c_int, [vp, u32, u32, u32, u32, u32p]),
        "mrg_tracer_push_texture_data": (C.c_int, [vp, u32, u32, vp, sz]),
    })
    for kind in ("mat", "trans", "light", "cam"):
        sig["mrg_tracer_commit_%s_reservations" % kind] = (C.c_int, [vp, u32])
        sig["mrg_tracer_is_%s_committed" % kind] = (C.c_int, [vp, u32, u32p])
    for name in ("mrg_tracer_create_mat_group", "mrg_tracer_create_trans_group", "mrg_tracer_create_camera_group"):
        sig[name] = (C.c_int, [vp, C.c_char_p, u32p])
    sig["mrg_tracer_create_light_group"] = (C.c_int, [vp, C.c_char_p, u32, u32p])
    for name in ("mrg_tracer_reserve_materials", "mrg_tracer_reserve_transforms", "mrg_tracer_reserve_cameras"):
        sig[name] = (C.c_int, [vp, u32, u32, vp])
    sig["mrg_tracer_reserve_lights"] = (C.c_int, [vp, u32, u32, vp, vp])
    for name in ("mrg_tracer_push_mat_attribute", "mrg_tracer_push_light_attribute"):
        sig[name] = (C.c_int, [vp, u32, u32, u32, u32, vp, sz, vp])
    for name in ("mrg_tracer_push_trans_attribute", "mrg_tracer_push_cam_attribute"):
        sig[name] = (C.c_int, [vp, u32, u32, u32, u32, vp, sz])
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def lib():
    """The CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libmray_gb300.so is not built; run __graft_entry__.build() "
                              "(mray_gb300.build.build()) first")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def scenes_lib():
    global _scenes
    if _scenes is None:
        if not os.path.exists(SCENES_PATH):
            raise ImportError("libmrg_scenes.so is not built; run mray_gb300.build.build_scenes()")
        s = C.CDLL(SCENES_PATH)
        d = C.c_double
        dp = C.POINTER(C.c_double)
        s.mrgs_icosphere_counts.argtypes = [u32, u32p, u32p]
        s.mrgs_icosphere_counts.restype = None
        s.mrgs_icosphere.argtypes = [u32, d, d, d, u32, vp, vp]
        s.mrgs_icosphere.restype = C.c_int
        s.mrgs_instance_field.argtypes = [u32, u32, d, d, vp]
        s.mrgs_instance_field.restype = C.c_int
        s.mrgs_primary_rays.argtypes = [u32, u32, dp, dp, dp, d, u32, vp]
        s.mrgs_primary_rays.restype = C.c_int
        s.mrgs_bounce_rays.argtypes = [u32, vp, vp, vp, vp, vp, vp, vp, u32, vp, vp]
        s.mrgs_bounce_rays.restype = u32
        s.mrgs_shadow_rays.argtypes = [u32, vp, dp, vp]
        s.mrgs_shadow_rays.restype = u32
        _scenes = s
    return _scenes


def check(status):
    if status != MRG_OK:
        raise MRGError(status, lib().mrg_last_error().decode())
