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
    }
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
