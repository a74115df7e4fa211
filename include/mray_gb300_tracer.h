/* mray_gb300_tracer.h -- MRay's TracerI (Source/Core/TracerI.h:150-376) as a
 * C ABI over libmray_gb300.so: scene construction through typed groups,
 * reservations and attribute pushes, surface commit, renderers and render
 * work, with MRay's type names, attribute lists, id layouts and error
 * behaviour for the types this library renders.  The MRay-side class that
 * implements TracerI over these calls is mray_gb300/shim/TracerGB300.h.
 *
 * Types (TypeNameGenerators.h prefixes; TracerConstants.h implicit groups):
 *   primitives  (P)Triangle                 PrimitiveDefaultTriangle.{h,cu}
 *               (P)Empty                    implicit group 0
 *   materials   (Mt)Lambert (Mt)Reflect (Mt)Refract (Mt)Unreal   MaterialsDefault.{h,cpp}
 *               (Mt)Passthrough             implicit group 0 (not renderable here)
 *   transforms  (T)Identity (implicit group 0, id 0)  (T)Single   TransformsDefault.{h,cu}
 *   lights      (L)Null (implicit group 0, id 0)  (L)Prim(P)Triangle  (L)Skysphere_Spherical
 *                                           LightsDefault.{h,hpp,cu}
 *   cameras     (C)Pinhole                  CamerasDefault.{h,cpp}
 *   media       (Md)Vacuum                  implicit group 0, nothing else
 *   renderers   (R)PathTracerRGB (R)PathTracerSpectral   TracerDLL/PathTracerRenderer.{h,cu}
 *
 * Ids are MRay's keys (Source/Tracer/TracerTypes.h:168-174): a primitive
 * batch id is group << 28 | index, a material or light id group << 21 |
 * index, a transform or camera id group << 24 | index; texture ids count
 * from 1 (0 is TracerConstants::InvalidTexture); surface, light-surface,
 * camera-surface and renderer ids count from 0.
 *
 * Everything before mrg_tracer_commit_surfaces is host bookkeeping (no
 * device call); the commit creates the device context, uploads meshes,
 * builds the accelerator and sets the path tracer's surfaces.  Each call
 * returns MRG_OK or an error status with mrg_last_error() set, where MRay
 * throws MRayError.  Calls on one tracer may come from several threads
 * (MRay's scene loader pushes attributes from its thread pool). */
#ifndef MRAY_GB300_TRACER_H
#define MRAY_GB300_TRACER_H

#include "mray_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mrg_tracer mrg_tracer;

/* TracerParameters (Source/Core/TracerI.h:45-68), the fields this tracer
 * reads.  A zeroed struct is MRay's defaults on device 0. */
#define MRG_TRACER_SAMPLER_INDEPENDENT 0u   /* MRay's PCG32 group: MRG_PT_SAMPLER_PCG32 */
#define MRG_TRACER_SAMPLER_ZSOBOL      1u   /* MRG_PT_SAMPLER_ZSOBOL */
typedef struct mrg_tracer_params
{
    uint64_t seed;               /* seed (the samplers use hi ^ lo) */
    int      device;             /* CUDA device ordinal */
    uint32_t samplerType;        /* MRG_TRACER_SAMPLER_* */
    float    filmFilterRadius;   /* filmFilter: Gaussian of this radius; 0 = MRay's default 1 */
    uint32_t triangleTest;       /* MRG_TRI_* (MRay: Moller-Trumbore) */
    uint32_t genMips;            /* genMips: every texture gets its full mip chain */
    float    mipGenFilterRadius; /* mipGenFilter: Gaussian of this radius; 0 = MRay's default 2 */
    uint32_t reserved[2];
} mrg_tracer_params;

/* ConstructTracer / DestroyTracer (Source/TracerDLL/EntryPoint.h:12-18). */
mrg_status mrg_tracer_create(const mrg_tracer_params* params, mrg_tracer** out);
mrg_status mrg_tracer_destroy(mrg_tracer* t);
/* Parameters() */
mrg_status mrg_tracer_parameters(const mrg_tracer* t, mrg_tracer_params* out);

/* ---- Generic: type lists and attribute information ----------------------- */
#define MRG_KIND_PRIM     0u
#define MRG_KIND_MATERIAL 1u
#define MRG_KIND_TRANSFORM 2u
#define MRG_KIND_CAMERA   3u
#define MRG_KIND_MEDIUM   4u
#define MRG_KIND_LIGHT    5u
#define MRG_KIND_RENDERER 6u

/* PrimitiveGroups() ... Renderers(): the creatable type names of a kind,
 * '\n'-separated, NUL-terminated into buf (cap bytes); *need = bytes needed. */
mrg_status mrg_tracer_type_names(const mrg_tracer* t, uint32_t kind, char* buf, size_t cap, size_t* need);

/* MRayDataEnum members the attributes use (Source/Core/MRayDataType.h). */
#define MRG_DT_FLOAT      0u
#define MRG_DT_VECTOR_2   1u
#define MRG_DT_VECTOR_3   2u
#define MRG_DT_VECTOR_4   3u
#define MRG_DT_QUATERNION 4u
#define MRG_DT_MATRIX_4x4 5u
#define MRG_DT_UINT32     6u
#define MRG_DT_VECTOR_2UI 7u
#define MRG_DT_VECTOR_3UI 8u
#define MRG_DT_BOOL       9u
#define MRG_DT_STRING     10u
/* AttributeTexturable */
#define MRG_ATTR_CONSTANT_ONLY       0u
#define MRG_ATTR_TEXTURE_OR_CONSTANT 1u
#define MRG_ATTR_TEXTURE_ONLY        2u
typedef struct mrg_tracer_attrib_info
{
    char     name[32];
    uint32_t dataType;           /* MRG_DT_* */
    uint32_t elementBytes;       /* bytes per item (0 for strings) */
    uint32_t optional;           /* AttributeOptionality: 1 = MR_OPTIONAL */
    uint32_t texturable;         /* MRG_ATTR_* */
    uint32_t isColor;            /* AttributeIsColor */
} mrg_tracer_attrib_info;
/* AttributeInfoPrim / Mat / Trans / Cam / Light / Renderer(typeName):
 * attribute `index` of the type, MRG_ERR_INVALID_ARG past the last;
 * *count (optional) = the type's attribute count. */
mrg_status mrg_tracer_attribute_info(const mrg_tracer* t, uint32_t kind, const char* type_name, uint32_t index,
                                     mrg_tracer_attrib_info* out, uint32_t* count);
/* TypeName(PrimGroupId) ... TypeName(RendererId) */
mrg_status mrg_tracer_group_type_name(const mrg_tracer* t, uint32_t kind, uint32_t group_id,
                                      char* buf, size_t cap);

/* ---- Primitives ------------------------------------------------------------ */
mrg_status mrg_tracer_create_prim_group(mrg_tracer* t, const char* type_name, uint32_t* group_id);
/* ReservePrimitiveBatches: counts = n pairs (primCount, attributeCount), the
 * PrimCount struct (Source/Core/TracerAttribInfo.h:45). */
mrg_status mrg_tracer_reserve_prim_batches(mrg_tracer* t, uint32_t group_id, const uint32_t* counts, uint32_t n,
                                           uint32_t* batch_ids);
mrg_status mrg_tracer_commit_prim_reservations(mrg_tracer* t, uint32_t group_id);
mrg_status mrg_tracer_is_prim_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out);
/* PushPrimAttribute: the whole batch when sub_begin == sub_end == 0, else
 * items [sub_begin, sub_end) of it (the subBatchRange overload).  Triangle
 * attributes: 0 position (vector3 x attributeCount), 1 normal (quaternion,
 * tangent space; accepted, the renderer shades with geometric normals),
 * 2 uv0 (vector2), 3 index (vector3ui x primCount, batch-local vertices). */
mrg_status mrg_tracer_push_prim_attribute(mrg_tracer* t, uint32_t group_id, uint32_t batch_id,
                                          uint32_t attribute_index, uint32_t sub_begin, uint32_t sub_end,
                                          const void* data, size_t bytes);
/* TransformPrimitives: positions of each batch multiplied in place by its
 * row-major 3x4 matrix (12 floats per batch); normals are not rotated. */
mrg_status mrg_tracer_transform_primitives(mrg_tracer* t, uint32_t group_id, const uint32_t* batch_ids,
                                           const float* m3x4, uint32_t n);

/* ---- Materials, transforms, lights, cameras: reservations and pushes ------ */
/* Reserve*: n items of the group; ids written to ids[0..n) (consecutive).
 * Light reservations of a primitive-backed group name each light's
 * primitive batch (prim_batches, n ids); other light groups pass NULL.
 * Push*Attribute covers ids [id_begin, id_end] of one group (MRay's
 * CommonIdRange, inclusive ends as SceneLoaderMRay passes them): data holds
 * id_end - id_begin + 1 items; textures, where not NULL, holds one texture id
 * per item (0 = use the constant) for a texturable attribute, and data may be
 * NULL for a texture-only one. */
mrg_status mrg_tracer_create_mat_group(mrg_tracer* t, const char* type_name, uint32_t* group_id);
mrg_status mrg_tracer_reserve_materials(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids);
mrg_status mrg_tracer_commit_mat_reservations(mrg_tracer* t, uint32_t group_id);
mrg_status mrg_tracer_is_mat_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out);
mrg_status mrg_tracer_push_mat_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                         uint32_t attribute_index, const void* data, size_t bytes,
                                         const uint32_t* textures);

mrg_status mrg_tracer_create_trans_group(mrg_tracer* t, const char* type_name, uint32_t* group_id);
mrg_status mrg_tracer_reserve_transforms(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids);
mrg_status mrg_tracer_commit_trans_reservations(mrg_tracer* t, uint32_t group_id);
mrg_status mrg_tracer_is_trans_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out);
/* (T)Single attribute 0: a row-major 4x4 matrix per item. */
mrg_status mrg_tracer_push_trans_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                           uint32_t attribute_index, const void* data, size_t bytes);

mrg_status mrg_tracer_create_light_group(mrg_tracer* t, const char* type_name, uint32_t prim_group_id,
                                         uint32_t* group_id);
mrg_status mrg_tracer_reserve_lights(mrg_tracer* t, uint32_t group_id, uint32_t n, const uint32_t* prim_batches,
                                     uint32_t* ids);
mrg_status mrg_tracer_commit_light_reservations(mrg_tracer* t, uint32_t group_id);
mrg_status mrg_tracer_is_light_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out);
mrg_status mrg_tracer_push_light_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                           uint32_t attribute_index, const void* data, size_t bytes,
                                           const uint32_t* textures);

mrg_status mrg_tracer_create_camera_group(mrg_tracer* t, const char* type_name, uint32_t* group_id);
mrg_status mrg_tracer_reserve_cameras(mrg_tracer* t, uint32_t group_id, uint32_t n, uint32_t* ids);
mrg_status mrg_tracer_commit_cam_reservations(mrg_tracer* t, uint32_t group_id);
mrg_status mrg_tracer_is_cam_committed(const mrg_tracer* t, uint32_t group_id, uint32_t* out);
/* (C)Pinhole: 0 FovAndPlanes (vector4: fov x, fov y in radians, near, far),
 * 1 gaze (a point), 2 position, 3 up. */
mrg_status mrg_tracer_push_cam_attribute(mrg_tracer* t, uint32_t group_id, uint32_t id_begin, uint32_t id_end,
                                         uint32_t attribute_index, const void* data, size_t bytes);

/* ---- Textures ------------------------------------------------------------- */
/* MRayPixelEnum members accepted (Source/Core/MRayDataType.h). */
#define MRG_PIX_RGBA8_UNORM 0u
#define MRG_PIX_RGB_FLOAT   1u
#define MRG_PIX_RGBA_FLOAT  2u
#define MRG_PIX_R8_UNORM    3u   /* single channel: read as (r, r, r, 1) */
#define MRG_PIX_R_FLOAT     4u
/* CreateTexture2D: colour space, gamma and read mode are not applied
 * (texels are taken as linear values of the renderer's colour space);
 * filtering is bilinear with wrap addressing on mip 0, the data of further
 * mips is accepted and not read. */
mrg_status mrg_tracer_create_texture2d(mrg_tracer* t, uint32_t width, uint32_t height, uint32_t mip_count,
                                       uint32_t pixel_type, uint32_t* texture_id);
mrg_status mrg_tracer_commit_textures(mrg_tracer* t);
mrg_status mrg_tracer_push_texture_data(mrg_tracer* t, uint32_t texture_id, uint32_t mip_level,
                                        const void* data, size_t bytes);

/* ---- Surfaces --------------------------------------------------------------- */
#define MRG_TRACER_MAX_BATCHES_PER_SURFACE 8u   /* TracerConstants::MaxPrimBatchPerSurface */
typedef struct mrg_tracer_surface
{
    uint32_t count;                                        /* primitive batches */
    uint32_t primBatches[MRG_TRACER_MAX_BATCHES_PER_SURFACE];
    uint32_t materials[MRG_TRACER_MAX_BATCHES_PER_SURFACE];
    uint32_t alphaMaps[MRG_TRACER_MAX_BATCHES_PER_SURFACE];  /* texture id or 0 (none); only 0 is accepted */
    uint32_t cullFace[MRG_TRACER_MAX_BATCHES_PER_SURFACE];   /* back-face culling per batch */
    uint32_t transformId;
} mrg_tracer_surface;
typedef struct mrg_tracer_commit_result   /* SurfaceCommitResult */
{
    float    aabb[6];
    uint64_t instanceCount;
    uint64_t acceleratorCount;
} mrg_tracer_commit_result;
mrg_status mrg_tracer_create_surface(mrg_tracer* t, const mrg_tracer_surface* s, uint32_t* surface_id);
mrg_status mrg_tracer_set_boundary_surface(mrg_tracer* t, uint32_t light_id, uint32_t transform_id,
                                           uint32_t* light_surface_id);
mrg_status mrg_tracer_create_light_surface(mrg_tracer* t, uint32_t light_id, uint32_t transform_id,
                                           uint32_t* light_surface_id);
mrg_status mrg_tracer_create_camera_surface(mrg_tracer* t, uint32_t camera_id, uint32_t transform_id,
                                            uint32_t* cam_surface_id);
mrg_status mrg_tracer_commit_surfaces(mrg_tracer* t, mrg_tracer_commit_result* out);
/* GetCamTransform / SetCameraTransform: CameraTransform = position, gaze
 * point, up (9 floats) in world space. */
mrg_status mrg_tracer_get_cam_transform(const mrg_tracer* t, uint32_t cam_surface_id, float out[9]);

/* ---- Spectral tables -------------------------------------------------------- */
/* The data (PathTracerSpectral) needs, as mrg_pt_set_spectral takes it;
 * copied.  MRay loads the same LUT and colour tables when it creates the
 * spectral renderer's context. */
mrg_status mrg_tracer_set_spectral_data(mrg_tracer* t, uint32_t lut_res, const float* lut, uint32_t cie_count,
                                        const float* cie_xyz, const float cie_integrals[3],
                                        const float* illuminant_spd, float illuminant_norm,
                                        const float xyz_to_rgb[9]);

/* ---- Renderers and rendering ------------------------------------------------ */
/* (R)PathTracerRGB / (R)PathTracerSpectral attributes (PathTracerRenderer.cu:
 * 1386-1400): 0 totalSPP (uint32), 1 burstSize (uint32, samples per pixel per
 * render work, default 1), 2 renderMode (string "Throughput" | "Latency"),
 * 3 sampleMode (string "Pure" | "WithNextEventEstimation" | "WithNEEAndMIS"),
 * 4 rrRange (vector2ui: Russian roulette from [0], paths end at [1]),
 * 5 neeSamplerType (string "Uniform").  Strings are passed as their bytes. */
mrg_status mrg_tracer_create_renderer(mrg_tracer* t, const char* type_name, uint32_t* renderer_id);
mrg_status mrg_tracer_destroy_renderer(mrg_tracer* t, uint32_t renderer_id);
mrg_status mrg_tracer_push_renderer_attribute(mrg_tracer* t, uint32_t renderer_id, uint32_t attribute_index,
                                              const void* data, size_t bytes);

typedef struct mrg_tracer_render_info     /* RenderBufferInfo, the parts a caller reads */
{
    uint32_t width, height;      /* film resolution */
    uint32_t totalSpp;
    uint32_t channels;           /* 4: R, G, B, filter weight */
    const float* d_film;         /* device film, row 0 at the bottom of the image plane */
} mrg_tracer_render_info;
/* StartRender(renderer, camera surface, RenderImageParams, ...): the region
 * must be the whole film. */
mrg_status mrg_tracer_start_render(mrg_tracer* t, uint32_t renderer_id, uint32_t cam_surface_id,
                                   uint32_t width, uint32_t height, const uint32_t region_min[2],
                                   const uint32_t region_max[2], mrg_tracer_render_info* out);
mrg_status mrg_tracer_set_camera_transform(mrg_tracer* t, uint32_t renderer_id, const float cam[9]);
typedef struct mrg_tracer_render_output   /* RendererOutput, the parts a caller reads */
{
    uint32_t samplesDone;        /* samples per pixel accumulated so far */
    uint32_t totalSpp;
    uint32_t finished;           /* samplesDone == totalSpp */
    float    workMs;             /* device time of this render work */
    double   pathsPerSecond;     /* paths of this work / workMs (MRay's "M paths/s" x 1e6) */
} mrg_tracer_render_output;
/* DoRenderWork: burstSize more samples per pixel (none once finished). */
mrg_status mrg_tracer_do_render_work(mrg_tracer* t, mrg_tracer_render_output* out);
/* The film as RGBA float32 (R, G, B, weight), width x height, to host memory. */
mrg_status mrg_tracer_read_film(mrg_tracer* t, float* h_rgbw, size_t bytes);
mrg_status mrg_tracer_stop_render(mrg_tracer* t);

/* ---- Misc ------------------------------------------------------------------- */
mrg_status mrg_tracer_clear_all(mrg_tracer* t);
mrg_status mrg_tracer_flush(const mrg_tracer* t);
/* TotalDeviceMemory / UsedDeviceMemory (0 before the device is used). */
mrg_status mrg_tracer_device_memory(const mrg_tracer* t, uint64_t* total, uint64_t* used);
/* The accelerator / path-tracer context behind the tracer (NULL before the
 * surface commit), for the calls with no TracerI counterpart (casts, the
 * radiance cache, the adjoint). */
mrg_ctx* mrg_tracer_context(mrg_tracer* t);

#ifdef __cplusplus
}
#endif

#endif /* MRAY_GB300_TRACER_H */
