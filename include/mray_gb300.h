/*
 * mray_gb300.h -- C ABI of the GB300-native MRay ray-tracing hot path.
 *
 * The library (mray_gb300/libmray_gb300.so) replaces the CUDA backend's
 * accelerator slot of MRay's TracerDLL: a GPU-built wide BVH (8-wide,
 * quantised child boxes) traversed in software by hand-written sm_103a
 * kernels.  Every entry point below names the reference interface it stands
 * in for (paths relative to the MRay source tree).
 *
 * Conventions
 *  - Plain C types only; no exceptions cross this boundary.  Every call
 *    returns an mrg_status; mrg_last_error() gives a message for the calling
 *    thread's last failure.
 *  - "d_" pointers are caller-owned DEVICE buffers; "h_" pointers are host
 *    buffers.  Outputs are written in place at the ray's index, like MRay's
 *    Span-based interfaces (Source/Tracer/AcceleratorC.h:375-430).
 *  - stream is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Calls are stream-ordered; the cast calls do not synchronise.
 *  - One context per thread at a time (MRay drives TracerI from a single
 *    tracer thread, Source/MRay/TracerThread.cpp:498).
 */
#ifndef MRAY_GB300_H
#define MRAY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mrg_status
{
    MRG_OK                  = 0,
    MRG_ERR_INVALID_ARG     = 1,   /* null pointer, bad id, size out of range */
    MRG_ERR_CUDA            = 2,   /* a CUDA runtime call failed */
    MRG_ERR_OUT_OF_MEMORY   = 3,
    MRG_ERR_NOT_BUILT       = 4,   /* cast before mrg_build / after a scene change */
    MRG_ERR_LIMIT           = 5,   /* a documented capacity was exceeded */
    MRG_ERR_TRAVERSAL       = 6    /* a kernel reported a stack overflow / step cap */
} mrg_status;

/* RayGMem (Source/Tracer/TracerTypes.h:276-283): 32 bytes, 32-byte aligned. */
typedef struct mrg_ray
{
    float pos[3];
    float tMin;
    float dir[3];
    float tMax;
} mrg_ray;

/* HitKeyPack (Source/Tracer/TracerTypes.h:199-205): 16 bytes.  Key encodings
 * follow Source/Tracer/TracerTypes.h:165-178: PrimitiveKey 4|28,
 * LightOrMatKey 1|10|21, TransformKey 8|24, AcceleratorKey 12|20 (batch|id). */
typedef struct mrg_hit_keys
{
    uint32_t primKey;
    uint32_t lightOrMatKey;
    uint32_t transKey;
    uint32_t accelKey;
} mrg_hit_keys;

/* MetaHit of a triangle hit (PrimitiveDefaultTriangle.h:32): the first two
 * barycentrics in MRay's order (w, u) with w = 1 - u - v. */
typedef struct mrg_meta_hit
{
    float bary[2];
} mrg_meta_hit;

/* Triangle test of a context's casts.  MRG_TRI_MOLLER_TRUMBORE (0, the
 * default) is MRay's Ray::IntersectsTriangle (Source/Core/Ray.hpp:121-167),
 * bit for bit.  MRG_TRI_WATERTIGHT (1) has no counterpart in the reference:
 * the watertight test of Woop, Benthin and Wald (JCGT 2013), under which a ray
 * through an edge shared by two triangles hits one of them; same outputs
 * (t > 1e-7, MetaHit weights of v0 and v1, back-face culling), but hits can
 * differ from MRay's on edges and at grazing angles. */
#define MRG_TRI_MOLLER_TRUMBORE 0u
#define MRG_TRI_WATERTIGHT      1u

typedef struct mrg_params
{
    int      device;           /* CUDA device ordinal */
    uint32_t triangle_test;    /* MRG_TRI_* */
    uint32_t reserved[6];
} mrg_params;

/* Accelerator figures: BaseAcceleratorI::GPUMemoryUsage, TotalAccelCount,
 * TotalInstanceCount (Source/Tracer/AcceleratorC.h:425-428) and build data. */
typedef struct mrg_accel_stats
{
    uint64_t blasNodes;        /* 8-wide nodes over all BLASes */
    uint64_t blasTriangles;    /* triangle records */
    uint64_t tlasNodes;
    uint64_t instances;        /* TotalInstanceCount */
    uint64_t deviceBytes;      /* accelerator bytes resident on the device (GPUMemoryUsage) */
    double   buildMs;          /* last mrg_build wall time */
    uint64_t accelerators;     /* BLASes, one per uploaded mesh (TotalAccelCount) */
} mrg_accel_stats;

typedef struct mrg_ctx mrg_ctx;

/* Instance flags. */
#define MRG_INSTANCE_CULL_BACKFACE 0x1u   /* cullFaceFlags, default on (SceneLoaderMRay/JsonNode.hpp:31-32) */
/* MRay's Matrix3x4::Inverse stores +s1 for the [1][2] element whose cofactor
 * is -s1 (Source/Core/Matrix.hpp:888), so its world->local transform is wrong
 * for rotations with m0*m6 != m2*m4.  By default the inverse reproduces that
 * arithmetic bit for bit (parity with MRay); this flag negates the element. */
#define MRG_INSTANCE_CORRECTED_INVERSE 0x2u

/* Context.  Replaces ConstructTracer / DestroyTracer for the accelerator
 * slot (Source/TracerDLL/EntryPoint.h:12-18, Source/TracerDLL/EntryPoint.cpp:4-13)
 * and the BaseAcceleratorLBVH constructor (Source/Tracer/AcceleratorLBVH.h:236-330). */
mrg_status mrg_create(const mrg_params* params, mrg_ctx** out_ctx);
mrg_status mrg_destroy(mrg_ctx* ctx);
const char* mrg_last_error(void);
const char* mrg_status_string(mrg_status s);

/* Upload an indexed triangle mesh (host pointers, copied).  Replaces
 * PrimGroupTriangle attribute pushes (TracerI::PushPrimAttribute,
 * Source/Core/TracerI.h:209-219; TriangleData, PrimitiveDefaultTriangle.h:22-30).
 * Primitive keys of the mesh are prim_key_base + local triangle index. */
mrg_status mrg_upload_mesh(mrg_ctx* ctx, const float* h_pos, uint32_t vertex_count,
                           const uint32_t* h_idx, uint32_t triangle_count,
                           uint32_t prim_key_base, uint32_t* out_mesh_id);

/* Add an instance of a mesh with a row-major 3x4 local-to-world transform.
 * Replaces CreateSurface + TransformGroupSingle pushes (TracerI.h:270-281;
 * Source/Tracer/TransformsDefault.h:13-17).  The inverse is computed here
 * with MRay's Matrix3x4::Inverse arithmetic (Source/Core/Matrix.hpp:855-904);
 * see MRG_INSTANCE_CORRECTED_INVERSE. */
mrg_status mrg_add_instance(mrg_ctx* ctx, uint32_t mesh_id, const float m3x4[12],
                            uint32_t flags, uint32_t light_or_mat_key,
                            uint32_t trans_key, uint32_t accel_key,
                            uint32_t* out_instance_id);

/* Build every BLAS and the TLAS on the GPU.  Replaces
 * BaseAccelerator::Construct (Source/Tracer/AcceleratorCommon.cu:709-805)
 * + AllocateForTraversal (Source/Tracer/AcceleratorLBVH.cu:742-758).
 * Synchronous. */
mrg_status mrg_build(mrg_ctx* ctx);

/* Local cast.  Replaces BaseAcceleratorI::CastLocalRays
 * (Source/Tracer/AcceleratorC.h:407-421; KCLocalRayCast,
 * Source/Tracer/AcceleratorWork.kt.h:179-244).  For i in [0, n):
 * r = d_ray_idx ? d_ray_idx[i] : i; ray r is cast against instance
 * d_inst_ids[i] only (its BLAS, in the instance's local space, no instance-box
 * test).  Writes as mrg_cast_closest (instance keys of d_inst_ids[i]).  An id
 * >= the instance count skips the ray; mrg_sync_status reports it. */
mrg_status mrg_cast_local(mrg_ctx* ctx, mrg_ray* d_rays, const uint32_t* d_ray_idx,
                          const uint32_t* d_inst_ids, uint32_t n, mrg_hit_keys* d_hits,
                          mrg_meta_hit* d_meta, void* stream);

/* Closest hit.  Replaces BaseAcceleratorI::CastRays
 * (Source/Tracer/AcceleratorC.h:391-398; Source/Tracer/AcceleratorLBVH.cu:760-896).
 * For i in [0, n): r = d_ray_idx ? d_ray_idx[i] : i.  On a hit in
 * [tMin, tMax): d_hits[r], d_meta[r] and d_rays[r].tMax are written; misses
 * leave all three untouched.  d_rays must be 32-byte aligned. */
mrg_status mrg_cast_closest(mrg_ctx* ctx, mrg_ray* d_rays, const uint32_t* d_ray_idx,
                            uint32_t n, mrg_hit_keys* d_hits, mrg_meta_hit* d_meta,
                            void* stream);

/* Any hit (occlusion).  Replaces BaseAcceleratorI::CastVisibilityRays
 * (Source/Tracer/AcceleratorC.h:400-405; Source/Tracer/AcceleratorLBVH.cu:898-1035).
 * Bit r of d_visible_bits is set for every listed ray, then cleared if any
 * hit lies in [tMin, tMax). */
mrg_status mrg_cast_visibility(mrg_ctx* ctx, uint32_t* d_visible_bits,
                               const mrg_ray* d_rays, const uint32_t* d_ray_idx,
                               uint32_t n, void* stream);

/* Closest hit on HOST buffers: copies h_rays to the device, casts, copies the
 * hits, meta hits and updated rays back, and synchronises.  The staging
 * buffers are owned by the context and grow to the largest n seen. */
mrg_status mrg_cast_closest_host(mrg_ctx* ctx, mrg_ray* h_rays, uint32_t n,
                                 mrg_hit_keys* h_hits, mrg_meta_hit* h_meta);

/* Closest hit on HOST buffers without any device allocation.  No
 * counterpart in the reference.  For callers that cannot call cudaMalloc
 * when they cast (an application whose own allocator owns all device memory,
 * or a real-time / plugin thread that may not grow the device heap): the
 * device staging for rays, hit keys and meta hits plus the kernel's work
 * counter and error flag live in one static __device__ array of the library
 * (about 14 MiB).  The driver allocates that array on a device when the
 * library's module loads there; mrg_create forces the load and looks up the
 * array's device address (with the device current), so the array is resident
 * from the first context on a device until the process exits.  The call
 * itself calls no cudaMalloc / cudaFree and nothing that allocates.
 *  - n must be <= MRG_NOALLOC_MAX_RAYS, otherwise MRG_ERR_LIMIT;
 *  - the device address is cached per process and refreshed by every
 *    mrg_create; after a device reset (cudaDeviceReset or a primary-context
 *    reset by the application) contexts created before the reset are invalid
 *    and a new one must be created;
 *  - every call shares the one array and leaves its contents behind, so calls
 *    that overlap on the GPU (other threads, other contexts on the same
 *    device) race: serialise them.
 * Same semantics and results as mrg_cast_closest_host; synchronous. */
#define MRG_NOALLOC_MAX_RAYS 262144u
mrg_status mrg_cast_closest_host_noalloc(mrg_ctx* ctx, mrg_ray* h_rays, uint32_t n,
                                         mrg_hit_keys* h_hits, mrg_meta_hit* h_meta);

/* World-space AABB of the scene (BaseAcceleratorI::SceneAABB,
 * Source/Tracer/AcceleratorC.h:416): min xyz, max xyz; the union of every
 * instance's TransformAABB of its mesh box, as MRay computes it (the TLAS
 * itself uses slightly padded boxes). */
mrg_status mrg_scene_aabb(mrg_ctx* ctx, float out_minmax[6]);

mrg_status mrg_get_stats(mrg_ctx* ctx, mrg_accel_stats* out);

/* Synchronises `stream` and reports (then clears) a traversal error recorded
 * by any cast since the last check: MRG_ERR_TRAVERSAL if a ray overflowed the
 * traversal stack or hit the step cap.  MRay's kernels trap instead
 * (HybridTerminateOrTrap, Source/Core/Definitions.h); here the kernel records
 * the fault, abandons the ray and returns, so the context stays usable. */
mrg_status mrg_sync_status(mrg_ctx* ctx, void* stream);

/* Traversal statistics for the algorithmic-byte count: casts the rays with
 * counters on and returns [0] rays, [1] wide-node visits, [2] triangle tests,
 * [3] instance entries, [4] of [1] in the TLAS, [5] of [3] that found no
 * closer hit, [6..7] zero.  Rays are not modified. */
mrg_status mrg_cast_closest_stats(mrg_ctx* ctx, const mrg_ray* d_rays, uint32_t n,
                                  uint64_t out_counts[8], void* stream);

/* ---------------------------------------------------------------------- */
/* Path tracer (MRay's PathTracerRenderer, RGB; TracerI::CreateRenderer /   */
/* PushRendererAttribute / DoRenderWork, Source/Core/TracerI.h:331-376;     */
/* options Source/TracerDLL/PathTracerRendererShaders.h:36-45)              */
/* ---------------------------------------------------------------------- */
#define MRG_PT_PURE     0u   /* SampleMode "Pure" */
#define MRG_PT_NEE      1u   /* "WithNextEventEstimation" */
#define MRG_PT_NEE_MIS  2u   /* "WithNEEAndMIS" */

typedef struct mrg_pt_params
{
    uint32_t width, height;      /* film size */
    uint32_t spp;                /* samples per pixel rendered by this call */
    uint32_t samplesPerPass;     /* paths in flight = width * height * samplesPerPass (0 = auto) */
    uint32_t rrStart, maxDepth;  /* russianRouletteRange (RR from rrStart, paths end at maxDepth) */
    uint32_t sampleMode;         /* MRG_PT_* */
    uint32_t seed;
    float    filterRadius;       /* Gaussian film filter radius in pixels (MRay default 1) */
    float    camPos[3];          /* pinhole camera: position, gaze point, up */
    float    camGaze[3];
    float    camUp[3];
    float    fov[2];             /* radians, x and y */
    float    nearFar[2];
    uint32_t sampleStart;        /* index of the first sample (continue an accumulation) */
    uint32_t partitionByMaterial;/* group paths by work key (miss, light, material
                                    group) before every shade, as MRay's
                                    RayPartitioner does: 1 always, 0 never
                                    (shade in hit order), 2 when the scene has
                                    more than one material group or a skysphere */
    uint32_t sampler;            /* MRG_PT_SAMPLER_*: the paths' random numbers */
    uint32_t samplerMaxSpp;      /* ZSobol initialMaxSampleCount (0: sampleStart + spp) */
} mrg_pt_params;
/* Samplers (TracerParameters::samplerType, Source/Core/TracerI.h:56):
 * counter-based independent numbers (the default), or MRay's ZSobol group (see
 * mrg_zsobol_generate) with seeds from params.seed. */
#define MRG_PT_SAMPLER_INDEPENDENT 0u
#define MRG_PT_SAMPLER_ZSOBOL      1u
/* ZSobol with the scrambled value bit-reversed back (Laine-Karras Owen
 * scrambling as published), which keeps the Sobol points' stratification that
 * MRay's ScambleOwenFast (Source/Tracer/Random.cu:141-150) loses. */
#define MRG_PT_SAMPLER_ZSOBOL_OWEN 2u
/* MRay's independent group (RNGGroupIndependent, Source/Tracer/Random.cu:
 * 661-726): one PCG32 stream per pixel (PermutedCG32, Source/Tracer/Random.h:
 * 235-266), its state GenerateState(i-th output of std::mt19937(seed32)),
 * seed32 = params.seed.  Number k of bounce b of sample s is the stream's
 * number at position ((s * (maxDepth + 1) + b) * 16 + k), so that a sample
 * reads the same numbers however the film is split into passes;
 * (sampleStart + spp) * (maxDepth + 1) * 16 must not exceed 2^32. */
#define MRG_PT_SAMPLER_PCG32       3u

/* Surface description of an instance, the equivalent of attaching a
 * material / light group to a surface (TracerI::CreateSurface, CreateLightSurface).
 * Rendering requires trans_key index = instance id and dense primitive keys. */
mrg_status mrg_pt_set_lambert(mrg_ctx* ctx, uint32_t instance_id, const float albedo[3]);

/* Material groups (Source/Tracer/MaterialsDefault.h): Lambert, Reflect,
 * Refract (smooth dielectric; RGB uses the first Cauchy coefficient as the
 * index of refraction, front / back), Unreal (GGX metallic-roughness).
 * Refracting surfaces need their instance added without back-face culling. */
#define MRG_MAT_LAMBERT 0u
#define MRG_MAT_REFLECT 1u
#define MRG_MAT_REFRACT 2u
#define MRG_MAT_UNREAL  3u
typedef struct mrg_pt_material
{
    uint32_t type;               /* MRG_MAT_* */
    float    albedo[3];
    float    roughness, metallic, specular;
    float    iorFront, iorBack;
} mrg_pt_material;
mrg_status mrg_pt_set_material(mrg_ctx* ctx, uint32_t instance_id, const mrg_pt_material* material);
mrg_status mrg_pt_set_area_light(mrg_ctx* ctx, uint32_t instance_id, const float radiance[3],
                                 uint32_t two_sided);

/* ---- Ray partitioning ---------------------------------------------------- */
/* RayPartitioner::MultiPartition (Source/Tracer/RayPartitioner.cu:263-411):
 * a stable sort of the n (key, index) pairs by the key's batch bits and, unless
 * only_sort_for_batches, its data bits below them (bit ranges [begin, end)),
 * then the runs of equal batch bits: *d_partition_count runs, run i starting at
 * d_partition_offsets[i] with key d_partition_keys[i] (the sorted key there),
 * and d_partition_offsets[count] = n.  Entries past max_partitions are not
 * written (the count is still exact; offsets[count] is written only when
 * count <= max_partitions).  d_indices == NULL sorts the identity 0..n-1.
 * Inputs are not modified.  Device buffers; stream-ordered, no host
 * synchronisation.  n <= 2^28. */
mrg_status mrg_multi_partition(mrg_ctx* ctx, const uint32_t* d_keys, const uint32_t* d_indices, uint32_t n,
                               const uint32_t key_data_bits[2], const uint32_t key_batch_bits[2],
                               uint32_t only_sort_for_batches,
                               uint32_t* d_sorted_keys, uint32_t* d_sorted_indices,
                               uint32_t* d_partition_count, uint32_t* d_partition_offsets,
                               uint32_t* d_partition_keys, uint32_t max_partitions, void* stream);

/* Per-vertex texture coordinates of a mesh (the triangle group's "uv"
 * attribute, PrimitiveDefaultTriangle.h:22-30): nv x 2 floats, nv equal to
 * the mesh's vertex count. */
mrg_status mrg_upload_mesh_uv(mrg_ctx* ctx, uint32_t mesh_id, const float* uv, uint32_t nv);

/* An albedo texture: width x height RGBA texels, format 0 = UNORM8 (read as
 * v / 255) or 1 = f32; bilinear, wrap addressed, one mip level (MRay's
 * default "Linear" / "Wrap" texture, Docs/markdown/scene/mrayScene.md:76-77).
 * borrow = 0 copies host texels; borrow = 1 keeps the DEVICE pointer, which
 * must stay valid and may be rewritten between renders (a parameter texture
 * being optimised). */
#define MRG_TEX_RGBA8 0u
#define MRG_TEX_RGBA32F 1u
mrg_status mrg_pt_add_texture(mrg_ctx* ctx, uint32_t width, uint32_t height, uint32_t format,
                              const void* texels, uint32_t borrow, uint32_t* texture_id);
/* The instance's albedo comes from the texture at the hit's interpolated uv
 * (its mesh needs uvs); texture_id = 0xFFFFFFFF returns to the constant. */
mrg_status mrg_pt_set_albedo_texture(mrg_ctx* ctx, uint32_t instance_id, uint32_t texture_id);
/* Unreal's texturable parameters (UnrealMatData's roughness, metallic and
 * specular ParamVaryingData, Source/Tracer/MaterialsDefault.h:151-160; read in
 * UnrealMaterial's constructor, MaterialsDefault.hpp:521-533): each texture's
 * first channel at the hit's uv (RGBA8: v / 255), read like the albedo
 * (level 0, or the ray cone's level when the texture has a mip chain),
 * replaces the instance's constant.  0xFFFFFFFF keeps the constant; the mesh
 * needs uvs; instances of other materials ignore them. */
mrg_status mrg_pt_set_unreal_textures(mrg_ctx* ctx, uint32_t instance_id, uint32_t roughness_texture,
                                      uint32_t metallic_texture, uint32_t specular_texture);
/* A mip chain for a texture (TextureMemory::GenerateMipmaps with the tracer's
 * mipGenFilter, Source/Tracer/TextureMemory.cpp:491-525,
 * TextureFilter.cu:124-192, 1006-1100): every level down to 1 x 1, each texel
 * the normalised sum of 8 x 8 stratified samples of the level above weighted
 * by a Gaussian filter of filter_radius pixels (MRay's default 2), in the
 * texture's own format.  Made on the device at the next render (from the
 * texels of that moment, for a borrowed texture); filter_radius = 0 drops the
 * chain.  Reads of a texture with a chain take their level from the path's ray
 * cone (RT Gems I ch. 20; the camera's cone, widened along the path and
 * refracted by smooth dielectrics, projected on the hit triangle for uv
 * gradients) and blend the two nearest levels (TextureViewCPU's trilinear
 * read, the gradients in texels).  mrg_pt_adjoint's texture parameter must have
 * no chain. */
mrg_status mrg_pt_generate_mips(mrg_ctx* ctx, uint32_t texture_id, float filter_radius);
/* Texels of one mip level of a texture (TracerI::PushTextureData with
 * mipLevel > 0, Source/Core/TracerI.h:243): level in [1, bits(max(w, h))),
 * max(w >> level, 1) x max(h >> level, 1) texels in the texture's format,
 * copied.  A given level is kept when the chain is generated (MRay's
 * validMips, TextureFilter.cu:160-164) and the levels below it are filtered
 * from it; without a generation filter the chain ends at the last given
 * level, and every level up to it must be given (else the next render fails). */
mrg_status mrg_pt_set_texture_mip(mrg_ctx* ctx, uint32_t texture_id, uint32_t level, const void* texels);

/* ---- Path-replay adjoint (no reference counterpart) ---------------------- */
/* Gradient of  sum_pixels <d_image_adjoint[p].rgb, I[p].rgb>  with respect to
 * the RGB texels of f32 texture texture_id (a Lambert albedo) and to the RGB
 * radiance of every area light, I being the image of params (RGB mode):
 * I[p] = (sum of the pixel's spp sample radiances) / spp.  Each pass runs
 * twice with the same paths (counter-based random numbers): the primal records
 * every path's radiance, the replay adds at every vertex on the texture
 * d * (radiance after the vertex) / albedo  into the four texels of its
 * bilinear read (Vicini et al. 2021, "Path Replay Backpropagation"), and, for
 * every emission it gathers (a light hit, or a visible NEE sample), d * (the
 * contribution / the light's radiance) into the light's instance.
 * d_grad (RGBA f32 per texel, A unused) and d_grad_emission (RGBA f32 per
 * instance, A unused; entries of instances that are not area lights stay
 * untouched) are ADDED to (atomics).  texture_id = MRG_PT_NO_TEXTURE asks for
 * the emission gradient alone (d_grad may then be NULL); d_grad_emission =
 * NULL skips it.  Russian roulette probabilities are treated as constants.
 * When d_image is not NULL the primal image is accumulated into it as
 * mrg_pt_render does.  Device buffers, stream-ordered. */
#define MRG_PT_NO_TEXTURE 0xFFFFFFFFu
mrg_status mrg_pt_adjoint(mrg_ctx* ctx, const mrg_pt_params* params, uint32_t texture_id,
                          const float* d_image_adjoint, float* d_grad, float* d_grad_emission, float* d_image,
                          void* stream);

/* ---- ZSobol random numbers ---------------------------------------------------
 * MRay's RNGGroupZSobol (Source/Tracer/Random.h:454-523, Random.cu:1147-1380):
 * mrg_zsobol_seeds replaces its constructor's per-pixel seeds (the i-th output
 * of std::mt19937 seeded with (seed >> 32) ^ (seed & 0xFFFFFFFF), pixels in
 * row-major order, Random.cu:1149-1230) for a width x height image.
 * mrg_zsobol_generate replaces GenerateNumbers (KCGenRandomNumbersGeneric,
 * Random.cu:536-556) for one sample index of every pixel: `requests` is an
 * RNRequestList (request r = bits 2r..2r+1, 1..3 numbers, request_count of
 * them); request r reads dimension dim_start + (numbers before it) through
 * ZSobol::Next / Next2D / Next3D, and number k of pixel i lands at
 * d_out[i + width * height * k].  initial_max_spp is the group's
 * initialMaxSampleCount.  Device buffers, stream-ordered. */
mrg_status mrg_zsobol_seeds(uint32_t width, uint32_t height, uint64_t seed, uint32_t* h_seeds);
mrg_status mrg_zsobol_generate(uint32_t width, uint32_t height, const uint32_t* d_seeds, uint32_t initial_max_spp,
                               uint32_t sample_index, uint32_t dim_start, uint64_t requests,
                               uint32_t request_count, uint32_t* d_out, void* stream);

/* ---- Radiance cache (no reference counterpart) ----------------------------- */
/* A multiresolution hash grid (levels x 2 features x 2^log2_table_size fp16
 * entries per level, resolutions base..max geometrically) feeding a fully
 * fused MLP of 5 hidden 64-wide ReLU layers and a 16-wide output layer, BF16
 * tensor cores with FP32 accumulation (5 x 64x64 + 16x64 weights, no
 * biases), trained online with
 * Adam on a relative L2 loss.  One cache per context.
 * Per sample 16 floats: position xyz, roughness | outgoing direction xyz, 0 |
 * normal xyz, 0 | albedo rgb, 0; positions are normalised to aabb.  Outputs
 * 4 floats: predicted outgoing radiance rgb, 0. */
typedef struct mrg_cache_params
{
    uint32_t levels;            /* 16 */
    uint32_t log2_table_size;   /* 19 */
    uint32_t base_resolution;   /* 16 */
    uint32_t max_resolution;    /* 2048 */
    float    learning_rate;     /* 1e-2 */
    float    beta1, beta2, epsilon;
    uint32_t seed;              /* initial weights */
    uint32_t max_batch;         /* training samples per step, <= 2^20 */
    float    aabb[6];           /* min xyz, max xyz */
} mrg_cache_params;
mrg_status mrg_cache_create(mrg_ctx* ctx, const mrg_cache_params* params);
mrg_status mrg_cache_query(mrg_ctx* ctx, const float* d_inputs, uint32_t n, float* d_out, void* stream);
/* One Adam step on n <= max_batch samples (targets: 4 floats each, rgb used).
 * h_loss (optional) receives the batch's mean relative L2 loss and makes the
 * call synchronous. */
mrg_status mrg_cache_train(mrg_ctx* ctx, const float* d_inputs, const float* d_targets, uint32_t n,
                           float* h_loss, void* stream);
/* Parameters as fp32 host arrays: 21,504 MLP weights (hidden W0..W4 [64][64]
 * then output W5 [16][64], row-major out x in) and levels * 2^log2_table_size * 2 table
 * features; either pointer may be NULL. */
mrg_status mrg_cache_get_params(mrg_ctx* ctx, float* h_weights, float* h_table);
/* The loss gradients of one batch, without an optimiser step (layouts as
 * mrg_cache_get_params; a gradient check). Synchronous. */
mrg_status mrg_cache_gradients(mrg_ctx* ctx, const float* d_inputs, const float* d_targets, uint32_t n,
                               float* h_grad_weights, float* h_grad_table, float* h_loss);
mrg_status mrg_cache_set_params(mrg_ctx* ctx, const float* h_weights, const float* h_table);

/* Cache-assisted path tracing (Mueller et al. 2021): params->spp samples
 * per pixel, added to d_image as mrg_pt_render does, every path ending at its
 * second vertex on a cache query of the outgoing radiance.  The cache learns
 * RGB radiance; with a spectral context (mrg_pt_set_spectral) a path takes the
 * answer at its 4 wavelengths through the radiance conversion, and its
 * training targets are its wavelength estimates converted to RGB as the film
 * converts a sample.
 * About train_paths of each pass's paths (a hashed sparse subset) are training
 * paths instead: they record vertices 1 and 2 and end at vertex 3 on a cache
 * query (self-training); after the pass their (inputs, outgoing radiance)
 * samples, at most the cache's max_batch, make one mrg_cache_train step.
 * train_paths = 0 renders without training. */
mrg_status mrg_pt_render_cached(mrg_ctx* ctx, const mrg_pt_params* params, float* d_image,
                                uint32_t train_paths, float* h_loss, void* stream);

/* Skysphere boundary light (LightGroupSkysphere<SphericalCoordConverter>,
 * Source/Tracer/LightsDefault.hpp:300-420, 700-915): a lat-long radiance map
 * of width x height RGBA f32 texels (row-major, row 0 at v = 0; 1 x 1 = a
 * constant radiance) and an optional 3x4 transform (NULL = identity; only its
 * rotation is used).  The map is copied; its importance-sampling distribution
 * (luminance, piecewise-constant 2D) is built at the next render.  It joins
 * the uniform light sampler after the area lights and is seen by rays that
 * leave the scene.  width = 0 removes it. */
mrg_status mrg_pt_set_env(mrg_ctx* ctx, uint32_t width, uint32_t height, const float* rgba,
                          const float m3x4[12]);

/* Spectral rendering (SpectrumContextJakob2019, Source/Tracer/SpectrumContext.{h,hpp,cu};
 * SpectraPerSpectrum = 4, hyperbolic wavelength sampling, the renderer's
 * default): lut = the float data of an MR_SPECTRA file (9 * lut_res^3 floats,
 * [table][coefficient][z][y][x]); the CIE 1931 observer (cie_count x 3 from
 * 360 nm in 1 nm steps), its integrals, the colour space's illuminant SPD and
 * normalisation factor, and the XYZ -> RGB matrix (row-major), as MRay's
 * colour tables hold them.  Everything is copied.  lut_res = 0 returns to RGB
 * rendering.  Albedos and emissions stay RGB in the scene description and are
 * converted per path (Converter::ConvertAlbedo / ConvertRadiance). */
mrg_status mrg_pt_set_spectral(mrg_ctx* ctx, uint32_t lut_res, const float* lut, uint32_t cie_count,
                               const float* cie_xyz, const float cie_integrals[3],
                               const float* illuminant_spd, float illuminant_norm,
                               const float xyz_to_rgb[9]);

/* The pinhole frame MRay derives from the camera parameters
 * (CameraPinhole ctor, Source/Tracer/CamerasDefault.hpp:6-30): out = position[3],
 * bottomLeft[3], right[3], up[3], planeSize[2], near, far. */
mrg_status mrg_pt_camera_frame(const mrg_pt_params* params, float out[16]);

/* Renders params->spp samples per pixel and ADDS them to d_image, a device
 * float4 per pixel (R, G, B, filter weight), row 0 at the bottom of the image
 * plane; pixel value = RGB / weight.  Stream-ordered, no host synchronisation
 * inside a pass. */
mrg_status mrg_pt_render(mrg_ctx* ctx, const mrg_pt_params* params, float* d_image, void* stream);

/* ---------------------------------------------------------------------- */
/* Guided path tracing: MRay's GuidedPTRenderer (Markov-chain mixtures     */
/* after Alber et al. 2025 on a spatio-directional hash grid;              */
/* Source/TracerDLL/GuidedPTRenderer.{h,cu}, GuidedPTRendererShaders.h,    */
/* Source/Tracer/HashGrid.{h,cu}).                                         */
/* ---------------------------------------------------------------------- */
/* GuidedPTRDetail::Options (GuidedPTRendererShaders.h:75-133); defaults in
 * parentheses. */
typedef struct mrg_guide_params
{
    uint32_t entryLimit;        /* cacheEntryLimit (2,000,000): the table holds
                                   NextPowerOfTwo(entryLimit / 0.6) codes and
                                   takes new ones up to 60% of them */
    uint32_t posBits;           /* cachePosBits (14), at most 15 */
    uint32_t normalBits;        /* cacheNormalBits (2), at most 3 */
    uint32_t maxLevelOffset;    /* cacheMaxLvlOffset (3) */
    float    coneAperture;      /* cacheConeAperture, degrees (0.6) */
    float    lobeProbability;   /* lobeProbablity (0.75) */
    uint32_t fixZeroWeight;     /* 0 (MRay): a vertex whose chosen lobe has weight 0 (or
                                   that has no lobe) takes GaussLobeMixtureT::Sample's +Y
                                   direction with pdf 0 when it picks the mixture; 1: such
                                   a vertex samples the material only (mixture
                                   probability 0), which removes that bias */
    uint32_t reserved;
} mrg_guide_params;
mrg_status mrg_guide_defaults(mrg_guide_params* out);
/* Allocates the context's grid over the scene box of the last mrg_build
 * (HashGrid::Reset with the accelerator's SceneAABB) and empties it. */
mrg_status mrg_guide_create(mrg_ctx* ctx, const mrg_guide_params* params);
/* Empties the grid, its chains and irradiance averages, and restarts the
 * paths' backup random streams; the next render takes its camera position
 * (HashGrid::ClearAllEntries, SetCameraPos). */
mrg_status mrg_guide_clear(mrg_ctx* ctx);
mrg_status mrg_guide_destroy(mrg_ctx* ctx);
/* Entries in use and the table size.  Synchronous. */
mrg_status mrg_guide_stats(mrg_ctx* ctx, uint32_t* used, uint32_t* table_size);
/* Snapshot of the table: per slot its code (~0: empty), chain state (6
 * floats: target xyz, cosine, weight, sample count) and irradiance average
 * (2 floats: value, sample count).  Any pointer may be NULL.  Synchronous. */
mrg_status mrg_guide_read(mrg_ctx* ctx, uint64_t* h_codes, float* h_chain6, float* h_irr2);
/* Guided rendering: params->spp samples per pixel ADDED to d_image as
 * mrg_pt_render does, learning in the grid as it goes (one pass of
 * samplesPerPass samples per pixel at a time, bounce by bounce).
 * russianRouletteRange = (rrStart, maxDepth); NEE with MIS always (sampleMode
 * is not read); samplers MRG_PT_SAMPLER_INDEPENDENT and MRG_PT_SAMPLER_PCG32.
 * Each path slot (width * height * samplesPerPass of them) has a backup PCG32
 * stream for the grid's choices, its state GenerateState(output
 * width * height + slot of std::mt19937(params.seed)), continued from call to
 * call until mrg_guide_clear.  Irradiance updates of a bounce are applied in
 * a fixed order (path, NEE, light records, slot by slot per cell), so a
 * render is reproducible run to run. */
mrg_status mrg_pt_render_guided(mrg_ctx* ctx, const mrg_pt_params* params, float* d_image, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MRAY_GB300_H */
