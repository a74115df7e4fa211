/*
 * mrg_oracle.h -- CPU oracle for the mray_gb300 ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the mray_gb300 package
 * and its CUDA library) links, loads or calls this code.  Only tests/,
 * __graft_entry__.smoke() (as the checker) and bench.py's CPU-baseline /
 * reference arm use it.
 *
 * It restates, in plain C, the algorithms of MRay's host (CPU) backend for
 * the software-BVH accelerator and the wavefront path tracer.  Each function
 * cites the reference file:line it follows (paths relative to the MRay source
 * tree).  Floating-point order of operations follows the reference exactly;
 * the reference's Math::FMA / Dot / Cross use std::fma explicitly
 * (Source/Core/Math.h:1367-1380, 1586-1596, 1627-1633), which this file
 * reproduces with fmaf().  Build with -ffp-contract=off so that no other
 * expression is fused.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Layout of RayGMem (Source/Tracer/TracerTypes.h:276-283): 32 bytes. */
typedef struct { float pos[3]; float tMin; float dir[3]; float tMax; } orc_ray_gmem;
/* HitKeyPack (Source/Tracer/TracerTypes.h:199-205). */
typedef struct { uint32_t primKey, lmKey, transKey, accelKey; } orc_hit_keys;
/* MetaHit for triangles = Vector2 barycentrics (PrimitiveDefaultTriangle.h:32). */
typedef struct { float bary[2]; } orc_meta_hit;

/* ---- core math (pinned against the reference's own headers) ----------- */
/* Watertight alternative (Woop, Benthin, Wald 2013); same outputs. */
int  orc_intersect_triangle_wt(const float dir[3], const float pos[3],
                               const float v0[3], const float v1[3], const float v2[3],
                               int cull, float bary_out[3], float* t_out, int* backface_out);
int  orc_intersect_triangle(const float dir[3], const float pos[3],
                            const float v0[3], const float v1[3], const float v2[3],
                            int cull, float bary_out[3], float* t_out, int* backface_out);
int  orc_intersect_aabb(const float dir[3], const float pos[3],
                        const float bmin[3], const float bmax[3],
                        const float tmm[2], float tout[2]);
void orc_mat34_inverse(const float m[12], float inv[12]);
/* Same arithmetic with the [1][2] cofactor sign fixed (see mrg_oracle.c). */
void orc_mat34_inverse_corrected(const float m[12], float inv[12]);
void orc_transform_ray(const float m[12], const float dir[3], const float pos[3],
                       float dir_out[3], float pos_out[3]);
void orc_transform_aabb(const float m[12], const float bmin[3], const float bmax[3],
                        float omin[3], float omax[3]);
uint64_t orc_morton3d_u64(uint32_t x, uint32_t y, uint32_t z);
void orc_nudge(const float pos[3], const float ndir[3], float out[3]);
void orc_tri_center(const float v0[3], const float v1[3], const float v2[3], float c[3]);

/* ---- scene + two-level LBVH accelerator ------------------------------- */
typedef struct orc_scene orc_scene;
/* Triangle test of the scene's meshes: 0 Moller-Trumbore (MRay's, default),
 * 1 watertight (orc_intersect_triangle_wt). */
void orc_scene_set_watertight(orc_scene* s, int on);
orc_scene* orc_scene_create(void);
void       orc_scene_destroy(orc_scene*);
/* Returns mesh id (>=0) or -1.  prim keys are prim_key_base + local triangle index. */
int  orc_scene_add_mesh(orc_scene*, const float* pos, uint32_t nv,
                        const uint32_t* idx, uint32_t nt, uint32_t prim_key_base);
/* m = 3x4 row-major local->world.  Returns instance id or -1. */
#define ORC_INSTANCE_CULL_BACKFACE      0x1u
#define ORC_INSTANCE_CORRECTED_INVERSE  0x2u
int  orc_scene_add_instance(orc_scene*, uint32_t mesh, const float m[12], uint32_t flags,
                            uint32_t lm_key, uint32_t trans_key, uint32_t accel_key);
int  orc_scene_build(orc_scene*);
/* Instance inverse matrix as computed by the build (for cross-checks). */
void orc_scene_instance_inverse(const orc_scene*, uint32_t inst, float inv[12]);

/* Closest hit: BaseAcceleratorLBVH::CastRays semantics.  ray_idx may be NULL
 * (identity).  Writes hits/meta/tMax only for rays that hit (misses untouched).
 * hit_inst (optional) receives the instance index or 0xFFFFFFFF. */
void orc_cast_closest(const orc_scene*, orc_ray_gmem* rays, const uint32_t* ray_idx,
                      uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta,
                      uint32_t* hit_inst, int nthreads);
/* Same semantics, brute force over all triangles of every instance (no boxes). */
void orc_cast_closest_linear(const orc_scene*, orc_ray_gmem* rays, const uint32_t* ray_idx,
                             uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta,
                             uint32_t* hit_inst, int nthreads);
/* Local cast: BaseAcceleratorI::CastLocalRays semantics (AcceleratorC.h:407-421,
 * KCLocalRayCast AcceleratorWork.kt.h:179-244).  Listed ray i is cast against
 * instance inst_ids[i] only (its BLAS, local space, no instance-box test);
 * hits / meta / tMax as orc_cast_closest.  Out-of-range ids are skipped. */
void orc_cast_local(const orc_scene*, orc_ray_gmem* rays, const uint32_t* ray_idx, const uint32_t* inst_ids,
                    uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta, int nthreads);
/* Any hit: CastVisibilityRays semantics.  visible_bits has one bit per ray
 * index (set = visible); bits of the listed rays are set then cleared on a hit. */
void orc_cast_visibility(const orc_scene*, const orc_ray_gmem* rays, const uint32_t* ray_idx,
                         uint32_t n, uint32_t* visible_bits, int nthreads);
/* Node / leaf statistics of the last build. */
void orc_scene_stats(const orc_scene*, uint64_t out[4]);
/* Union of the instances' world AABBs (TransformAABB of each BLAS root box)
 * and MRay's boundary-light scene diameter, |(span.x, span.z)|
 * (TracerBase.cpp:1650-1664). */
void  orc_scene_aabb(const orc_scene*, float out[6]);
float orc_scene_diameter(const orc_scene*);

#ifdef __cplusplus
}
#endif
