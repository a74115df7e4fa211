/*
 * pt_oracle.h -- CPU path-tracer oracle (TEST INFRASTRUCTURE ONLY).
 * See pt_oracle.c for the reference functions each part restates.
 */
#pragma once
#include <stdint.h>
#include "mrg_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PT_PURE     0u
#define ORC_PT_NEE      1u
#define ORC_PT_NEE_MIS  2u

typedef struct
{
    uint32_t width, height;
    uint32_t spp;           /* samples per pixel in this call */
    uint32_t sampleStart;   /* index of the first sample (for accumulation) */
    uint32_t rrStart;       /* russianRouletteRange[0] */
    uint32_t maxDepth;      /* russianRouletteRange[1] */
    uint32_t sampleMode;    /* ORC_PT_* */
    uint32_t seed;
    float    filterRadius;
    float    camPos[3];
    float    camBottomLeft[3];
    float    camRight[3];
    float    camUp[3];
    float    planeSize[2];
    float    nearT, farT;
} orc_pt_params;

/* Per instance (surface): Lambert albedo or light, instance-space triangles
 * (9 floats each, indexed by local primitive), transform and inverse. */
#define ORC_MAT_LAMBERT 0
#define ORC_MAT_REFLECT 1
#define ORC_MAT_REFRACT 2
#define ORC_MAT_UNREAL  3

typedef struct
{
    int          isLight;
    float        albedo[3];
    int          matType;       /* ORC_MAT_* */
    float        roughness, metallic, specular;
    float        iorFront, iorBack;
    uint32_t     lightBase;     /* first light index of this surface */
    uint32_t     primKeyBase;
    const float* triangles;
    float        m[12];
    float        inv[12];
} orc_pt_surface;

typedef struct
{
    float    p0[3], p1[3], p2[3];
    float    n[3];
    float    area;
    float    radiance[3];
    int      twoSided;
} orc_pt_light_tri;

/* Accumulates spp samples per pixel into image (R, G, B, weight) per pixel,
 * row 0 at the bottom of the image plane. */
int  orc_pt_render(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                   const orc_pt_light_tri* lights, uint32_t nLights, float* image, int nthreads);
void orc_pt_camera_frame(const float pos[3], const float gaze[3], const float up[3],
                         float fovX, float fovY, float nearT, float farT, orc_pt_params* p);
void orc_pt_make_light(const float m[12], const float* v9, const float radiance[3], int twoSided,
                       orc_pt_light_tri* out);

#ifdef __cplusplus
}
#endif
