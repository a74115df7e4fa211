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
    uint32_t sampler;       /* 0: counter-based independent numbers, 1: ZSobol, 2: ZSobol with
                               the Owen bit order, 3: MRay's per-pixel PCG32 streams */
    uint32_t samplerMaxSpp; /* ZSobol initialMaxSampleCount (0: sampleStart + spp) */
    float    coneAperture;  /* camera rays' cone aperture 2 tan(fovY / 2) / height (orc_pt_camera_frame) */
} orc_pt_params;

/* Per instance (surface): Lambert albedo or light, instance-space triangles
 * (9 floats each, indexed by local primitive), transform and inverse. */
#define ORC_MAT_LAMBERT 0
#define ORC_MAT_REFLECT 1
#define ORC_MAT_REFRACT 2
#define ORC_MAT_UNREAL  3

/* a texture: RGBA, format 0 = UNORM8, 1 = f32, with its mip levels 1.. */
typedef struct
{
    const void*  texels;
    uint32_t     w, h, format;
    const void*  mips;
    uint32_t     mipCount;
} orc_pt_tex;

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
    /* albedo texture (replaces albedo[] when texels != NULL): RGBA, format
     * 0 = UNORM8, 1 = f32; bilinear, wrap addressed, single level; the
     * surface's uvs hold 6 floats (uv0 uv1 uv2) per local primitive */
    const void*  texels;
    uint32_t     texW, texH, texFormat;
    const float* uvs;
    /* the texture's mip levels 1.. (orc_gen_mips), or NULL / 1 for level 0 only */
    const void*  mips;
    uint32_t     mipCount;
    /* Unreal's roughness, metallic and specular textures (first channel; texels
     * NULL keeps the constant), read like the albedo texture */
    orc_pt_tex   param[3];
} orc_pt_surface;

/* KCGenerateMipmaps (Source/Tracer/TextureFilter.cu:62-192, 1006-1100) with a
 * Gaussian filter of the given radius: levels 1 .. count - 1 of a w x h
 * texture (format 0 RGBA8, 1 RGBA f32) into out, one after another;
 * returns the level count. */
uint32_t orc_gen_mips(const void* texels, uint32_t w, uint32_t h, uint32_t format, float radius, void* out);
/* levels 1 .. levels - 1 into out; the levels whose bit is set in validMask
 * are already in out and kept (their children are filtered from them) */
uint32_t orc_gen_mips_levels(const void* texels, uint32_t w, uint32_t h, uint32_t format, float radius,
                             uint32_t levels, uint32_t validMask, void* out);

/* Bilinear, wrap-addressed albedo read (TextureViewCPU.h:196-375, UNORM8
 * channels through NormConversion::FromUNorm). */
void orc_tex_read(const void* texels, uint32_t w, uint32_t h, uint32_t format, const float uv[2], float rgb[3]);

typedef struct
{
    float    p0[3], p1[3], p2[3];
    float    n[3];
    float    area;
    float    radiance[3];
    int      twoSided;
    uint32_t instance;          /* the light's instance (emission gradients) */
} orc_pt_light_tri;

/* Skysphere boundary light with a spherical (lat-long) radiance map
 * (LightSkysphere<SphericalCoordConverter>).  A 1x1 map is a constant
 * radiance, sampled uniformly over uv. */
typedef struct
{
    uint32_t     width, height;
    const float* texels;        /* RGBA f32 per texel, row-major, row 0 at v = 0 */
    const float* cdfX;          /* width * height row CDFs (orc_pwc2d_build) */
    const float* cdfY;          /* height: marginal CDF */
    float        m[12];         /* ApplyV rows (translation ignored) */
    float        inv[12];       /* InvApplyV rows */
    float        sceneDiameter; /* orc_scene_diameter */
} orc_pt_env;

/* Spectral rendering (Jakob & Hanika 2019 RGB -> spectrum, 4 wavelengths per
 * path; Source/Tracer/SpectrumContext.{h,hpp,cu}).  Tables as MRay prepares
 * them (SpectrumContext.cu:400-420): the observer already divided by the CIE
 * integrals, the illuminant already scaled by Y_INTEGRAL / normFactor. */
typedef struct
{
    uint32_t     lutRes;
    const float* lut;           /* 9 * res^3 floats: [table][coefficient][z][y][x] */
    uint32_t     cieCount;      /* 471 (360..830 nm) */
    const float* observer;      /* cieCount * 3 */
    const float* illuminant;    /* cieCount */
    float        xyzToRgb[9];
} orc_spectral;

/* Observer / illuminant preparation of SpectrumContextJakob2019 (from MRay's
 * raw tables; out arrays of cieCount * 3 and cieCount). */
void orc_spec_prepare(const float* cieXyz, const float integrals[3], const float* spd, float normFactor,
                      uint32_t cieCount, float* observer, float* illuminant);
/* SingleSampleSpectrumWavelength, HYPERBOLIC_PBRT (SpectrumContext.cu:40-135) */
void orc_spec_sample_waves(float xi0, float waves[4], float pdf[4]);
void orc_spec_convert_albedo(const orc_spectral* S, const float rgb[3], const float waves[4], float out[4]);
void orc_spec_convert_radiance(const orc_spectral* S, const float rgb[3], const float waves[4], float out[4]);
void orc_spec_to_rgb(const orc_spectral* S, const float value[4], const float waves[4], const float pdf[4],
                     float rgb[3]);

/* Accumulates spp samples per pixel into image (R, G, B, weight) per pixel,
 * row 0 at the bottom of the image plane.  env may be NULL (no boundary
 * light); it is the last light of the uniform light sampler.  spectral NULL
 * renders RGB, otherwise 4 wavelengths per path converted to RGB at the film. */
int  orc_pt_render(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                   const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                   const orc_spectral* spectral, float* image, int nthreads);

/* Path-replay adjoint (project-written reference; MRay has no adjoint):
 * for every pixel sample, the path is traced twice with the same random
 * numbers; the replay adds, at each Lambert vertex whose albedo is the texture
 * `texels`, delta[pixel] / spp * (primal radiance - radiance before the
 * vertex) / albedo, times each bilinear tap's weight, into grad (double RGBA
 * per texel, accumulated in FP64).  With gradEmission (double RGBA per
 * instance, nInstances entries) it also adds, for every emission the path
 * gathers from an area light (a hit, or a visible NEE sample), delta / spp *
 * (the contribution / the light's radiance) into the light's instance.
 * texels = NULL: no texture parameter.  RGB mode. */
int orc_pt_adjoint(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                   const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                   const void* texels, uint32_t texW, uint32_t texH, const float* delta,
                   double* grad, double* gradEmission, uint32_t nInstances, int nthreads);

/* Piecewise-constant 2D distribution (Source/Tracer/Distributions.h/.cu). */
/* Guided path tracing (GuidedPTRenderer) as a wavefront over the path slots,
 * in the GPU renderer's stage order.  The state (hash grid, chains,
 * irradiance averages, the slots' backup streams) persists across calls
 * until orc_guide_clear. */
typedef struct orc_guide_state orc_guide_state;
orc_guide_state* orc_guide_new(const orc_scene* s, uint32_t entryLimit, uint32_t posBits, uint32_t normalBits,
                               uint32_t maxLevelOffset, float coneDeg, float lobeProb, int fixZeroWeight);
void     orc_guide_delete(orc_guide_state* G);
void     orc_guide_clear(orc_guide_state* G);
uint32_t orc_guide_table_size(const orc_guide_state* G);
uint32_t orc_guide_used(const orc_guide_state* G);
void     orc_guide_snapshot(const orc_guide_state* G, uint64_t* codes, float* chain6, float* irr2);
int      orc_pt_render_guided(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                              const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                              const orc_spectral* spectral, orc_guide_state* G, uint32_t samplesPerPass,
                              float* image);

void  orc_pwc2d_build(const float* func, uint32_t w, uint32_t h, float* cdfX, float* cdfY);
void  orc_pwc2d_sample_uv(const float* cdfX, const float* cdfY, uint32_t w, uint32_t h,
                          const float xi[2], float uv[2], float* pdf);
float orc_pwc2d_pdf_uv(const float* cdfX, const float* cdfY, uint32_t w, uint32_t h, const float uv[2]);
/* Luminance of every texel of an RGBA map, read at texel centres through the
 * bilinear filter (ColorConverter.cu:405-475). */
void  orc_env_luminance(const float* texels, uint32_t w, uint32_t h, float* out);
/* Bilinear, wrap-addressed read (TextureViewCPU.h:196-375). */
void  orc_env_read(const float* texels, uint32_t w, uint32_t h, const float uv[2], float rgb[3]);
void  orc_env_dir_to_uv(const float dirYUp[3], float uv[2]);
void  orc_env_uv_to_dir(const float uv[2], float dirYUp[3]);
void orc_pt_camera_frame(const float pos[3], const float gaze[3], const float up[3],
                         float fovX, float fovY, float nearT, float farT, orc_pt_params* p);
void orc_pt_make_light(const float m[12], const float* v9, const float radiance[3], int twoSided,
                       orc_pt_light_tri* out);

/* Per-function entry points over the helpers the path loop uses (tangent
 * frame; uint32 random numbers converted as RNGFunctions::ToFloat01).  The
 * records match oracle/ref_pt_driver.cpp's, which runs MRay's own code. */
typedef struct
{
    float    albedo[3];
    float    rough, metal, spec, iorF, iorB;
    uint32_t backSide;
    float    pos[3];
    float    wo[3];
    float    wiEval[3];
    uint32_t xi[3];
} orc_fx_mat_in;
typedef struct
{
    float    wi[3];
    float    wiPos[3];
    float    pdf;
    float    refl[4];
    uint32_t passed;
    float    evalRefl[4];
    float    evalPdf;
    float    specularity;
} orc_fx_mat_out;
typedef struct
{
    float    m[12];
    float    v9[9];
    uint32_t twoSided;
    float    radiance[3];
    float    distant[3];
    uint32_t xi[2];
    float    hit[2];
    float    dir[3];
    float    wo[3];
} orc_fx_light_in;
typedef struct
{
    float point[3];
    float samplePdf;
    float pdfSolidAngle;
    float emitHit[4];
    float emitPoint[4];
    float area;
} orc_fx_light_out;

/* kind: ORC_MAT_* */
void orc_fx_material(int kind, const orc_fx_mat_in* in, orc_fx_mat_out* out, uint32_t n);
void orc_fx_fresnel_dielectric(const float* in3, float* out, uint32_t n);
void orc_fx_vndf_sample(const float* in6, float* out4, uint32_t n);
void orc_fx_russian_roulette(const float* in6, float* out5, uint32_t n);
void orc_fx_tri_light(const orc_fx_light_in* in, orc_fx_light_out* out, uint32_t n);
void orc_fx_gaussian_filter(const float* in3, float* out5, uint32_t n);
void orc_fx_sample_waves(const uint32_t* xi, float* waves4, float* pdf4, uint32_t n);
void orc_fx_cone(const float* in20, float* out12, uint32_t n);
void orc_fx_pixel_indices(const float* in6, float* out2, uint32_t n);
void orc_fx_spherical_coords(const float* in6, float* out7, uint32_t n);
void orc_fx_camera(const float* cam13, const uint32_t res[2], const uint32_t* pix, const float* off4, float* out6,
                   uint32_t n);

#ifdef __cplusplus
}
#endif
