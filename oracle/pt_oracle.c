/*
 * pt_oracle.c -- CPU path-tracer oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the estimator of MRay's wavefront path tracer with next-event
 * estimation and MIS (RGB variant), one path at a time:
 *   - camera rays, pinhole + stochastic Gaussian film filter
 *       Source/Tracer/RayGenKernels.kt.h:157-226, CamerasDefault.hpp:94-140,
 *       Filters.h:195-233 (sigma = 0.285714 r; weight = filter / pdf = 1)
 *   - surface work: NEE (light sample, shadow ray, MIS balance)
 *       Source/TracerDLL/PathTracerRendererShaders.h:354-445
 *   - BxDF sample, Russian roulette, next ray
 *       PathTracerRendererShaders.h:203-300; DistributionFunctions.h:943-953
 *   - light hit with MIS       PathTracerRendererShaders.h:450-517
 *   - shadow accumulation      Source/TracerDLL/PathTracerRenderer.cu:13-31
 *   - Lambert                  Source/Tracer/MaterialsDefault.hpp:29-110
 *   - triangle area light      Source/Tracer/LightsDefault.hpp:24-160,
 *                              PrimitiveDefaultTriangle.hpp:49-75
 *   - uniform light sampler    Source/Tracer/LightSampler.hpp:6-120
 *   - skysphere boundary light Source/Tracer/LightsDefault.hpp:175-222,
 *                              300-420 (spherical mapping), sampled with
 *                              the piecewise-constant 2D distribution of
 *                              Distributions.h:14-270 / Distributions.cu
 *                              (host-backend construction)
 *   - film                     Source/Tracer/TextureFilter.cu:673-697
 * Random numbers come from a counter-based hash of (seed, pixel, sample,
 * bounce, dimension), the same one the GPU renderer uses, so both render the
 * same paths (MRay's own streams depend on its ray-slot scheduling and cannot
 * be reproduced).  Intersections go through the LBVH oracle (mrg_oracle.c).
 */
#include "mrg_oracle.h"
#include "pt_oracle.h"
#include "zsobol_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.14159265358979323846f
#define INV_PI_F 0.318309886183790671538f

/* PCG hash (Jarzynski & Olano, "Hash Functions for GPU Rendering", 2020). */
static inline uint32_t pcg_hash(uint32_t v)
{
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
static inline uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample)
{
    return pcg_hash(pcg_hash(seed ^ 0x9E3779B9u) ^ pcg_hash(pixel) ^ pcg_hash(sample + 0x632BE5ABu));
}
static inline float rnd(uint32_t key, uint32_t bounce, uint32_t dim)
{
    uint32_t h = pcg_hash(key ^ pcg_hash((bounce << 4) | dim));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

/* The sample's random-number source: the counter-based hash; MRay's ZSobol
 * group under the path tracer's dimension plan (film-filter offset = Next2D(0),
 * wavelengths = Next(2); bounce b from dimension 3 + 7b: k 0..2 = Next3D(+0),
 * k 3 = Next(+3), k 4, 5 = Next2D(+4), k 8 = Next(+6)); or MRay's independent
 * group, the pixel's PCG32 stream read at position
 * ((sample * (maxDepth + 1) + b) * 16 + k).  Numbers convert as
 * RNGFunctions::ToFloat01 does (Source/Tracer/Random.h:100-119). */
typedef struct
{
    uint32_t key, px, py, sample, seed, sampler, maxSpp, resBits, maxDepth;
} smp_ctx;

static float to_unit(uint32_t v)
{
    float f = (float)v * 0x1p-32f;
    const float prev1 = 0x1.fffffep-1f;
    return f < prev1 ? f : prev1;
}

static float urnd(const smp_ctx* c, uint32_t bounce, uint32_t k)
{
    if(c->sampler == 0u) return rnd(c->key, bounce, k);
    if(c->sampler == 3u)
    {
        const uint32_t n = ((c->sample * (c->maxDepth + 1u) + bounce) << 4) | k;
        return to_unit(orc_pcg32_permute(orc_pcg32_advance(orc_pcg32_state(c->seed), n)));
    }
    uint32_t dim, size, comp;
    if(k == 6u || k == 7u) { dim = 0u; size = 2u; comp = k - 6u; }
    else if(k == 9u) { dim = 2u; size = 1u; comp = 0u; }
    else
    {
        const uint32_t b = 3u + 7u * bounce;
        if(k <= 2u) { dim = b; size = 3u; comp = k; }
        else if(k == 3u) { dim = b + 3u; size = 1u; comp = 0u; }
        else if(k <= 5u) { dim = b + 4u; size = 2u; comp = k - 4u; }
        else { dim = b + 6u; size = 1u; comp = 0u; }
    }
    return to_unit(orc_zs_number(c->px, c->py, c->seed, c->sample, c->maxSpp, c->resBits, dim, size, comp,
                                 c->sampler == 2u));
}

/* Math::Dot (Source/Core/Math.h:1585-1596): r = 0; r = fma(a_i, b_i, r). */
static inline float dot3f(const float a[3], const float b[3])
{
    return fmaf(a[2], b[2], fmaf(a[1], b[1], fmaf(a[0], b[0], 0.0f)));
}
/* Math::Cross (Math.h:1627-1633): each component one fma. */
static inline void cross3f(const float a[3], const float b[3], float o[3])
{
    float x = fmaf(a[1], b[2], -(a[2] * b[1]));
    float y = fmaf(a[2], b[0], -(a[0] * b[2]));
    float z = fmaf(a[0], b[1], -(a[1] * b[0]));
    o[0] = x; o[1] = y; o[2] = z;
}
/* Math::Normalize (Math.h:1618-1624): v * (1 / Length(v)). */
static inline void normalize3f(float v[3])
{
    float inv = 1.0f / sqrtf(dot3f(v, v));
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}

/* Orthonormal basis about n (Duff et al., "Building an Orthonormal Basis,
 * Revisited", JCGT 2017). */
static void onb(const float n[3], float t[3], float b[3])
{
    float sign = copysignf(1.0f, n[2]);
    float a = -1.0f / (sign + n[2]);
    float bb = n[0] * n[1] * a;
    t[0] = 1.0f + sign * n[0] * n[0] * a; t[1] = sign * bb; t[2] = -sign * n[0];
    b[0] = bb; b[1] = sign + n[1] * n[1] * a; b[2] = -n[1];
}


/* ---------------------------------------------------------------------- */
/* Materials (Source/Tracer/MaterialsDefault.hpp; DistributionFunctions.h) */
/* ---------------------------------------------------------------------- */
#define SPECULAR_THRESHOLD 0.95f   /* MaterialC.h:11 */

static inline float sqrt_max(float x) { return sqrtf(fmaxf(x, 0.0f)); }

/* BxDF::DGGX (DistributionFunctions.h:434-443) */
static float d_ggx(float ndh, float alpha)
{
    float a2 = alpha * alpha;
    float den = ndh * ndh * (a2 - 1.0f) + 1.0f;
    den = den * den;
    den *= PI_F;
    return a2 / den;
}
/* BxDF::LambdaSmith (:445-454) */
static float lambda_smith(const float v[3], float alpha)
{
    float a2 = alpha * alpha;
    float inner = a2 * (v[0] * v[0] + v[1] * v[1]) / (v[2] * v[2]);
    return (sqrtf(1.0f + inner) - 1.0f) * 0.5f;
}
static float g_single(const float v[3], float alpha) { return 1.0f / (1.0f + lambda_smith(v, alpha)); }
static float g_correlated(const float o[3], const float i[3], float alpha)
{
    return 1.0f / (lambda_smith(o, alpha) + lambda_smith(i, alpha) + 1.0f);
}
/* BxDF::FSchlick (:502-511) */
static void f_schlick(float vdh, const float* f0, float* out, int nc)
{
    float pw = 1.0f - vdh;
    float pw2 = pw * pw;
    float pw5 = pw2 * pw2 * pw;
    for(int k = 0; k < nc; k++) out[k] = (1.0f - f0[k]) * pw5 + f0[k];
}
/* BxDF::VNDFGGXSmithPDF (:515-527) */
static float vndf_pdf(const float V[3], const float H[3], float alpha)
{
    float vdh = fmaxf(0.0f, dot3f(H, V));
    float ndh = fmaxf(0.0f, H[2]);
    float ndv = fmaxf(0.0f, V[2]);
    float D = d_ggx(ndh, alpha);
    float G = g_single(V, alpha);
    if(ndv == 0.0f) return 0.0f;
    return vdh * D * G / ndv;
}
/* BxDF::VNDFGGXSmithSample (:529-590), Heitz 2018 */
static void vndf_sample(const float V[3], float a, float xi0, float xi1, float H[3])
{
    float vh[3] = { a * V[0], a * V[1], V[2] };
    normalize3f(vh);
    float len2 = fmaf(vh[1], vh[1], fmaf(vh[0], vh[0], 0.0f));   /* LengthSqr(Vector2(VHemi)) */
    float T1[3];
    if(len2 > 0.0f)
    {
        float rs = 1.0f / sqrtf(len2);
        T1[0] = -vh[1] * rs; T1[1] = vh[0] * rs; T1[2] = 0.0f;
    }
    else { T1[0] = 1.0f; T1[1] = 0.0f; T1[2] = 0.0f; }
    float T2[3];
    cross3f(vh, T1, T2);
    float r = sqrtf(xi0);
    float phi = 2.0f * PI_F * xi1;
    float t1 = r * cosf(phi), t2 = r * sinf(phi);
    float sS = 0.5f * (1.0f + vh[2]);
    t2 = (1.0f - sS) * sqrtf(1.0f - t1 * t1) + sS * t2;
    float val = 1.0f - t1 * t1 - t2 * t2;
    float sq = sqrt_max(val);
    float nh[3];
    for(int k = 0; k < 3; k++) nh[k] = t1 * T1[k] + t2 * T2[k] + sq * vh[k];
    float nm[3] = { a * nh[0], a * nh[1], sqrt_max(nh[2]) };
    float n2 = dot3f(nm, nm);
    if(n2 < 1.0e-5f) { H[0] = 0.0f; H[1] = 0.0f; H[2] = 1.0f; }
    else { float rs = 1.0f / sqrtf(n2); H[0] = nm[0] * rs; H[1] = nm[1] * rs; H[2] = nm[2] * rs; }
}
/* BxDF::BurleyDiffuseCorrection (:592-603) */
static float burley(float ndl, float ndv, float ldh, float rough)
{
    float fd90 = 0.5f + 2.0f * rough * ldh * ldh;
    float p1 = 1.0f - ndl, p2 = 1.0f - ndv;
    float p1s = p1 * p1, p2s = p2 * p2;
    float a = 1.0f + (fd90 - 1.0f) * (p1s * p1s * p1);
    float b = 1.0f + (fd90 - 1.0f) * (p2s * p2s * p2);
    return a * b;
}
/* UnrealMaterial::MISRatio (MaterialsDefault.hpp:470-478) */
static float unreal_mis_ratio(const orc_pt_surface* m, float avgAlbedo)
{
    float integ = 2.0f * PI_F * avgAlbedo;
    integ *= (1.0f - m->metallic);
    float specR = m->specular * (1.0f - m->metallic) + avgAlbedo * m->metallic;   /* Lerp */
    float total = specR + integ;
    return (total == 0.0f) ? 0.0f : integ / total;
}
/* albedo.Sum() * 0.3333 over the Spectrum's channels (RGB: 3, spectral: 4;
 * MaterialsDefault.hpp:548) */
static inline float avg_albedo(const float* alb, int nc)
{
    float s = alb[0] + alb[1] + alb[2];
    if(nc == 4) s += alb[3];
    return s * 0.3333f;
}
static float specularity(const orc_pt_surface* m, const float* alb, int nc)
{
    if(m->matType == ORC_MAT_REFLECT || m->matType == ORC_MAT_REFRACT) return 1.0f;
    if(m->matType == ORC_MAT_UNREAL) return 1.0f - unreal_mis_ratio(m, avg_albedo(alb, nc));
    return 0.0f;
}
/* UnrealMaterial::Evaluate / Pdf (MaterialsDefault.hpp:628-720) in the
 * tangent frame; V, L unit vectors. */
static void unreal_eval(const orc_pt_surface* m, const float* alb, int nc, const float V[3], const float L[3],
                        float* refl, float* pdfOut)
{
    float alpha = m->roughness * m->roughness;
    float H[3] = { L[0] + V[0], L[1] + V[1], L[2] + V[2] };
    normalize3f(H);
    float ldh = fmaxf(0.0f, dot3f(L, H));
    float vdh = fmaxf(0.0f, dot3f(V, H));
    float ndh = fmaxf(0.0f, H[2]);
    float ndv = fmaxf(0.0f, V[2]);
    float D = d_ggx(ndh, alpha);
    int dBad = isnan(D) || isinf(D);
    float Dn = dBad ? 0.0f : D;
    float G = g_correlated(V, L, alpha);
    G = (ldh == 0.0f) ? 0.0f : G;
    G = (vdh == 0.0f) ? 0.0f : G;
    float f0[4];
    for(int k = 0; k < nc; k++) f0[k] = (m->specular * 0.08f) * (1.0f - m->metallic) + alb[k] * m->metallic;
    float F[4];
    f_schlick(vdh, f0, F, nc);
    float ndl = fmaxf(0.0f, L[2]);
    float corr = burley(ndl, ndv, ldh, m->roughness);
    for(int k = 0; k < nc; k++)
    {
        float spec = (ndv == 0.0f) ? 0.0f : Dn * F[k] * G * 0.25f / ndv;
        float diff = ndl * ((1.0f - m->metallic) * alb[k]) * INV_PI_F * corr;
        refl[k] = diff + spec;
    }
    float ratio = unreal_mis_ratio(m, avg_albedo(alb, nc));
    float pd = L[2] * INV_PI_F;
    pd = (pd <= 1.0e-5f) ? 0.0f : pd;
    float ps = vndf_pdf(V, H, alpha);
    ps = dBad ? 0.0f : ps;
    ps = (vdh == 0.0f) ? 0.0f : ps / (4.0f * vdh);
    *pdfOut = pd * ratio + ps * (1.0f - ratio);
}
/* Fresnel for dielectrics (DistributionFunctions.h:382-398) */
static float fresnel_dielectric(float cosF, float etaF, float etaB)
{
    float sinF = sqrt_max(1.0f - cosF * cosF);
    float sinB = etaF / etaB * sinF;
    if(sinF >= 1.0f) return 1.0f;
    float cosB = sqrt_max(1.0f - sinB * sinB);
    float par = (etaB * cosF - etaF * cosB) / (etaB * cosF + etaF * cosB);
    par = par * par;
    float per = (etaF * cosF - etaB * cosB) / (etaF * cosF + etaB * cosB);
    per = per * per;
    return (par + per) * 0.5f;
}

/* Common::SampleCosDirection (DistributionFunctions.h:847-870): the
 * tangent-frame direction and its pdf. */
static inline void cos_sample(float xi0, float xi1, float L[3], float* pdf)
{
    float ang = 2.0f * PI_F * xi1, sr = sqrtf(xi0);
    L[0] = sr * cosf(ang); L[1] = sr * sinf(ang);
    L[2] = sqrt_max(1.0f - fmaf(L[1], L[1], fmaf(L[0], L[0], 0.0f)));
    *pdf = L[2] * INV_PI_F;
}

/* BxDF sample in the tangent frame (z = shading normal), the SampleBxDF of
 * each material (MaterialsDefault.hpp: Lambert 29-62, Reflect 150-170,
 * Refract 263-305, Unreal 535-628).  xi0..xi2 are the dispenser's numbers
 * 0..2.  L is the sampled direction in the tangent frame (Reflect's is
 * normalised, as MRay's is); *passed is set for a refraction.  Refract's
 * one-ulp nudge of the position along the normal is the caller's. */
static void bxdf_sample(const orc_pt_surface* sf, const float* alb, int nc, int backSide, const float V[3],
                        float xi0, float xi1, float xi2, float L[3], float refl[4], float* pdfOut, int* passed)
{
    refl[0] = refl[1] = refl[2] = refl[3] = 0.0f;
    *passed = 0;
    if(sf->matType == ORC_MAT_REFLECT)
    {
        float d2 = 2.0f * V[2];
        L[0] = -V[0]; L[1] = -V[1]; L[2] = d2 - V[2];
        normalize3f(L);
        *pdfOut = 1.0f;
        refl[0] = refl[1] = refl[2] = refl[3] = 1.0f;
    }
    else if(sf->matType == ORC_MAT_REFRACT)
    {
        float fromEta = sf->iorFront, toEta = sf->iorBack;
        if(backSide) { float t = fromEta; fromEta = toEta; toEta = t; }
        float cosT = fabsf(V[2]);
        float f = fresnel_dielectric(cosT, fromEta, toEta);
        int doRefl = xi0 < f;
        if(doRefl) { L[0] = -V[0]; L[1] = -V[1]; L[2] = 2.0f * V[2] - V[2]; }
        else
        {
            float eta = fromEta / toEta;
            float cosIn = V[2];
            float sin2 = fmaxf(0.0f, 1.0f - cosIn * cosIn);
            float sinOut2 = eta * eta * sin2;
            float cosOut = sqrt_max(1.0f - sinOut2);
            for(int k = 0; k < 2; k++) L[k] = eta * -V[k];
            L[2] = eta * -V[2] + (eta * cosIn - cosOut);
        }
        float bpdf = doRefl ? f : (1.0f - f);
        *pdfOut = bpdf;
        refl[0] = refl[1] = refl[2] = refl[3] = bpdf;
        *passed = !doRefl;
    }
    else if(sf->matType == ORC_MAT_UNREAL)
    {
        float alpha = sf->roughness * sf->roughness;
        float ratio = unreal_mis_ratio(sf, avg_albedo(alb, nc));
        float sXi = xi0, x0 = xi1, x1 = xi2;
        float H[3], pd, ps;
        if(sXi < ratio)
        {
            cos_sample(x0, x1, L, &pd);
            H[0] = L[0] + V[0]; H[1] = L[1] + V[1]; H[2] = L[2] + V[2];
            normalize3f(H);
            float vdh = fmaxf(0.0f, dot3f(V, H));
            ps = vndf_pdf(V, H, alpha);
            ps = (vdh == 0.0f) ? 0.0f : ps / (4.0f * vdh);
        }
        else
        {
            vndf_sample(V, alpha, x0, x1, H);
            float dv = 2.0f * dot3f(V, H);
            for(int k = 0; k < 3; k++) L[k] = dv * H[k] - V[k];
            float vdh = fmaxf(0.0f, dot3f(V, H));
            ps = vndf_pdf(V, H, alpha);
            ps = (vdh == 0.0f) ? 0.0f : ps / (4.0f * vdh);
            pd = L[2] * INV_PI_F;
            pd = (pd <= 1.0e-5f) ? 0.0f : pd;
        }
        float vdh = fmaxf(0.0f, dot3f(V, H));
        float ldh = fmaxf(0.0f, dot3f(L, H));
        float ndh = fmaxf(0.0f, H[2]);
        float ndv = fmaxf(0.0f, V[2]);
        float D = d_ggx(ndh, alpha);
        float G = g_correlated(V, L, alpha);
        G = (ldh == 0.0f) ? 0.0f : G;
        G = (vdh == 0.0f) ? 0.0f : G;
        float f0[4], F[4];
        for(int k = 0; k < nc; k++) f0[k] = (sf->specular * 0.08f) * (1.0f - sf->metallic) + alb[k] * sf->metallic;
        f_schlick(vdh, f0, F, nc);
        float spec[4];
        for(int k = 0; k < nc; k++) spec[k] = (ndv == 0.0f) ? 0.0f : D * F[k] * G * 0.25f / ndv;
        if(isinf(D) || isnan(D))
        {
            float gs = g_single(V, alpha);
            for(int k = 0; k < nc; k++) spec[k] = G * F[k] / gs;
            ps = 1.0f;
        }
        float ndl = fmaxf(0.0f, L[2]);
        float corr = burley(ndl, ndv, ldh, sf->roughness);
        for(int k = 0; k < nc; k++)
            refl[k] = ndl * ((1.0f - sf->metallic) * alb[k]) * INV_PI_F * corr + spec[k];
        *pdfOut = pd * ratio + ps * (1.0f - ratio);
    }
    else
    {
        /* reflectance = albedo * nDotL * InvPi, nDotL = max(wI.z, 0) */
        cos_sample(xi0, xi1, L, pdfOut);
        float ndl = fmaxf(L[2], 0.0f);
        for(int k = 0; k < nc; k++) refl[k] = (alb[k] * ndl) * INV_PI_F;
    }
}

/* BxDF evaluation and pdf in the tangent frame for the NEE direction L
 * (Lambert Evaluate / Pdf, MaterialsDefault.hpp:64-86; Unreal 630-720).
 * Only non-specular materials are evaluated (specular ones take no NEE). */
static void bxdf_eval(const orc_pt_surface* sf, const float* alb, int nc, const float V[3], const float L[3],
                      float refl[4], float* pdfOut)
{
    refl[0] = refl[1] = refl[2] = refl[3] = 0.0f;
    if(sf->matType == ORC_MAT_UNREAL)
        unreal_eval(sf, alb, nc, V, L, refl, pdfOut);
    else
    {
        /* Evaluate: nDotL * albedo * InvPi */
        float ndl = fmaxf(L[2], 0.0f);
        for(int k = 0; k < nc; k++) refl[k] = (ndl * alb[k]) * INV_PI_F;
        float bpdf = L[2] * INV_PI_F;
        *pdfOut = (bpdf <= 1.0e-5f) ? 0.0f : bpdf;
    }
}

/* ------------------------------------------------------------------------ */
/* Piecewise-constant 2D distribution (Source/Tracer/Distributions.h:14-270, */
/* construction Distributions.cu:233-330, host backend)                     */
/* ------------------------------------------------------------------------ */
void orc_pwc2d_build(const float* func, uint32_t w, uint32_t h, float* cdfX, float* cdfY)
{
    /* KCSegmentedScanPrecise: per row, double running sum of |f| */
    for(uint32_t y = 0; y < h; y++)
    {
        double sum = 0.0;
        for(uint32_t x = 0; x < w; x++)
        {
            sum += (double)fabsf(func[(size_t)y * w + x]);
            cdfX[(size_t)y * w + x] = (float)sum;
        }
    }
    /* KCCopyScanY: float running sum of the row totals (before normalising) */
    float s = 0.0f;
    for(uint32_t y = 0; y < h; y++)
    {
        s += cdfX[(size_t)y * w + (w - 1)];
        cdfY[y] = s;
    }
    /* KCNormalizeXY: every row and the marginal, in double */
    for(uint32_t y = 0; y < h; y++)
    {
        float* row = cdfX + (size_t)y * w;
        double rr = 1.0 / (double)row[w - 1];
        for(uint32_t x = 0; x < w; x++) row[x] = (float)((double)row[x] * rr);
    }
    double ry = 1.0 / (double)cdfY[h - 1];
    for(uint32_t y = 0; y < h; y++) cdfY[y] = (float)((double)cdfY[y] * ry);
}

/* DistributionPwC<1>::SampleIndex (Distributions.h:128-146): lower bound,
 * linear position inside the bin, and the quirk that every value >= 1 is
 * moved down by one ulp. */
static float pwc1_sample_index(const float* cdf, uint32_t n, float xi, float* pdf)
{
    uint32_t lo = 0, cnt = n;
    while(cnt > 0)
    {
        uint32_t step = cnt / 2, mid = lo + step;
        if(cdf[mid] < xi) { lo = mid + 1; cnt -= step + 1; }
        else cnt = step;
    }
    uint32_t index = lo;
    float prev = (index == 0) ? 0.0f : cdf[index - 1];
    float my = cdf[index];
    float t = (xi - prev) / (my - prev);
    float indexF = (float)index + t;
    indexF = (indexF < 1.0f) ? indexF : nextafterf(indexF, -3.402823466e+38f);
    *pdf = (my - prev) * (float)n;
    return indexF;
}

static float pwc1_pdf_index(const float* cdf, uint32_t n, float index)
{
    uint32_t i = (uint32_t)index;
    float prev = (i == 0) ? 0.0f : cdf[i - 1];
    return (cdf[i] - prev) * (float)n;
}

void orc_pwc2d_sample_uv(const float* cdfX, const float* cdfY, uint32_t w, uint32_t h,
                         const float xi[2], float uv[2], float* pdf)
{
    float py, px;
    float iy = pwc1_sample_index(cdfY, h, xi[1], &py);
    uint32_t row = (uint32_t)iy;
    float ix = pwc1_sample_index(cdfX + (size_t)row * w, w, xi[0], &px);
    uv[0] = ix * (1.0f / (float)w);
    uv[1] = iy * (1.0f / (float)h);
    *pdf = py * px;
}

float orc_pwc2d_pdf_uv(const float* cdfX, const float* cdfY, uint32_t w, uint32_t h, const float uv[2])
{
    float ix = uv[0] * (float)w, iy = uv[1] * (float)h;
    ix = (ix < (float)w - 1.0f) ? ix : (float)w - 1.0f;
    iy = (iy < (float)h - 1.0f) ? iy : (float)h - 1.0f;
    uint32_t row = (uint32_t)iy;
    float marginal = pwc1_pdf_index(cdfY, h, iy);
    float conditional = pwc1_pdf_index(cdfX + (size_t)row * w, w, ix);
    return conditional * marginal;
}

/* ------------------------------------------------------------------------ */
/* Skysphere light (Source/Tracer/LightsDefault.hpp:175-222, 300-420)        */
/* ------------------------------------------------------------------------ */
#define PI_SQR_F (PI_F * PI_F)
/* Rec.709 / D65 luminance row of RGB -> XYZ (Color::XYZToYxy(ToXYZ(rgb)).x) */
#define LUM_R 0.2126729f
#define LUM_G 0.7151522f
#define LUM_B 0.0721750f

static inline int32_t wrap_index(int32_t i, int32_t n)
{
    i = i % n;
    return (i < 0) ? i + n : i;
}

/* ReadInterpolatedPixel + FindInterpolants of the host texture view,
 * including its treatment of negative texel coordinates (the fraction of a
 * negative coordinate is its absolute value). */
static inline void texel_rgb(const void* texels, uint32_t format, size_t i, float out[3])
{
    if(format == 0)
    {
        const uint8_t* t = (const uint8_t*)texels + 4 * i;
        /* FromUNorm: MIN + in * (1 / (MAX - MIN)) */
        const float delta = 1.0f / 255.0f;
        for(int k = 0; k < 3; k++) out[k] = 0.0f + (float)t[k] * delta;
    }
    else
    {
        const float* t = (const float*)texels + 4 * i;
        for(int k = 0; k < 3; k++) out[k] = t[k];
    }
}

void orc_tex_read(const void* texels, uint32_t w, uint32_t h, uint32_t format, const float uv[2], float rgb[3])
{
    float tx = uv[0] * (float)w - 0.5f, ty = uv[1] * (float)h - 0.5f;
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    float pix[4][3];
    for(int j = 0; j < 2; j++)
        for(int i = 0; i < 2; i++)
        {
            int32_t x = wrap_index(sx + i, (int32_t)w), y = wrap_index(sy + j, (int32_t)h);
            texel_rgb(texels, format, (size_t)y * w + (size_t)x, pix[(j << 1) + i]);
        }
    for(int k = 0; k < 3; k++)
    {
        float a = pix[0][k] * (1.0f - fx) + pix[1][k] * fx;
        float b = pix[2][k] * (1.0f - fx) + pix[3][k] * fx;
        rgb[k] = a * (1.0f - fy) + b * fy;
    }
}

void orc_env_read(const float* texels, uint32_t w, uint32_t h, const float uv[2], float rgb[3])
{
    float tx = uv[0] * (float)w - 0.5f, ty = uv[1] * (float)h - 0.5f;
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    float pix[4][3];
    for(int j = 0; j < 2; j++)
        for(int i = 0; i < 2; i++)
        {
            int32_t x = wrap_index(sx + i, (int32_t)w), y = wrap_index(sy + j, (int32_t)h);
            const float* t = &texels[4 * ((size_t)y * w + (size_t)x)];
            for(int k = 0; k < 3; k++) pix[(j << 1) + i][k] = t[k];
        }
    for(int k = 0; k < 3; k++)
    {
        float a = pix[0][k] * (1.0f - fx) + pix[1][k] * fx;
        float b = pix[2][k] * (1.0f - fx) + pix[3][k] * fx;
        rgb[k] = a * (1.0f - fy) + b * fy;
    }
}

void orc_env_luminance(const float* texels, uint32_t w, uint32_t h, float* out)
{
    const float rx = 1.0f / (float)w, ry = 1.0f / (float)h;
    for(uint32_t y = 0; y < h; y++)
        for(uint32_t x = 0; x < w; x++)
        {
            float uv[2] = { ((float)x + 0.5f) * rx, ((float)y + 0.5f) * ry };
            float c[3];
            orc_env_read(texels, w, h, uv, c);
            out[(size_t)y * w + x] = fmaf(LUM_B, c[2], fmaf(LUM_G, c[1], LUM_R * c[0]));
        }
}

/* SphericalCoordConverter::DirToUV: Y-up -> Z-up, (azimuth, inclination),
 * u = (azimuth + pi) / 2pi, v = 1 - inclination / pi. */
void orc_env_dir_to_uv(const float d[3], float uv[2])
{
    float zx = d[2], zy = d[0], zz = d[1];
    float az = atan2f(zy, zx);
    float cl = (zz < -1.0f) ? -1.0f : ((zz > 1.0f) ? 1.0f : zz);
    float incl = acosf(cl);
    uv[0] = (az + PI_F) * 0.5f / PI_F;
    uv[1] = 1.0f - incl * INV_PI_F;
}

void orc_env_uv_to_dir(const float uv[2], float d[3])
{
    float theta = uv[0] * PI_F * 2.0f - PI_F;
    float phi = (1.0f - uv[1]) * PI_F;
    float sT = sinf(theta), cT = cosf(theta), sP = sinf(phi), cP = cosf(phi);
    /* Z-up (cT sP, sT sP, cP) -> Y-up */
    d[0] = sT * sP; d[1] = cP; d[2] = cT * sP;
}

static inline float env_sa_pdf_sin(float pdf, float sinPhi)
{
    return (sinPhi <= 0.0f) ? 0.0f : pdf / (2.0f * PI_SQR_F * sinPhi);
}

static void rows_apply(const float m[12], const float v[3], float o[3])
{
    for(int r = 0; r < 3; r++) o[r] = m[4 * r] * v[0] + m[4 * r + 1] * v[1] + m[4 * r + 2] * v[2];
}

static inline int env_constant(const orc_pt_env* E) { return E->width == 1u && E->height == 1u; }

/* EmitViaSurfacePoint(wO): radiance seen along -wO. */
static void env_emit(const orc_pt_env* E, const float minusWo[3], float rgb[3])
{
    float dy[3];
    rows_apply(E->inv, minusWo, dy);
    normalize3f(dy);
    float uv[2] = { 0.0f, 0.0f };
    if(!env_constant(E)) orc_env_dir_to_uv(dy, uv);
    orc_env_read(E->texels, E->width, E->height, uv, rgb);
}

/* PdfSolidAngle(dir) (solid-angle density of sampling dir). */
static float env_pdf(const orc_pt_env* E, const float dir[3])
{
    float dy[3];
    rows_apply(E->inv, dir, dy);
    float dn[3] = { dy[0], dy[1], dy[2] };
    normalize3f(dn);
    float uv[2];
    orc_env_dir_to_uv(dn, uv);
    float pdf = env_constant(E) ? 1.0f : orc_pwc2d_pdf_uv(E->cdfX, E->cdfY, E->width, E->height, uv);
    float cl = (dy[1] < -1.0f) ? -1.0f : ((dy[1] > 1.0f) ? 1.0f : dy[1]);
    return env_sa_pdf_sin(pdf, sinf(acosf(cl)));
}

/* SampleSolidAngle: world direction and solid-angle pdf. */
static void env_sample(const orc_pt_env* E, float xi0, float xi1, float wdir[3], float* pdf)
{
    float uv[2], uvPdf;
    if(env_constant(E)) { uv[0] = xi0; uv[1] = xi1; uvPdf = 1.0f; }
    else
    {
        const float xi[2] = { xi0, xi1 };
        orc_pwc2d_sample_uv(E->cdfX, E->cdfY, E->width, E->height, xi, uv, &uvPdf);
    }
    float dy[3];
    orc_env_uv_to_dir(uv, dy);
    *pdf = env_sa_pdf_sin(uvPdf, sinf((1.0f - uv[1]) * PI_F));
    rows_apply(E->m, dy, wdir);
}

/* ------------------------------------------------------------------------ */
/* Spectral (Source/Tracer/SpectrumContext.{hpp,cu}, host backend)           */
/* ------------------------------------------------------------------------ */
#define CIE_START 360.0f

void orc_spec_prepare(const float* cieXyz, const float integrals[3], const float* spd, float normFactor,
                      uint32_t cieCount, float* observer, float* illuminant)
{
    /* SpectrumContext.cu:405-420: WEIGHT = 1 / CIE_SUM; factor = Y / norm */
    float w[3] = { 1.0f / integrals[0], 1.0f / integrals[1], 1.0f / integrals[2] };
    float f = integrals[1] / normFactor;
    for(uint32_t i = 0; i < cieCount; i++)
    {
        for(int k = 0; k < 3; k++) observer[3 * i + k] = cieXyz[3 * i + k] * w[k];
        illuminant[i] = spd[i] * f;
    }
}

/* The host texture view's linear read of fraction and base index for one
 * axis: texel = uv * n - 0.5, modf, negative fractions made absolute; CLAMP
 * edge resolve. */
static inline void tex_axis(float uv, uint32_t n, int32_t* i0, int32_t* i1, float* frac)
{
    float t = uv * (float)n - 0.5f, b;
    float f = modff(t, &b);
    int32_t s = (int32_t)b;
    if(f < 0.0f) { s -= 1; f = fabsf(f); }
    int32_t hi = (int32_t)n - 1;
    *i0 = s < 0 ? 0 : (s > hi ? hi : s);
    *i1 = (s + 1) < 0 ? 0 : ((s + 1) > hi ? hi : (s + 1));
    *frac = f;
}

static inline float lerpf_(float a, float b, float t) { return a * (1.0f - t) + b * t; }

/* 1D table read at a texel coordinate (normCoordinates = false). */
static void tex1d(const float* tab, uint32_t n, uint32_t ch, float coord, float* out)
{
    float uv = coord / (float)n;
    int32_t i0, i1; float f;
    tex_axis(uv, n, &i0, &i1, &f);
    for(uint32_t c = 0; c < ch; c++) out[c] = lerpf_(tab[(size_t)i0 * ch + c], tab[(size_t)i1 * ch + c], f);
}

/* Trilinear read of LUT texture `tex` (0..8) at normalised uvw. */
static float tex3d(const orc_spectral* S, uint32_t tex, const float uvw[3])
{
    const uint32_t n = S->lutRes;
    const float* t = S->lut + (size_t)tex * n * n * n;
    int32_t a0, a1, b0, b1, c0, c1; float fx, fy, fz;
    tex_axis(uvw[0], n, &a0, &a1, &fx);
    tex_axis(uvw[1], n, &b0, &b1, &fy);
    tex_axis(uvw[2], n, &c0, &c1, &fz);
#define T3(x, y, z) t[((size_t)(z) * n + (size_t)(y)) * n + (size_t)(x)]
    float p0 = lerpf_(T3(a0, b0, c0), T3(a1, b0, c0), fx);
    float p1 = lerpf_(T3(a0, b1, c0), T3(a1, b1, c0), fx);
    float p2 = lerpf_(T3(a0, b0, c1), T3(a1, b0, c1), fx);
    float p3 = lerpf_(T3(a0, b1, c1), T3(a1, b1, c1), fx);
#undef T3
    float q0 = lerpf_(p0, p1, fy), q1 = lerpf_(p2, p3, fy);
    return lerpf_(q0, q1, fz);
}

static inline float inv_smoothstep(float y)
{
    return 0.5f - sinf(asinf(1.0f - 2.0f * y) * (1.0f / 3.0f));
}

void orc_spec_sample_waves(float xi0, float waves[4], float pdf[4])
{
    static const float OFF[4] = { -0.5f, -0.25f, 0.0f, 0.25f };
    for(int i = 0; i < 4; i++)
    {
        float x = xi0 + OFF[i];
        if(x < 0.0f) x += 1.0f;
        if(x >= 1.0f) x -= 1.0f;
        float a = 0.85691062f - 1.82750197f * x;
        float l = 538.0f - 138.888889f * atanhf(a);
        float d = coshf(0.0072f * (l - 538.0f));
        d = d * d;
        waves[i] = l;
        pdf[i] = 0.0039398042f / d;
    }
}

/* Converter::ConvertAlbedo (SpectrumContext.hpp:36-130) */
void orc_spec_convert_albedo(const orc_spectral* S, const float rgb[3], const float waves[4], float out[4])
{
    uint32_t maxI = 0;
    float mx = rgb[0];
    for(uint32_t i = 1; i < 3; i++) if(rgb[i] > mx) { mx = rgb[i]; maxI = i; }
    float xyz[3] = { 0.0f, 0.0f, 0.0f };
    if(mx > 1.0e-7f)
    {
        float f = 1.0f / mx;
        xyz[0] = rgb[(maxI + 1) % 3] * f;
        xyz[1] = rgb[(maxI + 2) % 3] * f;
    }
    float slice = mx < 0.0f ? 0.0f : (mx > 1.0f ? 1.0f : mx);
    xyz[2] = inv_smoothstep(inv_smoothstep(slice));
    const float N = (float)S->lutRes;
    const float A = (N - 1.0f) / N, B = 0.5f / N;
    float uvw[3];
    for(int k = 0; k < 3; k++) uvw[k] = xyz[k] * A + B;
    float c[3];
    for(uint32_t k = 0; k < 3; k++) c[k] = tex3d(S, 3 * maxI + k, uvw);
    for(int i = 0; i < 4; i++)
    {
        float t = fmaf(c[0], waves[i], c[1]);
        float x = fmaf(t, waves[i], c[2]);
        float dr = 1.0f / sqrtf(fmaf(x, x, 1.0f));
        out[i] = fmaf(0.5f * x, dr, 0.5f);
    }
}

/* Converter::ConvertRadiance (SpectrumContext.hpp:132-152) */
void orc_spec_convert_radiance(const orc_spectral* S, const float rgb[3], const float waves[4], float out[4])
{
    uint32_t maxI = 0;
    float mx = rgb[0];
    for(uint32_t i = 1; i < 3; i++) if(rgb[i] > mx) { mx = rgb[i]; maxI = i; }
    (void)maxI;
    float scale = mx * 2.0f;
    float c[3] = { 0.0f, 0.0f, 0.0f };
    if(scale != 0.0f) for(int k = 0; k < 3; k++) c[k] = rgb[k] / scale;
    orc_spec_convert_albedo(S, c, waves, out);
    for(int i = 0; i < 4; i++)
    {
        float il;
        tex1d(S->illuminant, S->cieCount, 1, waves[i] + (0.5f - CIE_START), &il);
        out[i] *= il;
    }
    for(int i = 0; i < 4; i++) out[i] *= scale;
}

/* ConvertSpectraToRGBSingle (SpectrumContext.cu:137-170), no dispersion */
void orc_spec_to_rgb(const orc_spectral* S, const float value[4], const float waves[4], const float pdf[4],
                     float rgb[3])
{
    float xyz[3] = { 0.0f, 0.0f, 0.0f };
    for(int i = 0; i < 4; i++)
    {
        float f[3];
        tex1d(S->observer, S->cieCount, 3, waves[i] + (0.5f - CIE_START), f);
        float v = (pdf[i] == 0.0f) ? 0.0f : value[i] / pdf[i];
        for(int k = 0; k < 3; k++) xyz[k] += f[k] * v;
    }
    for(int k = 0; k < 3; k++) xyz[k] *= 0.25f;
    for(int r = 0; r < 3; r++)
        rgb[r] = fmaf(S->xyzToRgb[3 * r + 2], xyz[2], fmaf(S->xyzToRgb[3 * r + 1], xyz[1], S->xyzToRgb[3 * r] * xyz[0]));
}

typedef struct
{
    const orc_scene*          scene;
    const orc_pt_params*      p;
    const orc_pt_surface*     surfaces;     /* per instance */
    const orc_pt_light_tri*   lights;
    uint32_t                  nLights;      /* triangle lights */
    const orc_pt_env*         env;          /* boundary light (last), or NULL */
    const orc_spectral*       spec;         /* NULL: RGB */
    /* adjoint (orc_pt_adjoint) */
    const void*               adjTexels;
    uint32_t                  adjW, adjH;
    const float*              adjDelta;
    double*                   adjGrad;      /* one buffer per worker */
    double*                   adjGradE;     /* one buffer per worker, or NULL */
    uint32_t                  adjInstances;
    int                       adjWorkers;
    atomic_int                adjNextBuffer;
    float*                    image;
    atomic_uint               nextRow;
    uint32_t*                 zsSeeds;      /* ZSobol per-pixel seeds, or NULL */
    uint32_t                  zsResBits;
} pt_job;

/* One ray cast through the oracle accelerator. */
static int cast1(const orc_scene* s, const float o[3], const float d[3], float tmin, float tmax,
                 orc_hit_keys* hk, orc_meta_hit* mh, uint32_t* inst, float* tOut)
{
    orc_ray_gmem r;
    memcpy(r.pos, o, 12); memcpy(r.dir, d, 12);
    r.tMin = tmin; r.tMax = tmax;
    uint32_t in = 0xFFFFFFFFu;
    orc_cast_closest(s, &r, NULL, 1, hk, mh, &in, 1);
    *inst = in;
    *tOut = r.tMax;
    return in != 0xFFFFFFFFu;
}
static int visible1(const orc_scene* s, const float o[3], const float d[3], float tmin, float tmax)
{
    orc_ray_gmem r;
    memcpy(r.pos, o, 12); memcpy(r.dir, d, 12);
    r.tMin = tmin; r.tMax = tmax;
    uint32_t bits = 0;
    orc_cast_visibility(s, &r, NULL, 1, &bits, 1);
    return (bits & 1u) != 0u;
}

/* Surface point of a hit: barycentric position in instance space, moved to
 * world space with ApplyP; geometric normal with ApplyN (transpose of the
 * inverse, TransformsDefault.hpp:19-36). */
static void surface_of(const orc_pt_surface* sf, const float* tri9 /* v0 v1 v2 local */,
                       float u, float v, float pos[3], float n[3])
{
    float e0[3] = { tri9[3] - tri9[0], tri9[4] - tri9[1], tri9[5] - tri9[2] };
    float e1[3] = { tri9[6] - tri9[0], tri9[7] - tri9[1], tri9[8] - tri9[2] };
    float pl[3];
    for(int k = 0; k < 3; k++) pl[k] = tri9[k] + e0[k] * u + e1[k] * v;
    for(int r = 0; r < 3; r++)
        pos[r] = sf->m[4 * r] * pl[0] + sf->m[4 * r + 1] * pl[1] + sf->m[4 * r + 2] * pl[2] + sf->m[4 * r + 3];
    float nl[3];
    cross3f(e0, e1, nl);
    /* ApplyN: inv^T * n */
    for(int c = 0; c < 3; c++)
        n[c] = sf->inv[c] * nl[0] + sf->inv[4 + c] * nl[1] + sf->inv[8 + c] * nl[2];
    normalize3f(n);
}

/* Math::InvErrFunc, host branch (Source/Core/Math.h:787-833): the
 * single-precision inverse error function of M. Giles, "Approximating the
 * erfinv function" (GPU Computing Gems, Jade Edition, 2011), evaluated with
 * fma as MRay writes it.  (MRay's CUDA backend calls erfinvf instead.) */
static float inv_erf(float x)
{
    float t = logf(fmaf(x, 0.0f - x, 1.0f));
    float p;
    if(fabsf(t) > 6.125f)
    {
        p = 3.03697567e-10f;
        p = fmaf(p, t, 2.93243101e-8f);
        p = fmaf(p, t, 1.22150334e-6f);
        p = fmaf(p, t, 2.84108955e-5f);
        p = fmaf(p, t, 3.93552968e-4f);
        p = fmaf(p, t, 3.02698812e-3f);
        p = fmaf(p, t, 4.83185798e-3f);
        p = fmaf(p, t, -2.64646143e-1f);
        p = fmaf(p, t, 8.40016484e-1f);
    }
    else
    {
        p = 5.438778320e-9f;
        p = fmaf(p, t, 1.43285448e-7f);
        p = fmaf(p, t, 1.22774793e-6f);
        p = fmaf(p, t, 1.12963626e-7f);
        p = fmaf(p, t, -5.61530760e-5f);
        p = fmaf(p, t, -1.47697632e-4f);
        p = fmaf(p, t, 2.31468678e-3f);
        p = fmaf(p, t, 1.15392581e-2f);
        p = fmaf(p, t, -2.32015476e-1f);
        p = fmaf(p, t, 8.86226892e-1f);
    }
    return x * p;
}

/* Math::Gaussian (Math.h:1031-1042) */
static float gaussian(float x, float sigma)
{
    const float invSqrt2Pi = (1.0f / 1.4142135623730950488f) * (1.0f / 1.772453850905516027298f);
    float sigmaInv = 1.0f / sigma;
    float r = invSqrt2Pi * sigmaInv;
    float pw = (x - 0.0f) * sigmaInv;
    return r * expf(-0.5f * pw * pw);
}

/* Common::SampleGaussian with mu = 0 (DistributionFunctions.h:686-705):
 * inverse-CDF sample, clamped to 3.5 sigma where the inverse error function
 * runs off to infinity. */
static float sample_gaussian(float xi, float sigma)
{
    float x = 1.4142135623730950488f * sigma;
    float e = inv_erf(2.0f * xi - 1.0f);
    x = x * e + 0.0f;
    if(isinf(e))
    {
        float mm = 3.5f * sigma;
        x = x < -mm ? -mm : (x > mm ? mm : x);
    }
    return x;
}

/* GaussianFilter::Sample (Filters.h:195-219): per-axis offsets in pixels,
 * sigma = radius * 0.285714.  The film weight Evaluate / pdf is the ratio of
 * equal products, so 1. */
static void filter_sample(float radius, float xi0, float xi1, float* ox, float* oy)
{
    float sigma = radius * 0.285714f;
    *ox = sample_gaussian(xi0, sigma);
    *oy = sample_gaussian(xi1, sigma);
}

/* LightPrim<Triangle>::SampleSolidAngle (LightsDefault.hpp:22-45) with the
 * triangle's area sampling (Osada et al., PrimitiveDefaultTriangle.hpp:48-80)
 * towards the shaded point pos, and EmitViaSurfacePoint's side test: lp,
 * the solid-angle pdf and the emitted RGB (zero from a one-sided light's
 * back). */
static void light_tri_sample(const orc_pt_light_tri* L, float xi0, float xi1, const float pos[3], float lp[3],
                             float* pdf, float emis[3])
{
    float r1 = sqrtf(xi0), r2 = xi1;
    float a = 1.0f - r1, b = (1.0f - r2) * r1, c = r1 * r2;
    for(int k = 0; k < 3; k++) lp[k] = L->p0[k] * a + L->p1[k] * b + L->p2[k] * c;
    float sd[3] = { pos[0] - lp[0], pos[1] - lp[1], pos[2] - lp[2] };
    float distSq = dot3f(sd, sd);
    normalize3f(sd);
    float ndl = dot3f(L->n, sd);
    ndl = L->twoSided ? fabsf(ndl) : fmaxf(0.0f, ndl);
    float ppdf = (ndl == 0.0f) ? 0.0f : (1.0f / L->area) / ndl;
    *pdf = ppdf * distSq;
    emis[0] = emis[1] = emis[2] = 0.0f;
    if(L->twoSided || dot3f(L->n, sd) > 0.0f)
        for(int k = 0; k < 3; k++) emis[k] = L->radiance[k];
}

/* LightPrim<Triangle>::PdfSolidAngle (LightsDefault.hpp:47-66): the light
 * hit at barycentrics (a, b) of its world-space vertices
 * (Triangle::SurfaceFromHit, PrimitiveDefaultTriangle.hpp:320-350), seen
 * from org along dir. */
static float light_tri_pdf(const orc_pt_light_tri* L, float a, float b, const float org[3], const float dir[3])
{
    const float md[3] = { -dir[0], -dir[1], -dir[2] };
    float ndl = dot3f(L->n, md);
    ndl = L->twoSided ? fabsf(ndl) : fmaxf(0.0f, ndl);
    float c = 1.0f - a - b;
    /* SurfaceFromHit / PdfSurface: no surface outside the triangle */
    if(a < 0.0f || a > 1.0f || b < 0.0f || b > 1.0f || c < 0.0f || c > 1.0f) return 0.0f;
    float pos[3];
    for(int k = 0; k < 3; k++) pos[k] = L->p0[k] * a + L->p1[k] * b + L->p2[k] * c;
    float dd[3] = { org[0] - pos[0], org[1] - pos[1], org[2] - pos[2] };
    float lpdf = (ndl == 0.0f) ? 0.0f : (1.0f / L->area) / ndl;
    return lpdf * dot3f(dd, dd);
}

/* EmitViaHit's side test (LightsDefault.hpp:125-145): a one-sided light
 * emits towards wo only when it faces it. */
static int light_tri_emits(const orc_pt_light_tri* L, const float wo[3])
{
    return L->twoSided ? 1 : (dot3f(L->n, wo) > 0.0f);
}

/* ------------------------------------------------------------------------ */
/* Mip chains, mip-mapped reads and ray cones.                              */
/*   KCGenerateMipmaps / FilterPixel     Source/Tracer/TextureFilter.cu:62-192 */
/*   ConvertPixelIndices, TextureMipSize Source/Core/GraphicsFunctions.h:474-538 */
/*   TextureViewCPU gradient / LOD read  Source/Device/CPU/TextureViewCPU.h:405-470 */
/*     (gradients taken in texels)                                          */
/*   RayCone Advance / Project, ConeAfterScatter  Source/Tracer/TracerTypes.h:323-380 */
/*   texture gradients of a hit          PrimitiveDefaultTriangle.hpp:491-569 */
/*   RefractMaterial::RefractRayCone     Source/Tracer/MaterialsDefault.hpp:353-462 */
/* ------------------------------------------------------------------------ */
#define CONE_EPS 1.0e-5f

static inline uint32_t mip_dim(uint32_t r, uint32_t m) { return (r >> m) ? (r >> m) : 1u; }

/* texels of levels 1 .. levels - 1 of a w x h chain (the offset of level m is
 * chain_texels(w, h, m)) */
static size_t chain_texels(uint32_t w, uint32_t h, uint32_t levels)
{
    size_t n = 0;
    for(uint32_t m = 1; m < levels && (mip_dim(w, m - 1) > 1u || mip_dim(h, m - 1) > 1u); m++)
        n += (size_t)mip_dim(w, m) * mip_dim(h, m);
    return n;
}

uint32_t orc_gen_mips_levels(const void* texels, uint32_t w, uint32_t h, uint32_t format, float radius,
                             uint32_t levels, uint32_t validMask, void* out)
{
    float off[8], g[8];
    const float sigma = radius * 0.285714f;
    for(int k = 0; k < 8; k++)
    {
        const float d = 1.0f / 8.0f;
        const float xi = d * 0.5f + d * (float)k;
        off[k] = xi * 2.0f * radius - radius;
        g[k] = gaussian(off[k], sigma);
    }
    const size_t bpp = (format == 0u) ? 4u : 16u;
    unsigned char* chain = (unsigned char*)out;
    for(uint32_t m = 1; m < levels; m++)
    {
        if(validMask & (1u << m)) continue;        /* a given level is kept */
        const uint32_t pw = mip_dim(w, m - 1), ph = mip_dim(h, m - 1);
        const uint32_t cw = mip_dim(w, m), ch = mip_dim(h, m);
        const unsigned char* src = (m == 1u) ? (const unsigned char*)texels : chain + chain_texels(w, h, m - 1) * bpp;
        unsigned char* dst = chain + chain_texels(w, h, m) * bpp;
        const float rx = (float)pw / (float)cw, ry = (float)ph / (float)ch;
        for(uint32_t y = 0; y < ch; y++)
            for(uint32_t x = 0; x < cw; x++)
            {
                float acc[4] = { 0, 0, 0, 0 }, wsum = 0.0f;
                for(int sy = 0; sy < 8; sy++)
                {
                    float py = (((float)y + off[sy]) + 0.5f) * ry - 0.5f;
                    py = fminf(fmaxf(0.0f, py), (float)(ph - 1u));
                    const uint32_t iy = (uint32_t)lroundf(py);
                    for(int sx = 0; sx < 8; sx++)
                    {
                        float px = (((float)x + off[sx]) + 0.5f) * rx - 0.5f;
                        px = fminf(fmaxf(0.0f, px), (float)(pw - 1u));
                        const uint32_t ix = (uint32_t)lroundf(px);
                        const float wgt = g[sx] * g[sy];
                        const size_t t = (size_t)iy * pw + ix;
                        float v[4];
                        if(format == 0u) for(int k = 0; k < 4; k++) v[k] = (float)src[4 * t + k];
                        else memcpy(v, src + 16 * t, 16);
                        for(int k = 0; k < 4; k++) acc[k] = acc[k] + wgt * v[k];
                        wsum = wsum + wgt;
                    }
                }
                const size_t o = (size_t)y * cw + x;
                for(int k = 0; k < 4; k++)
                {
                    const float r = acc[k] / wsum;
                    if(format == 0u) dst[4 * o + k] = (unsigned char)fminf(fmaxf(roundf(r), 0.0f), 255.0f);
                    else memcpy(dst + 16 * o + 4 * k, &r, 4);
                }
            }
    }
    return levels;
}

uint32_t orc_gen_mips(const void* texels, uint32_t w, uint32_t h, uint32_t format, float radius, void* out)
{
    uint32_t levels = 0;
    for(uint32_t m = w > h ? w : h; m; m >>= 1) levels++;
    return orc_gen_mips_levels(texels, w, h, format, radius, levels, 0u, out);
}

/* level m of a surface's texture: base pointer and size */
static const void* mip_base(const orc_pt_surface* sf, uint32_t m, uint32_t* w, uint32_t* h)
{
    *w = mip_dim(sf->texW, m);
    *h = mip_dim(sf->texH, m);
    if(m == 0u) return sf->texels;
    size_t start = 0;
    for(uint32_t k = 1; k < m; k++) start += (size_t)mip_dim(sf->texW, k) * mip_dim(sf->texH, k);
    return (const char*)sf->mips + start * (sf->texFormat == 0u ? 4u : 16u);
}

static void tex_read_grad(const orc_pt_surface* sf, const float uv[2], const float dx[2], const float dy[2], float rgb[3])
{
    const float sx = (float)sf->texW, sy = (float)sf->texH;
    const float gx0 = dx[0] * sx, gx1 = dx[1] * sy, gy0 = dy[0] * sx, gy1 = dy[1] * sy;
    const float lx = fmaf(gx1, gx1, fmaf(gx0, gx0, 0.0f)), ly = fmaf(gy1, gy1, fmaf(gy0, gy0, 0.0f));
    float level = 0.5f * log2f(fmaxf(lx, ly));
    level = fminf(fmaxf(0.0f, level), (float)(sf->mipCount - 1u));
    float m0f;
    const float frac = modff(level, &m0f);
    const uint32_t m0 = (uint32_t)m0f, m1 = (m0 + 1u < sf->mipCount) ? m0 + 1u : sf->mipCount - 1u;
    uint32_t w, h;
    const void* b0 = mip_base(sf, m0, &w, &h);
    float p0[3];
    orc_tex_read(b0, w, h, sf->texFormat, uv, p0);
    if(m0 == m1) { memcpy(rgb, p0, 12); return; }
    const void* b1 = mip_base(sf, m1, &w, &h);
    float p1[3];
    orc_tex_read(b1, w, h, sf->texFormat, uv, p1);
    for(int k = 0; k < 3; k++) rgb[k] = p0[k] * (1.0f - frac) + p1[k] * frac;
}

typedef struct { float aperture, width; } cone_t;

static cone_t cone_advance(cone_t c, float t)
{
    cone_t r = { c.aperture, fminf(fmaxf(CONE_EPS, c.width + c.aperture * t), 1.0e6f) };
    return r;
}

static void cone_project(cone_t c, const float f[3], const float dIn[3], float a1[3], float a2[3])
{
    float d[3] = { dIn[0], dIn[1], dIn[2] };
    const float fDotD = dot3f(f, d);
    if(fabsf(fDotD + 1.0f) < CONE_EPS) for(int k = 0; k < 3; k++) d[k] = d[k] + CONE_EPS;
    float h[2][3];
    for(int k = 0; k < 3; k++) h[0][k] = d[k] - fDotD * f[k];
    cross3f(f, h[0], h[1]);
    const float r = c.width * 0.5f;
    float* out[2] = { a1, a2 };
    for(int j = 0; j < 2; j++)
    {
        const float dh = dot3f(d, h[j]);
        float q[3];
        for(int k = 0; k < 3; k++) q[k] = h[j][k] - dh * d[k];
        const float denom = fmaxf(CONE_EPS, sqrtf(dot3f(q, q)));
        const float sc = r / denom;
        for(int k = 0; k < 3; k++) out[j][k] = sc * h[j][k];
    }
}

/* Albedo of a textured surface with a mip chain, read at the cone's level:
 * the triangle's corner and edges in world space (edges by the transform's
 * linear part), f its normal facing the ray, d the ray direction. */
static void albedo_lod(const orc_pt_surface* sf, const float* tri9, const float uv[2], const float uvq[6],
                       const float pos[3], const float f[3], const float d[3], cone_t cone, float rgb[3])
{
    const float e0l[3] = { tri9[3] - tri9[0], tri9[4] - tri9[1], tri9[5] - tri9[2] };
    const float e1l[3] = { tri9[6] - tri9[0], tri9[7] - tri9[1], tri9[8] - tri9[2] };
    float P0[3], E0[3], E1[3];
    for(int r = 0; r < 3; r++)
    {
        P0[r] = sf->m[4 * r] * tri9[0] + sf->m[4 * r + 1] * tri9[1] + sf->m[4 * r + 2] * tri9[2] + sf->m[4 * r + 3];
        E0[r] = sf->m[4 * r] * e0l[0] + sf->m[4 * r + 1] * e0l[1] + sf->m[4 * r + 2] * e0l[2];
        E1[r] = sf->m[4 * r] * e1l[0] + sf->m[4 * r + 1] * e1l[1] + sf->m[4 * r + 2] * e1l[2];
    }
    float dn[3] = { d[0], d[1], d[2] };
    normalize3f(dn);
    float a[2][3];
    cone_project(cone, f, dn, a[0], a[1]);
    float c01[3];
    cross3f(E0, E1, c01);
    const float areaRecip = 1.0f / dot3f(f, c01);
    float grad[2][2];
    for(int j = 0; j < 2; j++)
    {
        float eP[3], c1[3], c2[3];
        for(int k = 0; k < 3; k++) eP[k] = (pos[k] - P0[k]) + a[j][k];
        cross3f(eP, E1, c1);
        cross3f(E0, eP, c2);
        for(int k = 0; k < 3; k++) { c1[k] = c1[k] * areaRecip; c2[k] = c2[k] * areaRecip; }
        const float ba = dot3f(f, c1), bb = dot3f(f, c2);
        const float bc = (1.0f - ba) - bb;
        for(int k = 0; k < 2; k++) grad[j][k] = (uvq[k] * bc + uvq[2 + k] * ba + uvq[4 + k] * bb) - uv[k];
    }
    tex_read_grad(sf, uv, grad[0], grad[1], rgb);
}

/* Unreal's textured roughness / metallic / specular at a hit (UnrealMaterial's
 * constructor reads each at the surface's uv and gradients,
 * MaterialsDefault.hpp:521-533): the first channel, read like the albedo,
 * replaces the constant in a copy of the surface; other surfaces come back
 * as they are. */
static const orc_pt_surface* unreal_params(const orc_pt_surface* sf, uint32_t localPrim, const orc_meta_hit* mh,
                                           const float* tri9, const float pos[3], const float nrm[3],
                                           const float dir[3], cone_t cone, orc_pt_surface* tmp)
{
    if(sf->matType != ORC_MAT_UNREAL || !sf->uvs ||
       !(sf->param[0].texels || sf->param[1].texels || sf->param[2].texels))
        return sf;
    *tmp = *sf;
    const float* q = &sf->uvs[6 * localPrim];
    const float a = mh->bary[0], b = mh->bary[1], c = 1.0f - a - b;
    float uv[2];
    for(int k = 0; k < 2; k++) uv[k] = q[k] * a + q[2 + k] * b + q[4 + k] * c;
    float* dst[3] = { &tmp->roughness, &tmp->metallic, &tmp->specular };
    for(int k = 0; k < 3; k++)
    {
        const orc_pt_tex* t = &sf->param[k];
        if(!t->texels) continue;
        orc_pt_surface ts = *sf;
        ts.texels = t->texels; ts.texW = t->w; ts.texH = t->h; ts.texFormat = t->format;
        ts.mips = t->mips; ts.mipCount = t->mipCount ? t->mipCount : 1u;
        float v[4] = { 0, 0, 0, 0 };
        if(ts.mipCount > 1u) albedo_lod(&ts, tri9, uv, q, pos, nrm, dir, cone, v);
        else orc_tex_read(ts.texels, ts.texW, ts.texH, ts.texFormat, uv, v);
        *dst[k] = v[0];
    }
    return tmp;
}

static inline float dot2f(const float a[2], const float b[2]) { return fmaf(a[1], b[1], fmaf(a[0], b[0], 0.0f)); }

static void refract2d(const float v[2], const float n[2], float fromEta, float toEta, float out[2])
{
    const float etaRatio = fromEta / toEta;
    const float cosIn = fmaf(0.0f, 0.0f, fmaf(n[1], -v[1], fmaf(n[0], -v[0], 0.0f)));
    const float sinInSqr = fmaxf(0.0f, 1.0f - cosIn * cosIn);
    const float sinOutSqr = etaRatio * etaRatio * sinInSqr;
    const float cosOut = sqrt_max(1.0f - sinOutSqr);
    if(sinOutSqr >= 1.0f)
    {
        const float nv = dot2f(n, v);
        float q[2] = { v[0] - n[0] * nv, v[1] - n[1] * nv };
        const float inv = 1.0f / sqrtf(dot2f(q, q));
        out[0] = q[0] * inv;
        out[1] = q[1] * inv;
        return;
    }
    const float k = etaRatio * cosIn - cosOut;
    out[0] = etaRatio * v[0] + k * n[0];
    out[1] = etaRatio * v[1] + k * n[1];
}

static int refract_cone(cone_t front, float betaN, const float wo[3], const float n[3], float fromEta, float toEta,
                        cone_t* back)
{
    const float etaRatio = fromEta / toEta;
    const float cosIn = dot3f(n, wo);
    const float sinInSqr = fmaxf(0.0f, 1.0f - cosIn * cosIn);
    const float sinOutSqr = etaRatio * etaRatio * sinInSqr;
    if(sinOutSqr >= 1.0f) return 0;
    const float d3[3] = { -wo[0], -wo[1], -wo[2] };
    const float dn = dot3f(d3, n);
    float x[3] = { d3[0] - n[0] * dn, d3[1] - n[1] * dn, d3[2] - n[2] * dn };
    normalize3f(x);
    const float d[2] = { dot3f(x, d3), dot3f(n, d3) };
    const float wSign = (front.width > 0.0f) ? 1.0f : 0.0f;
    const float alpha = wSign * front.aperture * 0.5f;
    const float s = sinf(alpha), c = cosf(alpha);
    const float du[2] = { d[0] * c - d[1] * s, d[0] * s + d[1] * c };
    const float dl[2] = { d[0] * c + d[1] * s, d[0] * -s + d[1] * c };
    float orthoD[2] = { -d[1] * front.width * 0.5f, d[0] * front.width * 0.5f };
    const float uHitX = +orthoD[0] + du[0] * (-orthoD[1] / du[1]);
    const float lHitX = -orthoD[0] + dl[0] * (+orthoD[1] / dl[1]);
    const float nSign = (uHitX > lHitX) ? 1.0f : -1.0f;
    const float dTheta = -betaN * nSign * 0.5f;
    const float ns = sinf(dTheta), nc = cosf(dTheta);
    const float nu[2] = { 0.0f * nc - 1.0f * ns, 0.0f * ns + 1.0f * nc };
    const float nl[2] = { 0.0f * nc + 1.0f * ns, 0.0f * -ns + 1.0f * nc };
    float tu[2], tl[2];
    refract2d(du, nu, fromEta, toEta, tu);
    refract2d(dl, nl, fromEta, toEta, tl);
    orthoD[0] = -d[1];
    orthoD[1] = d[0];
    const float pu[2] = { -tu[1], tu[0] }, pl[2] = { -tl[1], tl[0] };
    float wl = -uHitX * tu[1];
    wl /= dot2f(orthoD, pu);
    float wu = +lHitX * tl[1];
    wu /= dot2f(orthoD, pl);
    const float sgn = copysignf(1.0f, tu[0] * tl[1] - tu[1] * tl[0]);
    const float cosTheta = fminf(fmaxf(-1.0f, dot2f(tu, tl)), 1.0f);
    float ap = acosf(cosTheta) * sgn;
    ap = fmaxf(ap, CONE_EPS);
    back->aperture = ap + betaN;
    back->width = wu + wl;
    return 1;
}

/* RefractRayCone then ConeAfterScatter (betaN = 0: no vertex normals) */
static cone_t cone_after_scatter(const orc_pt_surface* sf, int backSide, cone_t cone, const float wo[3],
                                 const float n[3], const float wi[3])
{
    cone_t back = cone;
    if(sf->matType == ORC_MAT_REFRACT && dot3f(wi, n) <= 0.0f)
    {
        float fromEta = sf->iorFront, toEta = sf->iorBack;
        if(backSide) { const float t = fromEta; fromEta = toEta; toEta = t; }
        cone_t r;
        if(refract_cone(cone, 0.0f, wo, n, fromEta, toEta, &r)) back = r;
    }
    cone_t out;
    if(dot3f(wi, n) > 0.0f) { out.aperture = cone.aperture + 2.0f * 0.0f; out.width = cone.width; }
    else { out.aperture = back.aperture - 0.0f; out.width = back.width; }
    return out;
}

/* CameraPinhole::EvaluateRay (CamerasDefault.hpp:94-135) for pixel (x, y)
 * and a film-filter offset (ox, oy) in pixels. */
static void camera_ray(const orc_pt_params* P, uint32_t x, uint32_t y, float ox, float oy, float dir[3], float org[3])
{
    float dx = P->planeSize[0] / (float)P->width, dy = P->planeSize[1] / (float)P->height;
    float sx = ((float)x + (ox + 0.5f)) * dx, sy = ((float)y + (oy + 0.5f)) * dy;
    for(int k = 0; k < 3; k++)
    {
        float sp = P->camBottomLeft[k] + sx * P->camRight[k] + sy * P->camUp[k];
        dir[k] = sp - P->camPos[k];
        org[k] = P->camPos[k];
    }
    normalize3f(dir);
}

/* adj: NULL for a primal trace; else {primal radiance[3], delta / spp [3]}
 * and the worker's gradient buffer. */
typedef struct { float tot[3]; float d[3]; double* grad; double* gradE; } adj_ctx;

static void tex_taps(uint32_t w, uint32_t h, const float uv[2], size_t idx[4], float wt[4])
{
    float tx = uv[0] * (float)w - 0.5f, ty = uv[1] * (float)h - 0.5f;
    float bx, by;
    float fx = modff(tx, &bx), fy = modff(ty, &by);
    int32_t sx = (int32_t)bx, sy = (int32_t)by;
    if(fx < 0.0f) { sx -= 1; fx = fabsf(fx); }
    if(fy < 0.0f) { sy -= 1; fy = fabsf(fy); }
    int32_t x0 = wrap_index(sx, (int32_t)w), x1 = wrap_index(sx + 1, (int32_t)w);
    int32_t y0 = wrap_index(sy, (int32_t)h), y1 = wrap_index(sy + 1, (int32_t)h);
    float gx = 1.0f - fx, gy = 1.0f - fy;
    idx[0] = (size_t)y0 * w + x0; wt[0] = gx * gy;
    idx[1] = (size_t)y0 * w + x1; wt[1] = fx * gy;
    idx[2] = (size_t)y1 * w + x0; wt[2] = gx * fy;
    idx[3] = (size_t)y1 * w + x1; wt[3] = fx * fy;
}

static void trace_sample_adj(pt_job* J, uint32_t x, uint32_t y, uint32_t sample, float outRad[3], adj_ctx* adj);

static void trace_sample(pt_job* J, uint32_t x, uint32_t y, uint32_t sample, float outRad[3])
{
    trace_sample_adj(J, x, y, sample, outRad, NULL);
}

static void trace_sample_adj(pt_job* J, uint32_t x, uint32_t y, uint32_t sample, float outRad[3], adj_ctx* adj)
{
    const orc_pt_params* P = J->p;
    const uint32_t pixel = y * P->width + x;
    const uint32_t key = path_key(P->seed, pixel, sample);
    smp_ctx SC = { key, x, y, sample, J->zsSeeds ? J->zsSeeds[pixel] : 0u, J->zsSeeds ? P->sampler : 0u,
                   P->samplerMaxSpp ? P->samplerMaxSpp : P->sampleStart + P->spp, J->zsResBits, P->maxDepth };
    outRad[0] = outRad[1] = outRad[2] = 0.0f;

    /* camera ray: Gaussian film-filter offset (weight Evaluate / pdf = 1) */
    float ox, oy;
    filter_sample(P->filterRadius, urnd(&SC, 0, 6), urnd(&SC, 0, 7), &ox, &oy);
    float dir[3], org[3];
    camera_ray(P, x, y, ox, oy, dir, org);
    float tmin = P->nearT, tmax = P->farT;
    cone_t cone = { P->coneAperture, 0.0f };

    float thr[4] = { 1.0f, 1.0f, 1.0f, 1.0f };
    float rad[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
    /* spectral: 4 wavelengths per path, sampled at the camera */
    const orc_spectral* S = J->spec;
    const int nc = S ? 4 : 3;
    float waves[4] = { 0, 0, 0, 0 }, wpdf[4] = { 1, 1, 1, 1 };
    if(S) orc_spec_sample_waves(urnd(&SC, 0, 9), waves, wpdf);
    uint32_t depth = 0;
    int type = 0;           /* 0 camera, 1 path (diffuse) */
    float prevPdf = 0.0f;
    const orc_pt_env* E = J->env;
    const uint32_t nAll = J->nLights + (E ? 1u : 0u);
    const float invN = nAll ? 1.0f / (float)nAll : 0.0f;

    for(;;)
    {
        orc_hit_keys hk; orc_meta_hit mh; uint32_t inst; float t;
        if(!cast1(J->scene, org, dir, tmin, tmax, &hk, &mh, &inst, &t))
        {
            /* miss: boundary light work (LightWorkFunction[WithNEE] with the
             * skysphere, PathTracerRendererShaders.h:308-345, 450-517) */
            if(!E || (P->sampleMode == ORC_PT_NEE && type == 1)) break;
            float tp[4] = { thr[0], thr[1], thr[2], thr[3] };
            if(P->sampleMode == ORC_PT_NEE_MIS && type == 1)
            {
                float lpdf = env_pdf(E, dir) * invN;
                float misPdf = prevPdf + lpdf;
                for(int k = 0; k < nc; k++) tp[k] *= prevPdf;
                if(misPdf == 0.0f) { tp[0] = tp[1] = tp[2] = tp[3] = 0.0f; }
                else { float inv = 1.0f / misPdf; for(int k = 0; k < nc; k++) tp[k] *= inv; }
            }
            float em[4];
            env_emit(E, dir, em);
            if(S) { float c[3] = { em[0], em[1], em[2] }; orc_spec_convert_radiance(S, c, waves, em); }
            if(depth + 1u <= P->maxDepth)
                for(int k = 0; k < nc; k++) rad[k] += em[k] * tp[k];
            break;
        }
        const orc_pt_surface* sf = &J->surfaces[inst];
        uint32_t localPrim = hk.primKey - sf->primKeyBase;
        const float* tri9 = &sf->triangles[9 * localPrim];
        /* MetaHit = (w, u); v = 1 - w - u */
        float bu = mh.bary[1];
        float bv = 1.0f - mh.bary[0] - mh.bary[1];
        float pos[3], gn[3];
        surface_of(sf, tri9, bu, bv, pos, gn);

        if(sf->isLight)
        {
            /* NEE-only mode: only camera and specular rays see emission */
            if(P->sampleMode == ORC_PT_NEE && type == 1) break;
            float tp[4] = { thr[0], thr[1], thr[2], thr[3] };
            if(P->sampleMode == ORC_PT_NEE_MIS && type == 1)
            {
                const orc_pt_light_tri* L = &J->lights[sf->lightBase + localPrim];
                /* PdfSolidAngle(hit, ray.pos, ray.dir) * 1/N; the hit is MRay's (a, b) = MetaHit */
                float lpdf = light_tri_pdf(L, mh.bary[0], mh.bary[1], org, dir) * invN;
                float misPdf = prevPdf + lpdf;
                for(int k = 0; k < nc; k++) tp[k] *= prevPdf;
                if(misPdf == 0.0f) { tp[0] = tp[1] = tp[2] = tp[3] = 0.0f; }
                else { float inv = 1.0f / misPdf; for(int k = 0; k < nc; k++) tp[k] *= inv; }
            }
            const orc_pt_light_tri* L = &J->lights[sf->lightBase + localPrim];
            float wo[3] = { -dir[0], -dir[1], -dir[2] };
            int emits = light_tri_emits(L, wo);
            float lr[4] = { L->radiance[0], L->radiance[1], L->radiance[2], 0.0f };
            if(S) orc_spec_convert_radiance(S, L->radiance, waves, lr);
            if(emits && depth + 1u <= P->maxDepth)
            {
                for(int k = 0; k < nc; k++) rad[k] += lr[k] * tp[k];
                /* the emission enters linearly: d(contribution) / d(radiance) = tp */
                if(adj && adj->gradE)
                    for(int k = 0; k < 3; k++) adj->gradE[4 * (size_t)L->instance + k] += (double)(adj->d[k] * tp[k]);
            }
            break;
        }

        /* GenerateSurface flips the normal towards the ray (PrimitiveDefaultTriangle.hpp:480-486) */
        int backSide = dot3f(gn, dir) > 0.0f;
        if(backSide) { gn[0] = -gn[0]; gn[1] = -gn[1]; gn[2] = -gn[2]; }
        float nrm[3] = { gn[0], gn[1], gn[2] };
        float tng[3], btg[3];
        onb(nrm, tng, btg);
        const float wo[3] = { -dir[0], -dir[1], -dir[2] };
        const float V[3] = { dot3f(wo, tng), dot3f(wo, btg), dot3f(wo, nrm) };
        float alb[4] = { sf->albedo[0], sf->albedo[1], sf->albedo[2], 0.0f };
        if(sf->texels)
        {
            /* GenerateSurface (PrimitiveDefaultTriangle.hpp:472-476):
             * uv = uv0 a + uv1 b + uv2 c, a = hit[0], b = hit[1], c = 1 - a - b */
            const float* q = &sf->uvs[6 * localPrim];
            float a = mh.bary[0], b = mh.bary[1], c = 1.0f - a - b;
            float uv[2];
            for(int k = 0; k < 2; k++) uv[k] = q[k] * a + q[2 + k] * b + q[4 + k] * c;
            if(sf->mipCount > 1u) albedo_lod(sf, tri9, uv, q, pos, nrm, dir, cone_advance(cone, t), alb);
            else orc_tex_read(sf->texels, sf->texW, sf->texH, sf->texFormat, uv, alb);
        }
        orc_pt_surface sfTex;
        sf = unreal_params(sf, localPrim, &mh, tri9, pos, nrm, dir, cone_advance(cone, t), &sfTex);
        if(S) { float c3[3] = { alb[0], alb[1], alb[2] }; orc_spec_convert_albedo(S, c3, waves, alb); }
        if(adj && J->adjTexels && sf->texels == J->adjTexels && sf->matType == ORC_MAT_LAMBERT)
        {
            const float* q = &sf->uvs[6 * localPrim];
            float a = mh.bary[0], b = mh.bary[1], c = 1.0f - a - b;
            float uv[2];
            for(int k = 0; k < 2; k++) uv[k] = q[k] * a + q[2 + k] * b + q[4 + k] * c;
            size_t ti[4]; float tw[4];
            tex_taps(J->adjW, J->adjH, uv, ti, tw);
            for(int k = 0; k < 3; k++)
            {
                float g = (alb[k] > 0.0f) ? adj->d[k] * ((adj->tot[k] - rad[k]) / alb[k]) : 0.0f;
                for(int j = 0; j < 4; j++) adj->grad[4 * ti[j] + k] += (double)(g * tw[j]);
            }
        }
        const int isSpec = specularity(sf, alb, nc) >= SPECULAR_THRESHOLD;

        /* ---- NEE (WorkFunctionNEE); no shadow ray for specular materials ---- */
        if(P->sampleMode != ORC_PT_PURE && nAll > 0 && !isSpec)
        {
            float dXi = urnd(&SC, depth, 3);
            uint32_t li = (uint32_t)(dXi * (float)nAll);
            if(li > nAll - 1u) li = nAll - 1u;
            float lp[3], lightPdf;
            float emis[4] = { 0, 0, 0, 0 };
            if(li == J->nLights)
            {
                /* skysphere: a point sceneDiameter away along the sampled direction */
                float wd[3], spdf;
                env_sample(E, urnd(&SC, depth, 4), urnd(&SC, depth, 5), wd, &spdf);
                for(int k = 0; k < 3; k++) lp[k] = pos[k] + wd[k] * E->sceneDiameter;
                float sd[3] = { pos[0] - lp[0], pos[1] - lp[1], pos[2] - lp[2] };
                normalize3f(sd);
                float toward[3] = { -sd[0], -sd[1], -sd[2] };
                env_emit(E, toward, emis);
                if(S) { float c[3] = { emis[0], emis[1], emis[2] }; orc_spec_convert_radiance(S, c, waves, emis); }
                lightPdf = invN * spdf;
            }
            else
            {
                const orc_pt_light_tri* L = &J->lights[li];
                float ppdf;
                light_tri_sample(L, urnd(&SC, depth, 4), urnd(&SC, depth, 5), pos, lp, &ppdf, emis);
                lightPdf = invN * ppdf;
                if(S && (emis[0] != 0.0f || emis[1] != 0.0f || emis[2] != 0.0f))
                    orc_spec_convert_radiance(S, L->radiance, waves, emis);
            }
            float sdir[3] = { lp[0] - pos[0], lp[1] - pos[1], lp[2] - pos[2] };
            normalize3f(sdir);
            float nd[3] = { -sdir[0], -sdir[1], -sdir[2] };
            float lpn[3];
            orc_nudge(lp, nd, lpn);
            float seg[3] = { lpn[0] - pos[0], lpn[1] - pos[1], lpn[2] - pos[2] };
            float length = sqrtf(dot3f(seg, seg));
            float refl[4] = { 0, 0, 0, 0 }, bpdf;
            const float Ls[3] = { dot3f(sdir, tng), dot3f(sdir, btg), dot3f(sdir, nrm) };
            bxdf_eval(sf, alb, nc, V, Ls, refl, &bpdf);
            float pdf = (P->sampleMode == ORC_PT_NEE_MIS) ? (bpdf + lightPdf) : lightPdf;
            float srad[4] = { 0, 0, 0, 0 };
            for(int k = 0; k < nc; k++) srad[k] = thr[k] * refl[k] * emis[k];
            if(pdf == 0.0f) srad[0] = srad[1] = srad[2] = srad[3] = 0.0f;
            else { float inv = 1.0f / pdf; for(int k = 0; k < nc; k++) srad[k] *= inv; }
            float sorg[3];
            orc_nudge(pos, nrm, sorg);
            if(depth + 2u <= P->maxDepth &&
               visible1(J->scene, sorg, sdir, 1.0e-5f, length * (1.0f - 1.0e-4f)))
            {
                for(int k = 0; k < nc; k++) rad[k] += srad[k];
                if(adj && adj->gradE && li < J->nLights)
                {
                    const orc_pt_light_tri* L = &J->lights[li];
                    for(int k = 0; k < 3; k++)
                        if(L->radiance[k] > 0.0f)
                            adj->gradE[4 * (size_t)L->instance + k] += (double)(adj->d[k] * (srad[k] / L->radiance[k]));
                }
            }
        }

        /* ---- BxDF sample (WorkFunction) ---- */
        float Ll[3], refl[4], bpdf;
        int passed = 0;
        float presample[3] = { pos[0], pos[1], pos[2] };    /* ray origin before the final nudge */
        bxdf_sample(sf, alb, nc, backSide, V, urnd(&SC, depth, 0), urnd(&SC, depth, 1), urnd(&SC, depth, 2),
                    Ll, refl, &bpdf, &passed);
        if(sf->matType == ORC_MAT_REFRACT) orc_nudge(pos, nrm, presample);   /* SampleBxDF nudges along n first */
        float wi[3];
        for(int k = 0; k < 3; k++) wi[k] = tng[k] * Ll[0] + btg[k] * Ll[1] + nrm[k] * Ll[2];
        normalize3f(wi);
        for(int k = 0; k < nc; k++) thr[k] *= refl[k];
        depth += 1u;
        int dead = depth >= P->maxDepth;
        if(!dead && depth >= P->rrStart && !isSpec)
        {
            /* throughput.Sum() * ChannelCountInv (PathTracerRendererShaders.h:250-256) */
            float pr = (nc == 4) ? (thr[0] + thr[1] + thr[2] + thr[3]) * 0.25f
                                 : (thr[0] + thr[1] + thr[2]) * 0.33333333f;
            pr = fminf(fmaxf(pr, 0.1f), 1.0f);
            float xr = urnd(&SC, depth - 1u, 8);
            if(xr >= pr) dead = 1;
            else { float inv = 1.0f / pr; for(int k = 0; k < nc; k++) thr[k] *= inv; }
        }
        type = isSpec ? 2 : 1;
        if(dead) break;
        if(bpdf == 0.0f) { thr[0] = thr[1] = thr[2] = thr[3] = 0.0f; }
        else { float inv = 1.0f / bpdf; for(int k = 0; k < nc; k++) thr[k] *= inv; }
        prevPdf = bpdf;
        float nn[3] = { nrm[0], nrm[1], nrm[2] };
        if(passed) { nn[0] = -nn[0]; nn[1] = -nn[1]; nn[2] = -nn[2]; }
        cone = cone_after_scatter(sf, backSide, cone_advance(cone, t), wo, nrm, wi);
        orc_nudge(presample, nn, org);
        memcpy(dir, wi, 12);
        tmin = 1.0e-4f;
        tmax = 3.402823466e+38f;
    }
    if(S) orc_spec_to_rgb(S, rad, waves, wpdf, outRad);
    else { outRad[0] = rad[0]; outRad[1] = rad[1]; outRad[2] = rad[2]; }
}

static void* pt_worker(void* arg)
{
    pt_job* J = (pt_job*)arg;
    const orc_pt_params* P = J->p;
    for(;;)
    {
        uint32_t y = atomic_fetch_add(&J->nextRow, 1u);
        if(y >= P->height) break;
        for(uint32_t x = 0; x < P->width; x++)
        {
            float* px = &J->image[4ull * (y * P->width + x)];
            for(uint32_t s = 0; s < P->spp; s++)
            {
                float r[3];
                trace_sample(J, x, y, P->sampleStart + s, r);
                px[0] += r[0]; px[1] += r[1]; px[2] += r[2]; px[3] += 1.0f;
            }
        }
    }
    return NULL;
}

static void* pt_adj_worker(void* arg)
{
    pt_job* J = (pt_job*)arg;
    const orc_pt_params* P = J->p;
    int b = atomic_fetch_add(&J->adjNextBuffer, 1);
    double* grad = J->adjGrad + (size_t)b * 4 * J->adjW * J->adjH;
    double* gradE = J->adjGradE ? J->adjGradE + (size_t)b * 4 * J->adjInstances : NULL;
    const float invSpp = 1.0f / (float)P->spp;
    for(;;)
    {
        uint32_t y = atomic_fetch_add(&J->nextRow, 1u);
        if(y >= P->height) break;
        for(uint32_t x = 0; x < P->width; x++)
        {
            const float* d = &J->adjDelta[4ull * (y * P->width + x)];
            for(uint32_t s = 0; s < P->spp; s++)
            {
                adj_ctx A;
                trace_sample(J, x, y, P->sampleStart + s, A.tot);
                for(int k = 0; k < 3; k++) A.d[k] = d[k] * invSpp;
                A.grad = grad;
                A.gradE = gradE;
                float r[3];
                trace_sample_adj(J, x, y, P->sampleStart + s, r, &A);
            }
        }
    }
    return NULL;
}

/* ZSobol sampler state of a job (seeds of the whole image). */
static int job_sampler(pt_job* J, const orc_pt_params* p)
{
    J->zsSeeds = NULL;
    if(p->sampler < 1u || p->sampler > 3u) return 0;
    J->zsSeeds = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)p->width * p->height);
    if(!J->zsSeeds) return -2;
    orc_zs_seeds(p->width, p->height, (uint64_t)p->seed, J->zsSeeds);
    J->zsResBits = orc_zs_res_max_bits(p->width, p->height);
    return 0;
}

int orc_pt_adjoint(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                   const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                   const void* texels, uint32_t texW, uint32_t texH, const float* delta,
                   double* grad, double* gradEmission, uint32_t nInstances, int nthreads)
{
    if(!s || !p || !surfaces || !delta || (texels && !grad) || (!texels && !gradEmission)) return -1;
    if(nthreads < 1) nthreads = 1;
    if(nthreads > 64) nthreads = 64;
    if(!texels) texW = texH = 0;
    const size_t n = 4ull * texW * texH, ne = gradEmission ? 4ull * nInstances : 0;
    double* bufs = (double*)calloc((size_t)nthreads * (n + ne) + 1, sizeof(double));
    if(!bufs) return -2;
    double* bufsE = bufs + (size_t)nthreads * n;
    pt_job J;
    memset(&J, 0, sizeof(J));
    J.scene = s; J.p = p; J.surfaces = surfaces; J.lights = lights; J.nLights = nLights;
    J.env = env;
    J.adjTexels = texels; J.adjW = texW; J.adjH = texH; J.adjDelta = delta; J.adjGrad = bufs;
    J.adjGradE = gradEmission ? bufsE : NULL;
    J.adjInstances = nInstances;
    J.adjWorkers = nthreads;
    if(job_sampler(&J, p) != 0) { free(bufs); return -2; }
    atomic_init(&J.nextRow, 0u);
    atomic_init(&J.adjNextBuffer, 0);
    pthread_t th[64];
    int started = 0;
    for(int t = 1; t < nthreads; t++)
        if(pthread_create(&th[started], NULL, pt_adj_worker, &J) == 0) started++;
    pt_adj_worker(&J);
    for(int t = 0; t < started; t++) pthread_join(th[t], NULL);
    for(int t = 0; t <= started; t++)
    {
        for(size_t i = 0; i < n; i++) grad[i] += bufs[(size_t)t * n + i];
        for(size_t i = 0; i < ne; i++) gradEmission[i] += bufsE[(size_t)t * ne + i];
    }
    free(bufs);
    free(J.zsSeeds);
    return 0;
}

int orc_pt_render(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                  const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                  const orc_spectral* spectral, float* image, int nthreads)
{
    if(!s || !p || !surfaces || !image) return -1;
    pt_job J;
    memset(&J, 0, sizeof(J));
    J.scene = s; J.p = p; J.surfaces = surfaces; J.lights = lights; J.nLights = nLights;
    J.env = env;
    J.spec = spectral;
    J.image = image;
    if(job_sampler(&J, p) != 0) return -2;
    atomic_init(&J.nextRow, 0u);
    if(nthreads < 1) nthreads = 1;
    if(nthreads > 256) nthreads = 256;
    pthread_t th[256];
    int started = 0;
    for(int t = 1; t < nthreads; t++)
        if(pthread_create(&th[started], NULL, pt_worker, &J) == 0) started++;
    pt_worker(&J);
    for(int t = 0; t < started; t++) pthread_join(th[t], NULL);
    free(J.zsSeeds);
    return 0;
}

/* CameraPinhole constructor (Source/Tracer/CamerasDefault.hpp:6-30): image
 * plane at distance near, frame from gaze point and up. */
static void cross_fma(const float a[3], const float b[3], float o[3])
{
    float x = fmaf(a[1], b[2], -a[2] * b[1]);
    float y = fmaf(a[2], b[0], -a[0] * b[2]);
    float z = fmaf(a[0], b[1], -a[1] * b[0]);
    o[0] = x; o[1] = y; o[2] = z;
}
static void normalize_fma(float v[3])
{
    float l = sqrtf(fmaf(v[2], v[2], fmaf(v[1], v[1], fmaf(v[0], v[0], 0.0f))));
    float inv = 1.0f / l;
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}
void orc_pt_camera_frame(const float pos[3], const float gaze[3], const float up[3],
                         float fovX, float fovY, float nearT, float farT, orc_pt_params* p)
{
    float wh = tanf(fovX * 0.5f) * nearT;
    float hh = tanf(fovY * 0.5f) * nearT;
    float g[3] = { gaze[0] - pos[0], gaze[1] - pos[1], gaze[2] - pos[2] };
    float r[3], u[3];
    cross_fma(g, up, r); normalize_fma(r);
    cross_fma(r, g, u); normalize_fma(u);
    cross_fma(u, r, g); normalize_fma(g);
    for(int k = 0; k < 3; k++)
    {
        p->camPos[k] = pos[k];
        p->camRight[k] = r[k];
        p->camUp[k] = u[k];
        p->camBottomLeft[k] = ((pos[k] - r[k] * wh) - u[k] * hh) + g[k] * nearT;
    }
    p->planeSize[0] = wh * 2.0f;
    p->planeSize[1] = hh * 2.0f;
    p->nearT = nearT;
    p->farT = farT;
    /* CameraPinhole's ray cone (CamerasDefault.hpp:80-86) */
    p->coneAperture = 2.0f * tanf(fovY * 0.5f) / (float)p->height;
}

/* World-space light triangle from instance-space vertices (ApplyP with the
 * 4-term fma Dot, TransformsDefault.hpp:19-23; Normal / Area,
 * ShapeFunctions.h:60-73). */
void orc_pt_make_light(const float m[12], const float* v9, const float radiance[3], int twoSided,
                       orc_pt_light_tri* out)
{
    float w[3][3];
    for(int c = 0; c < 3; c++)
        for(int r = 0; r < 3; r++)
        {
            float acc = 0.0f;
            acc = fmaf(m[4 * r + 0], v9[3 * c + 0], acc);
            acc = fmaf(m[4 * r + 1], v9[3 * c + 1], acc);
            acc = fmaf(m[4 * r + 2], v9[3 * c + 2], acc);
            acc = fmaf(m[4 * r + 3], 1.0f, acc);
            w[c][r] = acc;
        }
    memcpy(out->p0, w[0], 12); memcpy(out->p1, w[1], 12); memcpy(out->p2, w[2], 12);
    float e0[3] = { w[1][0] - w[0][0], w[1][1] - w[0][1], w[1][2] - w[0][2] };
    float e1[3] = { w[2][0] - w[0][0], w[2][1] - w[0][1], w[2][2] - w[0][2] };
    float c[3];
    c[0] = fmaf(e0[1], e1[2], -e0[2] * e1[1]);
    c[1] = fmaf(e0[2], e1[0], -e0[0] * e1[2]);
    c[2] = fmaf(e0[0], e1[1], -e0[1] * e1[0]);
    float len = sqrtf(fmaf(c[2], c[2], fmaf(c[1], c[1], fmaf(c[0], c[0], 0.0f))));
    out->area = len * 0.5f;
    float inv = 1.0f / len;
    out->n[0] = c[0] * inv; out->n[1] = c[1] * inv; out->n[2] = c[2] * inv;
    memcpy(out->radiance, radiance, 12);
    out->twoSided = twoSided;
    out->instance = 0u;
}

/* ------------------------------------------------------------------------ */
/* Per-function entry points: each runs the helper the path loop above uses */
/* on one record, so tests can hold it against the same function of MRay's   */
/* compiled code (oracle/ref_pt_driver.cpp).  Vectors are in the tangent     */
/* frame; random numbers are the dispenser's uint32 values.                  */
/* ------------------------------------------------------------------------ */

/* RNGFunctions::ToFloat01 (Source/Tracer/Random.h:102-125) */
static inline float to_float01(uint32_t v)
{
    float f = (float)v * 0x1p-32f;
    const float prev1 = 0x1.fffffep-1f;
    return f < prev1 ? f : prev1;
}

void orc_fx_material(int kind, const orc_fx_mat_in* in, orc_fx_mat_out* out, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const orc_fx_mat_in* q = &in[i];
        orc_fx_mat_out* o = &out[i];
        memset(o, 0, sizeof(*o));
        orc_pt_surface sf;
        memset(&sf, 0, sizeof(sf));
        sf.matType = kind;
        sf.roughness = q->rough; sf.metallic = q->metal; sf.specular = q->spec;
        sf.iorFront = q->iorF; sf.iorBack = q->iorB;
        float alb[4] = { q->albedo[0], q->albedo[1], q->albedo[2], 0.0f };
        float L[3], refl[4], pdf;
        int passed;
        bxdf_sample(&sf, alb, 3, (int)q->backSide, q->wo, to_float01(q->xi[0]), to_float01(q->xi[1]),
                    to_float01(q->xi[2]), L, refl, &pdf, &passed);
        memcpy(o->wi, L, 12);
        memcpy(o->wiPos, q->pos, 12);
        if(kind == ORC_MAT_REFRACT)
        {
            const float nz[3] = { 0.0f, 0.0f, 1.0f };
            orc_nudge(q->pos, nz, o->wiPos);
        }
        o->pdf = pdf;
        memcpy(o->refl, refl, 16);
        o->passed = (uint32_t)passed;
        if(kind == ORC_MAT_LAMBERT || kind == ORC_MAT_UNREAL)
            bxdf_eval(&sf, alb, 3, q->wo, q->wiEval, o->evalRefl, &o->evalPdf);
        o->specularity = specularity(&sf, alb, 3);
    }
}

void orc_fx_fresnel_dielectric(const float* in3, float* out, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++) out[i] = fresnel_dielectric(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2]);
}

void orc_fx_vndf_sample(const float* in6, float* out4, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        vndf_sample(q, q[3], q[4], q[5], out4 + 4 * i);
        out4[4 * i + 3] = vndf_pdf(q, out4 + 4 * i, q[3]);
    }
}

void orc_fx_russian_roulette(const float* in6, float* out5, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        float* o = out5 + 5 * i;
        float pr = fminf(fmaxf(q[4], 0.1f), 1.0f);
        o[0] = (q[5] >= pr) ? 0.0f : 1.0f;
        float inv = 1.0f / pr;
        for(int k = 0; k < 4; k++) o[1 + k] = o[0] != 0.0f ? q[k] * inv : 0.0f;
    }
}

void orc_fx_tri_light(const orc_fx_light_in* in, orc_fx_light_out* out, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const orc_fx_light_in* q = &in[i];
        orc_fx_light_out* o = &out[i];
        memset(o, 0, sizeof(*o));
        orc_pt_light_tri L;
        orc_pt_make_light(q->m, q->v9, q->radiance, (int)q->twoSided, &L);
        float emis[4] = { 0, 0, 0, 0 };
        light_tri_sample(&L, to_float01(q->xi[0]), to_float01(q->xi[1]), q->distant, o->point, &o->samplePdf,
                         emis);
        memcpy(o->emitPoint, emis, 12);
        o->pdfSolidAngle = light_tri_pdf(&L, q->hit[0], q->hit[1], q->distant, q->dir);
        if(light_tri_emits(&L, q->wo)) memcpy(o->emitHit, q->radiance, 12);
        o->area = L.area;
    }
}

void orc_fx_camera(const float* cam13, const uint32_t res[2], const uint32_t* pix, const float* off4, float* out6,
                   uint32_t n)
{
    orc_pt_params p;
    memset(&p, 0, sizeof(p));
    orc_pt_camera_frame(cam13, cam13 + 3, cam13 + 6, cam13[9], cam13[10], cam13[11], cam13[12], &p);
    p.width = res[0]; p.height = res[1];
    for(uint32_t i = 0; i < n; i++)
        camera_ray(&p, pix[2 * i], pix[2 * i + 1], off4[4 * i], off4[4 * i + 1], out6 + 6 * i, out6 + 6 * i + 3);
}

/* SphericalCoordConverter (LightsDefault.hpp:174-215) as the skysphere light
 * uses it: in dir[3], uv[2], pdf -> DirToUV(dir), UVToDir(uv),
 * ToSolidAnglePdf(pdf, dir), ToSolidAnglePdf(pdf, uv). */
void orc_fx_spherical_coords(const float* in6, float* out7, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        float* o = out7 + 7 * i;
        orc_env_dir_to_uv(q, o);
        orc_env_uv_to_dir(q + 3, o + 2);
        float cl = (q[1] < -1.0f) ? -1.0f : ((q[1] > 1.0f) ? 1.0f : q[1]);
        o[5] = env_sa_pdf_sin(q[5], sinf(acosf(cl)));
        o[6] = env_sa_pdf_sin(q[5], sinf((1.0f - q[4]) * PI_F));
    }
}

/* GaussianFilter (Filters.h:195-233): in radius, xi[2] -> offset[2], pdf,
 * Evaluate(offset), Evaluate / pdf. */
void orc_fx_gaussian_filter(const float* in3, float* out5, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in3 + 3 * i;
        float* o = out5 + 5 * i;
        filter_sample(q[0], q[1], q[2], &o[0], &o[1]);
        float sigma = q[0] * 0.285714f;
        o[2] = gaussian(o[0], sigma) * gaussian(o[1], sigma);
        o[3] = gaussian(o[0], sigma) * gaussian(o[1], sigma);
        o[4] = o[3] / o[2];
    }
}

/* SingleSampleSpectrumWavelength, hyperbolic mode (SpectrumContext.cu:9-130):
 * uint32 numbers in, wavelengths and pdfs out. */
/* The ray-cone steps on the tangent surface (geometric normal +z), in the
 * record layout of ref_cone (oracle/ref_pt_driver.cpp). */
void orc_fx_cone(const float* in20, float* out12, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in20 + 20 * i;
        float* o = out12 + 12 * i;
        const cone_t c = { q[0], q[1] };
        const cone_t adv = cone_advance(c, q[2]);
        o[0] = adv.aperture; o[1] = adv.width;
        cone_project(adv, q + 3, q + 6, o + 2, o + 5);
        const float nz[3] = { 0.0f, 0.0f, 1.0f };
        float fromEta = q[13], toEta = q[14];
        if(q[15] != 0.0f) { const float t = fromEta; fromEta = toEta; toEta = t; }
        cone_t back = adv, r;
        if(refract_cone(adv, q[9], q + 10, nz, fromEta, toEta, &r)) back = r;
        o[8] = back.aperture; o[9] = back.width;
        const float betaN = q[9];
        if(dot3f(q + 16, nz) > 0.0f) { o[10] = adv.aperture + 2.0f * betaN; o[11] = adv.width; }
        else { o[10] = back.aperture - betaN; o[11] = back.width; }
    }
}

/* Graphics::ConvertPixelIndices, as the mip generation applies it */
void orc_fx_pixel_indices(const float* in6, float* out2, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in6 + 6 * i;
        for(int k = 0; k < 2; k++)
        {
            const float ratio = q[2 + k] / q[4 + k];
            const float r = (q[k] + 0.5f) * ratio - 0.5f;
            out2[2 * i + k] = fminf(fmaxf(0.0f, r), q[2 + k] - 1.0f);
        }
    }
}

void orc_fx_sample_waves(const uint32_t* xi, float* waves4, float* pdf4, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++) orc_spec_sample_waves(to_float01(xi[i]), waves4 + 4 * i, pdf4 + 4 * i);
}

/* ======================================================================== */
/* Guided path tracing (MRay's GuidedPTRenderer), as a wavefront: every     */
/* bounce runs its stages over all path slots in slot order, the schedule   */
/* the GPU renderer's kernels reproduce (closest hit, backprop, chain       */
/* writes, shade, shadow rays, irradiance records applied per cell in       */
/* (path, NEE, light) then slot order).  The stages restate                 */
/*   KCBackpropagateHashGridPath      Source/TracerDLL/GuidedPTRenderer.cu:164-311 */
/*   KCWriteMarkovChains              GuidedPTRenderer.cu:313-344          */
/*   WorkFunction / LightWorkFunction GuidedPTRendererShaders.h:588-931    */
/*   GaussLobeMixtureT                GuidedPTRendererShaders.h:381-450    */
/*   KCAccumulateShadowRaysGPT, KCBackpropagateIrradNEE / Light            */
/*                                    GuidedPTRenderer.cu:13-33, 346-430   */
/* with the building blocks of guide_oracle.c.                             */
/* ======================================================================== */
#include "guide_oracle.h"

struct orc_guide_state
{
    orc_guide_grid g;
    float*    mcA;          /* 4 per table slot: target xyz, cosine */
    float*    mcW;
    uint32_t* mcN;
    float*    irr;
    uint32_t* irrN;
    uint32_t* lock;
    float     lobeProb;
    int       fixZeroWeight;   /* 1: no mixture sample where the chosen lobe has weight 0 */
    int       camSet;
    uint32_t* bk;           /* backup PCG32 state per path slot */
    uint32_t  bkSlots, bkSeed, bkW, bkH;
    int       bkValid;
};

static uint32_t next_pow2_u32(uint32_t v)
{
    uint32_t p = 1;
    while(p < v) p <<= 1;
    return p;
}

orc_guide_state* orc_guide_new(const orc_scene* s, uint32_t entryLimit, uint32_t posBits, uint32_t normalBits,
                               uint32_t maxLevelOffset, float coneDeg, float lobeProb, int fixZeroWeight)
{
    orc_guide_state* G = (orc_guide_state*)calloc(1, sizeof(orc_guide_state));
    if(!G) return NULL;
    const float mult = 1.0f / 0.6f;
    const uint32_t T = next_pow2_u32((uint32_t)((float)entryLimit * mult));
    float box[6], cam[3] = { 0, 0, 0 };
    orc_scene_aabb(s, box);
    orc_guide_view(&G->g, box, cam, posBits, normalBits, maxLevelOffset, coneDeg, T);
    G->g.codes = (uint64_t*)malloc(sizeof(uint64_t) * T);
    G->mcA = (float*)malloc(sizeof(float) * 4 * T);
    G->mcW = (float*)malloc(sizeof(float) * T);
    G->mcN = (uint32_t*)malloc(sizeof(uint32_t) * T);
    G->irr = (float*)malloc(sizeof(float) * T);
    G->irrN = (uint32_t*)malloc(sizeof(uint32_t) * T);
    G->lock = (uint32_t*)malloc(sizeof(uint32_t) * T);
    G->lobeProb = lobeProb;
    G->fixZeroWeight = fixZeroWeight;
    if(!G->g.codes || !G->mcA || !G->mcW || !G->mcN || !G->irr || !G->irrN || !G->lock)
    {
        orc_guide_delete(G);
        return NULL;
    }
    orc_guide_clear(G);
    return G;
}

void orc_guide_delete(orc_guide_state* G)
{
    if(!G) return;
    free(G->g.codes); free(G->mcA); free(G->mcW); free(G->mcN); free(G->irr); free(G->irrN); free(G->lock);
    free(G->bk);
    free(G);
}

void orc_guide_clear(orc_guide_state* G)
{
    const uint32_t T = G->g.tableSize;
    for(uint32_t i = 0; i < T; i++) G->g.codes[i] = ORC_GUIDE_EMPTY;
    G->g.counter = 0;
    memset(G->mcA, 0, sizeof(float) * 4 * T);
    memset(G->mcW, 0, sizeof(float) * T);
    memset(G->mcN, 0, sizeof(uint32_t) * T);
    memset(G->irr, 0, sizeof(float) * T);
    memset(G->irrN, 0, sizeof(uint32_t) * T);
    G->camSet = 0;
    G->bkValid = 0;
}

uint32_t orc_guide_table_size(const orc_guide_state* G) { return G->g.tableSize; }
uint32_t orc_guide_used(const orc_guide_state* G) { return G->g.counter; }

void orc_guide_snapshot(const orc_guide_state* G, uint64_t* codes, float* chain6, float* irr2)
{
    for(uint32_t i = 0; i < G->g.tableSize; i++)
    {
        if(codes) codes[i] = G->g.codes[i];
        if(chain6)
        {
            float* o = chain6 + 6 * (size_t)i;
            for(int k = 0; k < 4; k++) o[k] = G->mcA[4 * (size_t)i + k];
            o[4] = G->mcW[i];
            o[5] = (float)G->mcN[i];
        }
        if(irr2) { irr2[2 * (size_t)i] = G->irr[i]; irr2[2 * (size_t)i + 1] = (float)G->irrN[i]; }
    }
}

typedef struct
{
    smp_ctx  sc;
    float    org[3], dir[3], tmin, tmax;
    float    thr[4], rad[4], waves[4], wpdf[4];
    float    prevPdf;
    cone_t   cone;                 /* ray cone of the current ray */
    uint32_t depth, type;          /* type 0 camera, 1 path, 2 specular */
    int      alive;
    int      hit;                  /* closest hit of this bounce */
    uint32_t inst;
    orc_hit_keys hk;
    orc_meta_hit mh;
    /* guided state (GuidedPTRDetail::RayState) */
    uint32_t lifted;
    float    prevRefl, scoreSum, prevNormal[2], shadowOut;
    float    tmpA[4], tmpW;
    uint32_t tmpN;
    /* shadow ray */
    int      shadow;
    float    sorg[3], sdir[3], stmax, srad[4];
} g_slot;

typedef struct { uint32_t key, pos; } g_rec;

static int g_rec_cmp(const void* a, const void* b)
{
    const g_rec* x = (const g_rec*)a;
    const g_rec* y = (const g_rec*)b;
    if(x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);
}

static float g_avg(const float* c, int nc)
{
    return (nc == 4) ? (c[0] + c[1] + c[2] + c[3]) * 0.25f : (c[0] + c[1] + c[2]) * 0.33333333f;
}

static void g_put(uint32_t* recKey, float* recVal, uint32_t pos, uint32_t cell, uint32_t light, float v)
{
    recKey[pos] = (cell << 1) | light;
    recVal[pos] = isfinite(v) ? v : 0.0f;
}

/* GaussLobeMixtureT::Pdf */
static float g_mix_pdf(const orc_lobe* lobes, const float* w, float sumW, const float d[3])
{
    if(sumW == 0.0f) return 0.0f;
    float pdf = 0.0f;
    for(uint32_t j = 0; j < ORC_GUIDE_LOBES; j++)
        if(w[j] != 0.0f) pdf = pdf + w[j] * orc_lobe_pdf(&lobes[j], d);
    return pdf / sumW;
}

static void g_albedo(const orc_pt_surface* sf, uint32_t localPrim, const orc_meta_hit* mh, const orc_spectral* S,
                     const float waves[4], const float* tri9, const float pos[3], const float nrm[3],
                     const float dir[3], cone_t cone, float alb[4])
{
    alb[0] = sf->albedo[0]; alb[1] = sf->albedo[1]; alb[2] = sf->albedo[2]; alb[3] = 0.0f;
    if(sf->texels)
    {
        const float* q = &sf->uvs[6 * localPrim];
        float a = mh->bary[0], b = mh->bary[1], c = 1.0f - a - b;
        float uv[2];
        for(int k = 0; k < 2; k++) uv[k] = q[k] * a + q[2 + k] * b + q[4 + k] * c;
        if(sf->mipCount > 1u) albedo_lod(sf, tri9, uv, q, pos, nrm, dir, cone, alb);
        else orc_tex_read(sf->texels, sf->texW, sf->texH, sf->texFormat, uv, alb);
    }
    if(S) { float c3[3] = { alb[0], alb[1], alb[2] }; orc_spec_convert_albedo(S, c3, waves, alb); }
}

/* Light work of a miss (inst == ~0: the boundary light) or of a light
 * surface hit: emission with MIS for path rays, and the light-cache radiance
 * of the previous vertex. */
static void g_light_work(const orc_pt_params* P, const orc_pt_surface* surfaces, const orc_pt_light_tri* lights,
                         const orc_pt_env* E, const orc_spectral* S, float invN, g_slot* q, uint32_t i,
                         uint32_t slots, uint32_t* recKey, float* recVal)
{
    const int nc = S ? 4 : 3;
    float tp[4] = { q->thr[0], q->thr[1], q->thr[2], q->thr[3] };
    float lcRefl = q->prevRefl;
    float lpdf = 0.0f;
    float em[4] = { 0, 0, 0, 0 };
    if(q->hit)
    {
        const orc_pt_surface* sf = &surfaces[q->inst];
        const orc_pt_light_tri* L = &lights[sf->lightBase + (q->hk.primKey - sf->primKeyBase)];
        if(q->type == 1u) lpdf = light_tri_pdf(L, q->mh.bary[0], q->mh.bary[1], q->org, q->dir) * invN;
        const float wo[3] = { -q->dir[0], -q->dir[1], -q->dir[2] };
        if(light_tri_emits(L, wo))
        {
            em[0] = L->radiance[0]; em[1] = L->radiance[1]; em[2] = L->radiance[2];
            if(S) orc_spec_convert_radiance(S, L->radiance, q->waves, em);
        }
    }
    else if(E)
    {
        if(q->type == 1u) lpdf = env_pdf(E, q->dir) * invN;
        env_emit(E, q->dir, em);
        if(S) { float c[3] = { em[0], em[1], em[2] }; orc_spec_convert_radiance(S, c, q->waves, em); }
    }
    if(q->type == 1u)
    {
        const float p0 = q->prevPdf;
        const float misPdf = p0 + lpdf;
        for(int k = 0; k < nc; k++) tp[k] *= p0;
        if(misPdf == 0.0f) tp[0] = tp[1] = tp[2] = tp[3] = 0.0f;
        else { float inv = 1.0f / misPdf; for(int k = 0; k < nc; k++) tp[k] *= inv; }
        lcRefl = lcRefl * p0;
        lcRefl = (misPdf == 0.0f) ? 0.0f : lcRefl / misPdf;
    }
    float lcRad = 0.0f;
    if(q->depth + 1u <= P->maxDepth)
    {
        for(int k = 0; k < nc; k++) q->rad[k] += em[k] * tp[k];
        lcRad = lcRefl * g_avg(em, nc);
    }
    if(q->lifted != ORC_GUIDE_INVALID) g_put(recKey, recVal, slots + i, q->lifted, 1u, lcRad);
    q->alive = 0;
}

/* WorkFunction of the guided renderer for a surface hit. */
static void g_surface_work(const orc_scene* scene, const orc_pt_params* P, const orc_pt_surface* surfaces,
                           const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* E,
                           const orc_spectral* S, orc_guide_state* G, float invN, uint32_t nAll, g_slot* q,
                           uint32_t i)
{
    const int nc = S ? 4 : 3;
    const orc_pt_surface* sf = &surfaces[q->inst];
    const uint32_t localPrim = q->hk.primKey - sf->primKeyBase;
    const float* tri9 = &sf->triangles[9 * localPrim];
    const float bu = q->mh.bary[1];
    const float bv = 1.0f - q->mh.bary[0] - q->mh.bary[1];
    float pos[3], gn[3];
    surface_of(sf, tri9, bu, bv, pos, gn);
    const int backSide = dot3f(gn, q->dir) > 0.0f;
    if(backSide) { gn[0] = -gn[0]; gn[1] = -gn[1]; gn[2] = -gn[2]; }
    const float nrm[3] = { gn[0], gn[1], gn[2] };
    float tng[3], btg[3];
    onb(nrm, tng, btg);
    const float wo[3] = { -q->dir[0], -q->dir[1], -q->dir[2] };
    const float V[3] = { dot3f(wo, tng), dot3f(wo, btg), dot3f(wo, nrm) };
    float alb[4];
    const cone_t cone = cone_advance(q->cone, q->tmax);
    g_albedo(sf, localPrim, &q->mh, S, q->waves, tri9, pos, nrm, q->dir, cone, alb);
    orc_pt_surface sfTex;
    sf = unreal_params(sf, localPrim, &q->mh, tri9, pos, nrm, q->dir, cone, &sfTex);
    const float specv = specularity(sf, alb, nc);
    const int isSpec = specv >= SPECULAR_THRESHOLD;
    float woW[3] = { wo[0], wo[1], wo[2] };
    normalize3f(woW);
    const uint32_t d = q->depth;

    /* GaussLobeMixtureT::LoadStochastic */
    orc_lobe lobes[ORC_GUIDE_LOBES];
    float wts[ORC_GUIDE_LOBES];
    float sumW = 0.0f, selW = 0.0f;
    int selected = 0;
    uint32_t sel = 0, liftedMC = ORC_GUIDE_INVALID;
    uint32_t* rng = &G->bk[i];
    float codeN[3] = { woW[0], woW[1], woW[2] };
    normalize3f(codeN);
    for(uint32_t j = 0; j < ORC_GUIDE_LOBES; j++)
    {
        const uint64_t code = orc_guide_gen_code_stochastic(&G->g, pos, codeN, rng);
        int ins;
        const uint32_t slot = orc_guide_try_insert(&G->g, code, &ins);
        if(slot == ORC_GUIDE_INVALID)
        {
            memset(&lobes[j], 0, sizeof(orc_lobe));
            wts[j] = 0.0f;
            continue;
        }
        orc_mc_state s;
        for(int k = 0; k < 3; k++) s.target[k] = G->mcA[4 * (size_t)slot + k];
        s.cosine = G->mcA[4 * (size_t)slot + 3];
        s.weight = G->mcW[slot];
        lobes[j] = orc_mc_to_lobe(&s, G->mcN[slot], pos);
        wts[j] = s.weight;
        sumW = sumW + wts[j];
        const float ratio = (sumW != 0.0f) ? wts[j] / sumW : 1.0f;
        if(orc_guide_next_float(rng) < ratio) { sel = j; selW = wts[j]; selected = 1; liftedMC = slot; }
    }
    float coN[2];
    orc_dir_to_conc_octa(woW, coN);

    /* mixture or material sample, balance-heuristic pdf */
    float mw0 = 0.0f;
    if(!isSpec)
    {
        float t = 1.0f - specv;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        mw0 = 0.0f * (1.0f - t) + G->lobeProb * t;           /* Math::Lerp(0, p, t) */
        if(G->fixZeroWeight && (!selected || selW == 0.0f)) mw0 = 0.0f;
    }
    const float mw1 = 1.0f - mw0;
    float refl[4] = { 0, 0, 0, 0 }, pdf0, pdf1, wdir[3], orgOut[3] = { pos[0], pos[1], pos[2] };
    int passed = 0, lobeSampled = 0;
    if(urnd(&q->sc, d, 10) < mw0)
    {
        float v[3] = { 0.0f, 1.0f, 0.0f }, mpdf = 0.0f;
        if(selected && selW != 0.0f)
        {
            orc_lobe_sample(&lobes[sel], urnd(&q->sc, d, 0), urnd(&q->sc, d, 1), v);
            mpdf = g_mix_pdf(lobes, wts, sumW, v);
        }
        memcpy(wdir, v, 12);
        float vn[3] = { v[0], v[1], v[2] };
        normalize3f(vn);
        const float Ls[3] = { dot3f(vn, tng), dot3f(vn, btg), dot3f(vn, nrm) };
        float bpdf;
        bxdf_eval(sf, alb, nc, V, Ls, refl, &bpdf);
        pdf0 = mpdf;
        pdf1 = bpdf;
        lobeSampled = 1;
    }
    else
    {
        float Ll[3], bpdf;
        bxdf_sample(sf, alb, nc, backSide, V, urnd(&q->sc, d, 0), urnd(&q->sc, d, 1), urnd(&q->sc, d, 2),
                    Ll, refl, &bpdf, &passed);
        if(sf->matType == ORC_MAT_REFRACT) orc_nudge(pos, nrm, orgOut);
        for(int k = 0; k < 3; k++) wdir[k] = tng[k] * Ll[0] + btg[k] * Ll[1] + nrm[k] * Ll[2];
        normalize3f(wdir);
        pdf0 = g_mix_pdf(lobes, wts, sumW, wdir);
        pdf1 = bpdf;
    }
    const float pdfPath = pdf0 * mw0 + pdf1 * mw1;

    /* Russian roulette on the throughput before this vertex */
    q->depth += 1u;
    int dead = q->depth >= P->maxDepth;
    if(!dead && q->depth >= P->rrStart && !isSpec)
    {
        float pr = g_avg(q->thr, nc);
        pr = fminf(fmaxf(pr, 0.1f), 1.0f);
        if(urnd(&q->sc, d, 8) >= pr) dead = 1;
        else { float inv = 1.0f / pr; for(int k = 0; k < nc; k++) q->thr[k] *= inv; }
    }
    const float avgRefl = g_avg(refl, nc);
    const float thr[4] = { q->thr[0], q->thr[1], q->thr[2], q->thr[3] };   /* NEE's throughput */
    q->alive = 0;
    q->shadow = 0;
    if(!dead)
    {
        float pthr[4] = { 0, 0, 0, 0 };
        for(int k = 0; k < nc; k++) pthr[k] = thr[k] * refl[k];
        if(pdfPath == 0.0f) pthr[0] = pthr[1] = pthr[2] = pthr[3] = 0.0f;
        else { float inv = 1.0f / pdfPath; for(int k = 0; k < nc; k++) pthr[k] *= inv; }
        float nn[3] = { nrm[0], nrm[1], nrm[2] };
        if(passed) { nn[0] = -nn[0]; nn[1] = -nn[1]; nn[2] = -nn[2]; }
        q->cone = cone_after_scatter(sf, backSide, cone, wo, nrm, wdir);
        orc_nudge(orgOut, nn, q->org);
        memcpy(q->dir, wdir, 12);
        memcpy(q->thr, pthr, 16);
        q->tmin = 1.0e-4f;
        q->tmax = 3.402823466e+38f;
        q->prevPdf = pdfPath;
        q->type = isSpec ? 2u : 1u;
        q->prevRefl = avgRefl / fmaxf(pdfPath, 10.0f);
        q->scoreSum = lobeSampled ? sumW : INFINITY;
        q->lifted = liftedMC;
        q->prevNormal[0] = coN[0]; q->prevNormal[1] = coN[1];
        q->alive = 1;
    }
    /* NEE with the mixture / material MIS, then with the light */
    if(!dead && !isSpec && nAll > 0)
    {
        float dXi = urnd(&q->sc, d, 3);
        uint32_t li = (uint32_t)(dXi * (float)nAll);
        if(li > nAll - 1u) li = nAll - 1u;
        float lp[3], lightPdf;
        float emis[4] = { 0, 0, 0, 0 };
        if(li == nLights)
        {
            float wd[3], spdf;
            env_sample(E, urnd(&q->sc, d, 4), urnd(&q->sc, d, 5), wd, &spdf);
            for(int k = 0; k < 3; k++) lp[k] = pos[k] + wd[k] * E->sceneDiameter;
            float sd[3] = { pos[0] - lp[0], pos[1] - lp[1], pos[2] - lp[2] };
            normalize3f(sd);
            float toward[3] = { -sd[0], -sd[1], -sd[2] };
            env_emit(E, toward, emis);
            if(S) { float c[3] = { emis[0], emis[1], emis[2] }; orc_spec_convert_radiance(S, c, q->waves, emis); }
            lightPdf = invN * spdf;
        }
        else
        {
            const orc_pt_light_tri* L = &lights[li];
            float ppdf;
            light_tri_sample(L, urnd(&q->sc, d, 4), urnd(&q->sc, d, 5), pos, lp, &ppdf, emis);
            lightPdf = invN * ppdf;
            if(S && (emis[0] != 0.0f || emis[1] != 0.0f || emis[2] != 0.0f))
                orc_spec_convert_radiance(S, L->radiance, q->waves, emis);
        }
        float sdir[3] = { lp[0] - pos[0], lp[1] - pos[1], lp[2] - pos[2] };
        normalize3f(sdir);
        float nd[3] = { -sdir[0], -sdir[1], -sdir[2] };
        float lpn[3];
        orc_nudge(lp, nd, lpn);
        float seg[3] = { lpn[0] - pos[0], lpn[1] - pos[1], lpn[2] - pos[2] };
        const float length = sqrtf(dot3f(seg, seg));
        const float Ls[3] = { dot3f(sdir, tng), dot3f(sdir, btg), dot3f(sdir, nrm) };
        float srefl[4] = { 0, 0, 0, 0 }, bpdf;
        bxdf_eval(sf, alb, nc, V, Ls, srefl, &bpdf);
        float pdfS = g_mix_pdf(lobes, wts, sumW, sdir) * mw0 + bpdf * mw1;
        pdfS = pdfS + lightPdf;
        float srad[4] = { 0, 0, 0, 0 };
        if(pdfS != 0.0f)
        {
            float inv = 1.0f / pdfS;
            for(int k = 0; k < nc; k++) srad[k] = thr[k] * srefl[k] * emis[k] * inv;
        }
        orc_nudge(pos, nrm, q->sorg);
        memcpy(q->sdir, sdir, 12);
        q->stmax = length * (1.0f - 1.0e-4f);
        memcpy(q->srad, srad, 16);
        const float se = g_avg(srefl, nc) * g_avg(emis, nc);
        q->shadowOut = se / fmaxf(pdfS, 10.0f);
        q->shadow = 1;
    }
    (void)scene;
}

int orc_pt_render_guided(const orc_scene* s, const orc_pt_params* p, const orc_pt_surface* surfaces,
                         const orc_pt_light_tri* lights, uint32_t nLights, const orc_pt_env* env,
                         const orc_spectral* spectral, orc_guide_state* G, uint32_t samplesPerPass, float* image)
{
    if(!s || !p || !surfaces || !G || !image || samplesPerPass == 0 || p->spp % samplesPerPass != 0) return -1;
    if(p->sampler != 0u && p->sampler != 3u) return -1;
    const uint32_t wh = p->width * p->height;
    const uint32_t slots = wh * samplesPerPass;
    const orc_spectral* S = spectral;
    const int nc = S ? 4 : 3;
    /* backup streams: GenerateState of output wh + i of std::mt19937(seed) */
    if(!G->bkValid || G->bkSlots != slots || G->bkSeed != p->seed || G->bkW != p->width || G->bkH != p->height)
    {
        uint32_t* mt = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)wh + slots));
        uint32_t* bk = (uint32_t*)realloc(G->bk, sizeof(uint32_t) * slots);
        if(!mt || !bk) { free(mt); if(bk) G->bk = bk; return -2; }
        G->bk = bk;
        orc_mt19937(p->seed, wh + slots, mt);
        for(uint32_t i = 0; i < slots; i++) G->bk[i] = orc_pcg32_state(mt[wh + i]);
        free(mt);
        G->bkValid = 1; G->bkSlots = slots; G->bkSeed = p->seed; G->bkW = p->width; G->bkH = p->height;
    }
    if(!G->camSet)
    {
        for(int k = 0; k < 3; k++) G->g.cam[k] = p->camPos[k];
        G->camSet = 1;
    }
    pt_job J;
    memset(&J, 0, sizeof(J));
    if(job_sampler(&J, p) != 0) return -2;
    g_slot* Q = (g_slot*)calloc(slots, sizeof(g_slot));
    uint32_t* recKey = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)slots);
    float* recVal = (float*)malloc(sizeof(float) * 2 * (size_t)slots);
    g_rec* recs = (g_rec*)malloc(sizeof(g_rec) * 2 * (size_t)slots);
    if(!Q || !recKey || !recVal || !recs) { free(Q); free(recKey); free(recVal); free(recs); free(J.zsSeeds); return -2; }
    const uint32_t nAll = nLights + (env ? 1u : 0u);
    const float invN = nAll ? 1.0f / (float)nAll : 0.0f;
    const uint32_t T = G->g.tableSize;
    const uint32_t passes = p->spp / samplesPerPass;
    for(uint32_t pass = 0; pass < passes; pass++)
    {
        const uint32_t sampleBase = p->sampleStart + pass * samplesPerPass;
        /* raygen */
        for(uint32_t i = 0; i < slots; i++)
        {
            g_slot* q = &Q[i];
            memset(q, 0, sizeof(*q));
            const uint32_t pixel = i % wh, sample = sampleBase + i / wh;
            const uint32_t x = pixel % p->width, y = pixel / p->width;
            smp_ctx SC = { path_key(p->seed, pixel, sample), x, y, sample, J.zsSeeds ? J.zsSeeds[pixel] : 0u,
                           J.zsSeeds ? p->sampler : 0u, p->samplerMaxSpp ? p->samplerMaxSpp : p->sampleStart + p->spp,
                           J.zsResBits, p->maxDepth };
            q->sc = SC;
            float ox, oy;
            filter_sample(p->filterRadius, urnd(&SC, 0, 6), urnd(&SC, 0, 7), &ox, &oy);
            camera_ray(p, x, y, ox, oy, q->dir, q->org);
            q->tmin = p->nearT; q->tmax = p->farT;
            q->cone.aperture = p->coneAperture;
            q->cone.width = 0.0f;
            for(int k = 0; k < 4; k++) { q->thr[k] = 1.0f; q->wpdf[k] = 1.0f; }
            if(S) orc_spec_sample_waves(urnd(&SC, 0, 9), q->waves, q->wpdf);
            q->alive = 1;
            q->lifted = ORC_GUIDE_INVALID;
        }
        for(uint32_t i = 0; i < 2 * slots; i++) recKey[i] = 0xFFFFFFFFu;
        for(uint32_t depth = 0; depth < p->maxDepth; depth++)
        {
            int any = 0;
            /* closest hit */
            for(uint32_t i = 0; i < slots; i++)
            {
                g_slot* q = &Q[i];
                q->shadow = 0;
                if(!q->alive) continue;
                any = 1;
                float t;
                q->hit = cast1(s, q->org, q->dir, q->tmin, q->tmax, &q->hk, &q->mh, &q->inst, &t);
                if(q->hit) q->tmax = t;
            }
            if(!any) break;
            /* backprop (KCBackpropagateHashGridPath); locks: smallest slot wins */
            for(uint32_t c = 0; c < T; c++) G->lock[c] = 0xFFFFFFFFu;
            for(uint32_t i = 0; i < slots; i++)
            {
                g_slot* q = &Q[i];
                if(!q->alive || !q->hit || surfaces[q->inst].isLight) continue;
                const uint32_t prev = q->lifted;
                if(prev == ORC_GUIDE_INVALID) continue;
                float nextPos[3], wdir[3];
                for(int k = 0; k < 3; k++) { nextPos[k] = q->org[k] + q->tmax * q->dir[k]; wdir[k] = -q->dir[k]; }
                normalize3f(wdir);
                const uint32_t loc = orc_guide_search(&G->g, orc_guide_gen_code(&G->g, nextPos, wdir));
                if(loc == ORC_GUIDE_INVALID) continue;
                float out = q->prevRefl * G->irr[loc];
                if(!isfinite(out)) out = 0.0f;
                g_put(recKey, recVal, i, prev, 0u, out);
                uint32_t* rng = &G->bk[i];
                const float score = q->scoreSum;
                if(score != INFINITY && orc_guide_next_float(rng) * score > out * (float)ORC_GUIDE_LOBES) continue;
                float mcN[3];
                orc_conc_octa_to_dir(q->prevNormal, mcN);
                const uint64_t mcCode = orc_guide_gen_code_stochastic(&G->g, q->org, mcN, rng);
                uint32_t ni = orc_guide_search(&G->g, mcCode);
                if(ni == ORC_GUIDE_INVALID) ni = prev;
                q->lifted = ni;
                if(G->lock[ni] < i + 1u) continue;
                G->lock[ni] = i + 1u;
                orc_mc_state st;
                uint32_t cnt;
                if(score == INFINITY)
                {
                    memset(&st, 0, sizeof(st));
                    cnt = 0u;
                }
                else
                {
                    for(int k = 0; k < 3; k++) st.target[k] = G->mcA[4 * (size_t)prev + k];
                    st.cosine = G->mcA[4 * (size_t)prev + 3];
                    st.weight = G->mcW[prev];
                    cnt = orc_mc_ema(&st, q->org, nextPos, out, G->mcN[prev]);
                }
                if(!isfinite(st.cosine)) st.cosine = 0.0f;
                if(!isfinite(st.target[0]) || !isfinite(st.target[1]) || !isfinite(st.target[2]))
                    st.target[0] = st.target[1] = st.target[2] = 0.0f;
                if(!isfinite(st.weight)) st.weight = 0.0f;
                for(int k = 0; k < 3; k++) q->tmpA[k] = st.target[k];
                q->tmpA[3] = st.cosine;
                q->tmpW = st.weight;
                q->tmpN = cnt;
            }
            /* KCWriteMarkovChains */
            for(uint32_t i = 0; i < slots; i++)
            {
                g_slot* q = &Q[i];
                if(!q->alive || !q->hit || surfaces[q->inst].isLight) continue;
                const uint32_t w = q->lifted;
                if(w == ORC_GUIDE_INVALID || G->lock[w] != i + 1u) continue;
                for(int k = 0; k < 4; k++) G->mcA[4 * (size_t)w + k] = q->tmpA[k];
                G->mcW[w] = q->tmpW;
                G->mcN[w] = q->tmpN;
            }
            /* shade */
            for(uint32_t i = 0; i < slots; i++)
            {
                g_slot* q = &Q[i];
                if(!q->alive) continue;
                if(!q->hit || surfaces[q->inst].isLight)
                    g_light_work(p, surfaces, lights, env, S, invN, q, i, slots, recKey, recVal);
                else
                    g_surface_work(s, p, surfaces, lights, nLights, env, S, G, invN, nAll, q, i);
            }
            /* shadow rays (KCAccumulateShadowRaysGPT) and NEE records */
            for(uint32_t i = 0; i < slots; i++)
            {
                g_slot* q = &Q[i];
                if(!q->shadow) continue;
                if(!visible1(s, q->sorg, q->sdir, 1.0e-5f, q->stmax)) continue;
                for(int k = 0; k < 4; k++) q->rad[k] += q->srad[k];
                if(q->lifted != ORC_GUIDE_INVALID) g_put(recKey, recVal, slots + i, q->lifted, 0u, q->shadowOut);
            }
            /* irradiance records, per cell in (key, position) order */
            uint32_t nr = 0;
            for(uint32_t r = 0; r < 2 * slots; r++)
                if(recKey[r] != 0xFFFFFFFFu) { recs[nr].key = recKey[r]; recs[nr].pos = r; nr++; }
            qsort(recs, nr, sizeof(g_rec), g_rec_cmp);
            for(uint32_t r = 0; r < nr; r++)
            {
                const uint32_t cell = recs[r].key >> 1;
                orc_irr_ema(&G->irr[cell], &G->irrN[cell], recVal[recs[r].pos]);
            }
            for(uint32_t r = 0; r < 2 * slots; r++) recKey[r] = 0xFFFFFFFFu;
        }
        /* film */
        for(uint32_t px = 0; px < wh; px++)
        {
            float* o = &image[4 * (size_t)px];
            for(uint32_t k = 0; k < samplesPerPass; k++)
            {
                const g_slot* q = &Q[px + (size_t)k * wh];
                float rgb[3];
                if(S) orc_spec_to_rgb(S, q->rad, q->waves, q->wpdf, rgb);
                else { rgb[0] = q->rad[0]; rgb[1] = q->rad[1]; rgb[2] = q->rad[2]; }
                o[0] += rgb[0]; o[1] += rgb[1]; o[2] += rgb[2]; o[3] += 1.0f;
            }
        }
    }
    (void)nc;
    free(Q); free(recKey); free(recVal); free(recs); free(J.zsSeeds);
    return 0;
}
