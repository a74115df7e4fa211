// mrg_pt.h -- device data and host launch interface of the wavefront path tracer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mrg_build.h"

namespace mrg {

// Per surface (= per instance; indexed by the transform key's index portion).
enum PtMaterial : uint32_t
{
    kMatLambert = 0,    // MaterialsDefault.hpp:29-110
    kMatReflect = 1,    // perfect mirror
    kMatRefract = 2,    // smooth dielectric, Fresnel-sampled (:230-355)
    kMatUnreal  = 3     // GGX metallic-roughness + Burley diffuse (:465-720)
};

struct __align__(16) PtSurface
{
    float4 m[3];        // local -> world rows
    float4 inv[3];      // world -> local rows (normals use its transpose)
    float4 albedo;      // xyz albedo, w: roughness
    float4 mat;         // x: metallic, y: specular, z: front IoR, w: back IoR
    uint4  info;        // x: 1 if light, y: first light index, z: primitive key base, w: PtMaterial
    uint4  tex;         // x: albedo texture index + 1 (0: constant albedo)
};

// Albedo texture: RGBA texels, bilinear, wrap addressed; levels 1.. of its
// mip chain (mipCount > 1) follow one another in `mips`, each max(w >> m, 1) x
// max(h >> m, 1) texels of the same format (Graphics::TextureMipPixelStart).
struct __align__(16) PtTexture
{
    const void* texels;
    uint32_t    width, height;
    uint32_t    format;         // 0 RGBA8 unorm, 1 RGBA f32
    uint32_t    mipCount;       // 1: level 0 only
    const void* mips;
};

// One light per emitting triangle (MRay's primitive-backed lights,
// Source/Tracer/LightsDefault.hpp:14-160), in world space.
struct __align__(16) PtLight
{
    float4 p0;          // w: area
    float4 p1;          // w: instance index (uint32 bits), for emission gradients
    float4 p2;
    float4 n;           // geometric normal, w: two-sided (0/1)
    float4 radiance;
};

// Skysphere boundary light (LightSkysphere<SphericalCoordConverter>,
// Source/Tracer/LightsDefault.hpp:175-222, 300-420): a lat-long radiance map
// with its piecewise-constant 2D sampling distribution (Distributions.h).
// It is the last light of the uniform light sampler.
struct PtEnv
{
    const float4* texels;        // RGBA per texel, row-major, row 0 at v = 0
    const float*  cdfX;          // width * height row CDFs
    const float*  cdfY;          // height marginal CDF
    float4        m[3];          // ApplyV rows
    float4        inv[3];        // InvApplyV rows
    uint32_t      width, height; // 1 x 1: constant radiance, uniform uv sampling
    float         sceneDiameter; // |(span.x, span.z)| of the scene box
    uint32_t      enabled;
};

// Spectral context (Jakob & Hanika 2019 RGB -> spectrum, 4 wavelengths per
// path; Source/Tracer/SpectrumContext.{h,hpp,cu}).
struct PtSpectral
{
    const float* lut;            // 9 * res^3: [table][coefficient][z][y][x]
    const float* observer;       // cieCount * 3, divided by the CIE integrals
    const float* illuminant;     // cieCount, scaled by Y integral / norm factor
    float        xyzToRgb[9];
    uint32_t     lutRes, cieCount;
    uint32_t     enabled;
};

// Path-replay adjoint of the image with respect to an f32 albedo texture
// (no reference counterpart): the replay of a pass scatters
// delta[pixel] * (radiance after the vertex) / albedo * bilinear weight
// into grad for every Lambert vertex whose albedo is the texture.
struct PtAdjoint
{
    const float4* delta;        // dLoss / dPixel (RGB) per pixel
    float*        grad;         // RGBA per texel (A unused)
    const float4* radTotal;     // primal radiance per path slot
    uint32_t      texIndex;     // texture id + 1 (0: no texture parameter)
    float         invSpp;       // 1 / samples per pixel of the image
    uint32_t      enabled;
    double*       gradEmission; // RGBA per instance: dLoss / d(area-light radiance), FP64 sums, or null
};

// Radiance-cache use by the path tracer (mode 1): a path ends at its second
// vertex with a cache query of the outgoing radiance there, except the sparse
// training paths (one slot in trainStride, chosen by hash), which record at
// vertices 1..recPerPath the cache inputs, the throughput on arrival and the
// radiance gathered before the vertex, and end at vertex recPerPath + 1 on a
// cache query themselves (self-training); targets follow from each training
// path's final radiance.
struct PtCacheUse
{
    uint32_t  mode;
    uint32_t  recPerPath;
    uint32_t  trainStride;    // 0: no training paths
    uint32_t  batchCap;       // training samples kept per pass
    float4*   queryIn;        // 4 per slot
    uint32_t* queryList;
    uint32_t* queryCount;
    float4*   queryOut;       // per slot
    float4*   recIn;          // 4 per record (slot * recPerPath + vertex - 1)
    float4*   recAux;         // 2 per record: throughput (w: 1 = valid), radiance before
};

struct PtCamera
{
    float pos[3];
    float bottomLeft[3];
    float right[3];
    float up[3];
    float planeSize[2];
    float nearT, farT;
};

struct PtLaunch
{
    uint32_t width, height;
    uint32_t slots;          // paths per pass = width * height * samplesPerPass
    uint32_t samplesPerPass;
    uint32_t sampleBase;     // sample index of the pass's first sample
    uint32_t rrStart, maxDepth;
    uint32_t sampleMode;     // 0 pure, 1 NEE, 2 NEE + MIS
    uint32_t seed;
    uint32_t nLights;        // triangle lights; the skysphere, if enabled, follows them
    float    filterSigma;
    float    coneAperture;   // camera rays' cone aperture: 2 tan(fovY / 2) / height
    uint32_t sampler;        // 0: counter-based independent numbers, 1: ZSobol, 2: ZSobol (Owen order), 3: PCG32
    uint32_t zsMaxSpp;       // ZSobol initialMaxSampleCount
    uint32_t zsResBits;      // ZSobol resMaxBits
    const uint32_t* zsSeeds; // ZSobol / PCG32 per-pixel mt19937 seeds (row-major)
    const uint32_t* zsTables;// ZSobol matrices (3 x 52) then digit permutations (4 x uint64)
    PtCamera cam;
    PtEnv    env;
    PtSpectral spec;
    PtAdjoint  adj;
    PtCacheUse cache;
};

// Path state, structure of arrays (device).
struct PtPaths
{
    float4*   rays;          // 2 per slot (RayGMem)
    uint4*    hits;          // HitKeyPack per slot
    float2*   meta;          // MetaHit per slot
    float2*   cone;          // ray cone of the path's current ray: aperture, width
    float4*   thr;           // throughput (RGB in xyz, or 4 wavelengths)
    float4*   rad;           // radiance (RGB in xyz, or 4 wavelengths)
    float*    prevPdf;       // pdf of the last BxDF sample (MIS)
    float4*   waves;         // spectral: wavelengths of the path
    float4*   wavePdf;       // spectral: their sampling pdfs
    uint32_t* state;         // depth | type << 8
    float4*   shadowRays;    // 2 per slot
    float4*   shadowRad;
    uint32_t* visBits;       // visibility, one bit per slot
    uint32_t* listA;         // alive lists (ping-pong)
    uint32_t* listB;
    uint32_t* shadowList;
    uint32_t* shadowLight;   // adjoint: area light of the slot's NEE sample (~0u: the skysphere)
    uint32_t* counts;        // [0] list A count, [1] list B count, [2] shadow count, [3] pad
    uint32_t* workKeys;      // work key per alive entry (partitioning)
    uint32_t* workKeysOut;
    uint32_t* listSorted;    // alive list grouped by work key
    uint32_t* sortHist;      // multi-split count table
    uint32_t  capacity;
};

// Work keys of the partition before shading: miss, light, then one per
// material group (PtMaterial).
constexpr uint32_t kPtWorkKeyBits = 3;

cudaError_t pt_raygen(const PtLaunch& L, const PtPaths& P, uint32_t* aliveList, uint32_t* aliveCount,
                      int smCount, cudaStream_t st);
// Scene tables the shade kernel reads.
struct PtSceneTables
{
    const PtSurface* surfaces;
    uint32_t         nSurfaces;
    const PtLight*   lights;
    const float4*    tris;        // 3 per primitive key
    uint32_t         nTris;
    const float4*    uvs;         // 2 per primitive key, or null
    const PtTexture* textures;
};

cudaError_t pt_shade_impl(const PtLaunch& L, const PtPaths& P, const PtSceneTables& T,
                          const uint32_t* aliveList, const uint32_t* aliveCount,
                          uint32_t* nextList, uint32_t* nextCount, int smCount, cudaStream_t st);
cudaError_t pt_work_keys(const PtPaths& P, const PtSurface* surfaces, uint32_t nSurfaces,
                         const uint32_t* aliveList, const uint32_t* aliveCount, int smCount, cudaStream_t st);
// rad[slot] += thr[slot] * queryOut[slot] for the queried slots (a
// spectral path takes the RGB answer at its wavelengths).
cudaError_t pt_cache_apply(const PtPaths& P, const PtCacheUse& C, const PtSpectral& S, int smCount,
                           cudaStream_t st);
// Training batch from the records of a pass: target = (final radiance -
// radiance before) / throughput (in RGB; spectral estimates converted as the
// film converts them), valid records compacted (at most batchCap).
cudaError_t pt_cache_targets(const PtPaths& P, const PtCacheUse& C, const PtSpectral& S, uint32_t slots,
                             float4* batchIn, float4* batchTarget, uint32_t* batchCount, int smCount,
                             cudaStream_t st);
cudaError_t pt_resolve(const PtLaunch& L, const PtPaths& P, const PtLight* lights, uint32_t depth, int smCount,
                       cudaStream_t st);
// out[i] += acc[i] (f32 from the FP64 emission-gradient sums), n entries.
cudaError_t pt_add_emission_grad(const double* acc, float* out, uint32_t n, cudaStream_t st);
cudaError_t pt_film(const PtLaunch& L, const PtPaths& P, float4* image, cudaStream_t st);

// Texels of mip levels 1 .. TextureMipCount - 1 of a w x h texture.
// Graphics::TextureMipCount: levels of a full chain, bits of max(w, h)
inline uint32_t mip_level_count(uint32_t w, uint32_t h)
{
    uint32_t m = w > h ? w : h, n = 0;
    for(; m; m >>= 1) n++;
    return n;
}
// Texels of levels 1 .. levels - 1 (all of a full chain by default); the
// offset of level m in a chain is mip_chain_texels(w, h, m).
inline size_t mip_chain_texels(uint32_t w, uint32_t h, uint32_t levels = 0xFFFFFFFFu)
{
    size_t n = 0;
    for(uint32_t m = 1; m < levels && ((w >> (m - 1)) > 1u || (h >> (m - 1)) > 1u); m++)
        n += (size_t)((w >> m) ? (w >> m) : 1u) * ((h >> m) ? (h >> m) : 1u);
    return n;
}
// The 8 per-axis sample offsets (pixels) of KCGenerateMipmaps' stratified
// accumulation and the Gaussian filter's 1D weights at them (GaussianFilter::
// Evaluate is their product), made on the host.
struct MipTaps
{
    float off[8];
    float g[8];
};
// Levels 1.. of the texture's mip chain into `mips` (KCGenerateMipmaps,
// Source/Tracer/TextureFilter.cu:124-192); *count = the chain's level count.
// Synchronous.
// Levels 1 .. levels - 1 of a chain, each filtered from its parent; the
// levels whose bit is set in validMask are already in place and kept
// (KCGenerateMipmaps' validMips).  Synchronous.
cudaError_t generate_mips(const void* texels, void* mips, uint32_t w, uint32_t h, uint32_t format, const MipTaps& taps,
                          uint32_t levels, uint32_t validMask);

} // namespace mrg
