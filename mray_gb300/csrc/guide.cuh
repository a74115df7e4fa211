// guide.cuh -- device building blocks of guided path tracing (Markov-chain
// mixtures on a spatio-directional hash grid, after Alber et al. 2025, as
// MRay's guided renderer implements it):
//   hash grid   HashGridView::GenCode / GenCodeStochastic / Search /
//               TryInsertAtomic, SpatioDirCode     Source/Tracer/HashGrid.h:18-56, 230-400
//   mapping     concentric octahedral map, ZUpToNSpace, Morton codes
//                                                  Source/Core/GraphicsFunctions.h:318-428, 540-625
//   lobe        Distribution::GaussianLobe         Source/Tracer/DistributionFunctions.h:230-380
//   chain       MCState, SufficientStatsToLobe, the irradiance average
//                                                  Source/TracerDLL/GuidedPTRendererShaders.h:278-365
// Arithmetic is MRay's, operation by operation, with no contraction (the
// _rn intrinsics); the host restatement is the oracle's guide_oracle.c.
#pragma once
#include "mrg_guide.h"
#include "zsobol.cuh"

#include <cstdint>
#include <cuda_runtime.h>

namespace mrg {
namespace guide {

constexpr unsigned long long kEmpty = 0xFFFFFFFFFFFFFFFFull;
constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr uint32_t kLobes = 8;                 // MC_LOBE_COUNT
constexpr float kPi = 3.1415926535897932384626433f;

__device__ __forceinline__ float gmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float gadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float gsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float gdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float gdot(float3 a, float3 b)
{
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmaf_rn(a.x, b.x, 0.0f)));
}
__device__ __forceinline__ float glerp(float a, float b, float t) { return gadd(gmul(a, gsub(1.0f, t)), gmul(b, t)); }
__device__ __forceinline__ float sign_pm1(float x) { return copysignf(1.0f, x); }
__device__ __forceinline__ uint32_t required_bits(uint32_t v) { return v ? 32u - (uint32_t)__clz(v) : 0u; }

// PermutedCG32 as the backup generator: ToFloat01(Next())
__device__ __forceinline__ float next_float(uint32_t& s)
{
    const uint32_t x0 = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    const uint32_t r = (x0 >> 22) ^ x0;
    s = s * 747796405u + 2891336453u;
    return zs_to_float01(r);
}

__device__ __forceinline__ uint64_t expand3_64(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x001f00000000ffffull;
    x = (x | x << 16) & 0x001f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
__device__ __forceinline__ uint32_t expand2_32(uint32_t x)
{
    x &= 0x0000ffffu;
    x = (x ^ (x << 8)) & 0x00ff00ffu;
    x = (x ^ (x << 4)) & 0x0f0f0f0fu;
    x = (x ^ (x << 2)) & 0x33333333u;
    x = (x ^ (x << 1)) & 0x55555555u;
    return x;
}
__device__ __forceinline__ uint64_t compose_code(uint64_t mcPos, uint32_t mcNormal, uint32_t level)
{
    return mcPos | ((uint64_t)mcNormal << 54) | ((uint64_t)level << 60);
}

__device__ __forceinline__ float2 dir_to_conc_octa(float3 d)
{
    const float twoOvrPi = gmul(gdiv(1.0f, kPi), 2.0f);
    if(d.x == 0.0f && d.y == 0.0f) return make_float2(0.0f, 0.0f);
    const float xa = fabsf(d.x), ya = fabsf(d.y);
    const float phiPrime = atanf(gdiv(ya, xa));
    const float radius = __fsqrt_rn(fmaxf(gsub(1.0f, fabsf(d.z)), 0.0f));
    float v = gmul(gmul(radius, twoOvrPi), phiPrime);
    float u = gsub(radius, v);
    if(d.z < 0.0f)
    {
        const float uP = gsub(1.0f, v), vP = gsub(1.0f, u);
        u = uP;
        v = vP;
    }
    u = gmul(u, sign_pm1(d.x));
    v = gmul(v, sign_pm1(d.y));
    return make_float2(gmul(gadd(u, 1.0f), 0.5f), gmul(gadd(v, 1.0f), 0.5f));
}

__device__ __forceinline__ float3 conc_octa_to_dir(float2 st)
{
    const float piOvr4 = gmul(kPi, 0.25f);
    const float u = gsub(gmul(st.x, 2.0f), 1.0f), v = gsub(gmul(st.y, 2.0f), 1.0f);
    const float ua = fabsf(u), va = fabsf(v);
    const float d = gsub(1.0f, gadd(ua, va));
    const float radius = gsub(1.0f, fabsf(d));
    float phiPrime = 0.0f;
    if(radius != 0.0f) phiPrime = gmul(gadd(gdiv(gsub(va, ua), radius), 1.0f), piOvr4);
    float sinP, cosP;
    sincosf(phiPrime, &sinP, &cosP);
    const float cosPhi = gmul(sign_pm1(u), cosP), sinPhi = gmul(sign_pm1(v), sinP);
    const float z = gmul(sign_pm1(d), gsub(1.0f, gmul(radius, radius)));
    const float xy = gmul(radius, __fsqrt_rn(gsub(2.0f, gmul(radius, radius))));
    return make_float3(gmul(cosPhi, xy), gmul(sinPhi, xy), z);
}

// ConcentricOctahedralWrapInt, square grid of `dim` texels a side
__device__ __forceinline__ int2 conc_octa_wrap_int(int32_t sx, int32_t sy, int32_t dim)
{
    const int32_t cx = (sx < 0) ? -2 * dim - sx : sx, cy = (sy < 0) ? -2 * dim - sy : sy;
    const int32_t ix = cx / dim, iy = cy / dim;
    int32_t fx = abs(cx % dim), fy = abs(cy % dim);
    if((ix & 1) ^ (iy & 1)) { fx = (dim - 1) - fx; fy = (dim - 1) - fy; }
    return make_int2(fx, fy);
}

using Grid = GuideGrid;

__device__ __forceinline__ uint32_t base_level(const Grid& g, float3 pos)
{
    const float3 d = make_float3(gsub(pos.x, g.cam.x), gsub(pos.y, g.cam.y), gsub(pos.z, g.cam.z));
    const float coneWidth = gmul(g.tanConeHalfTimes2, __fsqrt_rn(gdot(d, d)));
    const uint32_t ratio = (uint32_t)lroundf(gmul(coneWidth, g.baseDelta));
    return required_bits(ratio);
}

__device__ __forceinline__ uint64_t gen_code(const Grid& g, float3 pos, float3 normal)
{
    const uint32_t levelMax = required_bits(g.baseDim) - 1u;
    const uint32_t level = min(base_level(g, pos), levelMax);
    const float levelDelta = gdiv(g.baseDelta, (float)(1u << level));
    const int32_t edge = (int32_t)(g.baseDim >> level) - 1;
    const float p[3] = { pos.x, pos.y, pos.z }, r[3] = { g.rmin.x, g.rmin.y, g.rmin.z };
    uint32_t loc[3];
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
        int32_t i = (int32_t)gmul(gsub(p[k], r[k]), levelDelta);
        loc[k] = (uint32_t)max(0, min(i, edge));
    }
    const uint64_t mcPos = expand3_64(loc[0]) | (expand3_64(loc[1]) << 1) | (expand3_64(loc[2]) << 2);
    const float2 st = dir_to_conc_octa(make_float3(normal.y, normal.z, normal.x));   // ZUpToYUp
    const uint32_t tx = min((uint32_t)gmul(st.x, g.normalDelta), g.normalDim - 1u);
    const uint32_t ty = min((uint32_t)gmul(st.y, g.normalDelta), g.normalDim - 1u);
    return compose_code(mcPos, expand2_32(tx) | (expand2_32(ty) << 1), level);
}

// The parts of GenCodeStochastic that do not depend on the random numbers:
// the cone's base level at pos and the normal's texel and fractions.  Several
// stochastic codes at one point share them.
struct CodeBase
{
    uint32_t level;
    float    fx, fy;
    int32_t  nx, ny;
};

__device__ __forceinline__ CodeBase code_base(const Grid& g, float3 pos, float3 normal)
{
    CodeBase b;
    b.level = base_level(g, pos);
    const float2 st = dir_to_conc_octa(make_float3(normal.y, normal.z, normal.x));   // ZUpToYUp
    float ipx, ipy;
    b.fx = modff(gmul(st.x, g.normalDelta), &ipx);
    b.fy = modff(gmul(st.y, g.normalDelta), &ipy);
    b.nx = (int32_t)ipx;
    b.ny = (int32_t)ipy;
    return b;
}

__device__ __forceinline__ uint64_t gen_code_stochastic(const Grid& g, const CodeBase& b, float3 pos, uint32_t& rng)
{
    const uint32_t levelMax = required_bits(g.baseDim) - 1u;
    const uint32_t off = min((uint32_t)(-log2f(gsub(1.0f, next_float(rng)))), g.maxLevelOffset);
    const uint32_t level = min(b.level + off, levelMax);
    const float levelDelta = gdiv(g.baseDelta, (float)(1u << level));
    const int32_t edge = (int32_t)(g.baseDim >> level) - 1;
    const float p[3] = { pos.x, pos.y, pos.z }, r[3] = { g.rmin.x, g.rmin.y, g.rmin.z };
    int32_t iv[3];
    float fv[3];
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
        float ip;
        fv[k] = modff(gmul(gsub(p[k], r[k]), levelDelta), &ip);
        iv[k] = (int32_t)ip;
    }
    uint32_t loc[3];
#pragma unroll
    for(int k = 0; k < 3; k++)
    {
        const int32_t i = iv[k] + ((next_float(rng) > fv[k]) ? 0 : 1);
        loc[k] = (uint32_t)max(0, min(i, edge));
    }
    const uint64_t mcPos = expand3_64(loc[0]) | (expand3_64(loc[1]) << 1) | (expand3_64(loc[2]) << 2);
    int32_t nx = b.nx, ny = b.ny;
    nx += (next_float(rng) > b.fx) ? 0 : 1;
    ny += (next_float(rng) > b.fy) ? 0 : 1;
    int2 t = make_int2(0, 0);
    if(g.normalDim - 1u != 0u) t = conc_octa_wrap_int(nx, ny, (int32_t)g.normalDim);
    return compose_code(mcPos, expand2_32((uint32_t)t.x) | (expand2_32((uint32_t)t.y) << 1), level);
}

__device__ __forceinline__ uint64_t gen_code_stochastic(const Grid& g, float3 pos, float3 normal, uint32_t& rng)
{
    return gen_code_stochastic(g, code_base(g, pos, normal), pos, rng);
}

__device__ __forceinline__ uint32_t first_slot(const Grid& g, uint64_t code)
{
    const uint64_t v = zs_hash_pcg64(code + zs_hash_pcg64(code));
    return (uint32_t)(v >> 32) & g.tableMask;
}

__device__ __forceinline__ uint32_t search(const Grid& g, uint64_t code)
{
    const uint32_t index = first_slot(g, code);
    for(uint32_t i = index;; i = (i + 1u) & g.tableMask)
    {
        const unsigned long long c = g.codes[i];
        if(c == kEmpty) return kInvalid;
        if(c == code) return i;
        if(i == ((index - 1u) & g.tableMask)) break;
    }
    return kInvalid;
}

// TryInsertAtomic: linear probing with a 64-bit compare-and-swap on empty slots
__device__ __forceinline__ uint32_t try_insert(const Grid& g, uint64_t code)
{
    if(*(volatile uint32_t*)g.counter >= g.maxEntryLimit) return kInvalid;
    const uint32_t index = first_slot(g, code);
    for(uint32_t i = index;; i = (i + 1u) & g.tableMask)
    {
        const unsigned long long c = *(volatile unsigned long long*)&g.codes[i];
        if(c == code) return i;
        if(c == kEmpty)
        {
            const unsigned long long old = atomicCAS(&g.codes[i], kEmpty, (unsigned long long)code);
            if(old == kEmpty) { atomicAdd(g.counter, 1u); return i; }
            if(old == code) return i;
        }
        if(i == ((index - 1u) & g.tableMask)) break;
    }
    return kInvalid;
}

// TryInsertAtomic's probe from slot `index` whose code was already read as c
// (the entry-limit test done by the caller).
__device__ __forceinline__ uint32_t insert_from(const Grid& g, uint64_t code, uint32_t index, unsigned long long c)
{
    for(uint32_t i = index;; i = (i + 1u) & g.tableMask)
    {
        if(i != index) c = *(volatile unsigned long long*)&g.codes[i];
        if(c == code) return i;
        if(c == kEmpty)
        {
            const unsigned long long old = atomicCAS(&g.codes[i], kEmpty, (unsigned long long)code);
            if(old == kEmpty) { atomicAdd(g.counter, 1u); return i; }
            if(old == code) return i;
        }
        if(i == ((index - 1u) & g.tableMask)) break;
    }
    return kInvalid;
}

// ---- Gaussian (vMF) lobe ------------------------------------------------------
struct Lobe
{
    float3 dir;
    float  kappa, alpha;
};

__device__ __forceinline__ float x_over_exp1m(float x)
{
    const float u = expf(x);
    if(u == 1.0f) return 1.0f;
    if(fabsf(x) < 1.0f) return gdiv(logf(u), gsub(u, 1.0f));
    return gdiv(x, gsub(u, 1.0f));
}

__device__ __forceinline__ Lobe lobe_make(float3 dir, float kappa)
{
    Lobe l;
    l.dir = dir;
    l.kappa = kappa;
    l.alpha = x_over_exp1m(gmul(-2.0f, kappa));
    return l;
}

__device__ __forceinline__ float lobe_pdf(const Lobe& l, float3 w)
{
    const float3 d = make_float3(gsub(l.dir.x, w.x), gsub(l.dir.y, w.y), gsub(l.dir.z, w.z));
    float r = expf(gmul(gmul(-0.5f, l.kappa), gdot(d, d)));
    r = gmul(r, l.alpha);
    return gmul(r, gdiv(0.25f, kPi));
}

__device__ __forceinline__ float3 zup_to_n(float3 v, float3 n)
{
    const float s = sign_pm1(n.z);
    const float c = gdiv(-1.0f, gadd(s, n.z));
    const float b = gmul(gmul(n.x, n.y), c);
    const float3 r0 = make_float3(gadd(1.0f, gmul(gmul(gmul(s, n.x), n.x), c)), b, n.x);
    const float3 r1 = make_float3(gmul(s, b), gadd(s, gmul(gmul(n.y, n.y), c)), n.y);
    const float3 r2 = make_float3(gmul(-s, n.x), -n.y, n.z);
    return make_float3(gdot(r0, v), gdot(r1, v), gdot(r2, v));
}

__device__ __forceinline__ float3 lobe_sample(const Lobe& l, float xi0, float xi1)
{
    const float T = 1.19209290e-7f / 4.0f;
    float r;
    if(l.kappa > T)
    {
        r = gdiv(1.0f, l.kappa);
        r = gmul(r, log1pf(gmul(xi1, expm1f(gmul(-2.0f, l.kappa)))));
    }
    else r = gmul(-2.0f, xi1);
    const float cosPhi = gadd(1.0f, r);
    const float sinPhi = __fsqrt_rn(-__fmaf_rn(r, r, gmul(2.0f, r)));
    const float theta = gmul(gmul(2.0f, kPi), xi0);
    float sinT, cosT;
    sincosf(theta, &sinT, &cosT);
    return zup_to_n(make_float3(gmul(cosT, sinPhi), gmul(sinT, sinPhi), cosPhi), l.dir);
}

// ---- Markov-chain state --------------------------------------------------------
struct Chain
{
    float3 target;
    float  cosine, weight;
};

__device__ __forceinline__ float3 chain_target(const Chain& s)
{
    return (s.weight > 0.0f) ? make_float3(gdiv(s.target.x, s.weight), gdiv(s.target.y, s.weight),
                                           gdiv(s.target.z, s.weight))
                             : s.target;
}

__device__ __forceinline__ float3 chain_direction(const Chain& s, float3 pos)
{
    const float3 t = chain_target(s);
    float3 d = make_float3(gsub(t.x, pos.x), gsub(t.y, pos.y), gsub(t.z, pos.z));
    const float d2 = gdot(d, d);
    if(d2 != 0.0f)
    {
        const float len = __fsqrt_rn(d2);
        d = make_float3(gdiv(d.x, len), gdiv(d.y, len), gdiv(d.z, len));
    }
    return d;
}

__device__ __forceinline__ float chain_mean_cosine(const Chain& s, float3 pos, uint32_t n)
{
    const float3 t = chain_target(s);
    const float3 d = make_float3(gsub(pos.x, t.x), gsub(pos.y, t.y), gsub(pos.z, t.z));
    const float prior = fmaxf(0.0001f, gdiv(0.2f, gdot(d, d)));
    const float n2 = (float)(n * n);
    float c = (s.weight > 0.0f) ? gdiv(s.cosine, s.weight) : 0.0f;
    c = fminf(fmaxf(c, 0.0f), 0.999999f);
    return gdiv(gmul(c, n2), gadd(n2, prior));
}

__device__ __forceinline__ uint32_t chain_ema(Chain& s, float3 pos, float3 nt, float nw, uint32_t n)
{
    n = min(n + 1u, 1024u);
    const float a = fmaxf(gdiv(1.0f, (float)n), 0.01f);
    s.weight = glerp(s.weight, nw, a);
    s.target = make_float3(glerp(s.target.x, gmul(nw, nt.x), a), glerp(s.target.y, gmul(nw, nt.y), a),
                           glerp(s.target.z, gmul(nw, nt.z), a));
    float3 nd = make_float3(gsub(nt.x, pos.x), gsub(nt.y, pos.y), gsub(nt.z, pos.z));
    const float inl = gdiv(1.0f, __fsqrt_rn(gdot(nd, nd)));
    nd = make_float3(gmul(nd.x, inl), gmul(nd.y, inl), gmul(nd.z, inl));
    const float3 dir = chain_direction(s, pos);
    const float nc = fmaxf(0.0f, gdot(nd, dir));
    s.cosine = glerp(s.cosine, gmul(nw, nc), a);
    s.cosine = fminf(s.cosine, s.weight);
    return n;
}

__device__ __forceinline__ Lobe chain_to_lobe(const Chain& s, uint32_t n, float3 pos)
{
    const float3 dir = chain_direction(s, pos);
    const float r = chain_mean_cosine(s, pos, n);
    const float r2 = gmul(r, r), r3 = gmul(r, r2);
    const float kappa = gdiv(gsub(gmul(3.0f, r), r3), gsub(1.0f, r2));
    return lobe_make(dir, kappa);
}

__device__ __forceinline__ void irr_ema(float& irrad, uint32_t& n, float radEst)
{
    n = min(n + 1u, 128u);
    const float t = fmaxf(gdiv(1.0f, (float)n), 0.01f);
    irrad = glerp(irrad, radEst, t);
}

} // namespace guide
} // namespace mrg
