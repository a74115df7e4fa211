/* guide_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker for the GPU guided
 * path tracer; never linked into the product).
 *
 * A plain-C restatement of the building blocks of MRay's guided path tracer
 * (Markov-chain mixture guiding after Alber et al. 2025, as MRay implements
 * it):
 *   hash grid   HashGridView::GenCode / GenCodeStochastic / Search / TryInsert,
 *               SpatioDirCode layout               Source/Tracer/HashGrid.h:18-56, 230-400
 *               HashGrid::View                     HashGrid.h:410-440
 *   mapping     DirectionToConcentricOctahedral, ConcentricOctahedralToDirection,
 *               ConcentricOctahedralWrapInt        Source/Core/GraphicsFunctions.h:318-428
 *               ZUpToNSpace                        GraphicsFunctions.h:540-554
 *               MortonCode::Compose3D<uint64_t>    GraphicsFunctions.h:605-625
 *   lobe        Distribution::GaussianLobe         Source/Tracer/DistributionFunctions.h:230-325
 *   chain       MCState Direction / Target / MeanCosine / EMA, SufficientStatsToLobe,
 *               MCIrradiance::AtomicEMA's update   Source/TracerDLL/GuidedPTRendererShaders.h:278-365
 *   hash        RNGFunctions::HashPCG64::Hash(v, v) Source/Tracer/Random.h:603-633
 *   backup RNG  PermutedCG32                       Source/Tracer/Random.h:762-842
 * Built with -ffp-contract=off: every operation is MRay's, in its order (its
 * vector Dot is the fma chain from 0). */
#include "guide_oracle.h"
#include "zsobol_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI_F 3.1415926535897932384626433f

static inline float dot3(const float a[3], const float b[3])
{
    return fmaf(a[2], b[2], fmaf(a[1], b[1], fmaf(a[0], b[0], 0.0f)));
}
static inline float sign_pm1(float x) { return copysignf(1.0f, x); }
static inline float lerpf_(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline uint32_t required_bits(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

float orc_guide_next_float(uint32_t* s)
{
    const uint32_t r = orc_pcg32_permute(*s);
    *s = orc_pcg32_advance(*s, 1u);
    float f = (float)r * 0x1p-32f;
    const float prev1 = 0x1.fffffep-1f;
    return f < prev1 ? f : prev1;
}

static uint64_t hash_pcg64(uint64_t v)
{
    const uint64_t s = v * 6364136223846793005ull + 1442695040888963407ull;
    uint64_t w = ((s >> ((s >> 59u) + 5u)) ^ s);
    w *= 12605985483714917081ull;
    return (w >> 43u) ^ w;
}

static uint64_t expand3_64(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x001f00000000ffffull;
    x = (x | x << 16) & 0x001f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
static uint64_t morton3_64(uint32_t x, uint32_t y, uint32_t z)
{
    return expand3_64(x) | (expand3_64(y) << 1) | (expand3_64(z) << 2);
}
static uint32_t expand2_32(uint32_t x)
{
    x &= 0x0000ffffu;
    x = (x ^ (x << 8)) & 0x00ff00ffu;
    x = (x ^ (x << 4)) & 0x0f0f0f0fu;
    x = (x ^ (x << 2)) & 0x33333333u;
    x = (x ^ (x << 1)) & 0x55555555u;
    return x;
}
static uint32_t morton2_32(uint32_t x, uint32_t y) { return expand2_32(x) | (expand2_32(y) << 1); }

/* SpatioDirCode: 54 position bits, 6 normal bits, 4 level bits (LSB first). */
static uint64_t compose_code(uint64_t mcPos, uint32_t mcNormal, uint32_t level)
{
    return mcPos | ((uint64_t)mcNormal << 54) | ((uint64_t)level << 60);
}

void orc_dir_to_conc_octa(const float d[3], float st[2])
{
    const float twoOvrPi = (1.0f / PI_F) * 2.0f;        /* InvPi * 2 */
    if(d[0] == 0.0f && d[1] == 0.0f) { st[0] = st[1] = 0.0f; return; }
    const float xAbs = fabsf(d[0]), yAbs = fabsf(d[1]);
    const float phiPrime = atanf(yAbs / xAbs);
    const float one = 1.0f - fabsf(d[2]);
    const float radius = sqrtf(one > 0.0f ? one : 0.0f);
    float v = radius * twoOvrPi * phiPrime;
    float u = radius - v;
    if(d[2] < 0.0f)
    {
        const float uP = 1.0f - v, vP = 1.0f - u;
        u = uP;
        v = vP;
    }
    u *= sign_pm1(d[0]);
    v *= sign_pm1(d[1]);
    st[0] = (u + 1.0f) * 0.5f;
    st[1] = (v + 1.0f) * 0.5f;
}

void orc_conc_octa_to_dir(const float st[2], float out[3])
{
    const float piOvr4 = PI_F * 0.25f;
    const float u = st[0] * 2.0f - 1.0f, v = st[1] * 2.0f - 1.0f;
    const float ua = fabsf(u), va = fabsf(v);
    const float d = 1.0f - (ua + va);
    const float radius = 1.0f - fabsf(d);
    float phiPrime = 0.0f;
    if(radius != 0.0f) phiPrime = ((va - ua) / radius + 1.0f) * piOvr4;
    const float sinP = sinf(phiPrime), cosP = cosf(phiPrime);
    const float cosPhi = sign_pm1(u) * cosP, sinPhi = sign_pm1(v) * sinP;
    const float z = sign_pm1(d) * (1.0f - radius * radius);
    const float xy = radius * sqrtf(2.0f - radius * radius);
    out[0] = cosPhi * xy;
    out[1] = sinPhi * xy;
    out[2] = z;
}

/* ConcentricOctahedralWrapInt for signed texel coordinates, square grid. */
static void conc_octa_wrap_int(int32_t sx, int32_t sy, int32_t dim, int32_t out[2])
{
    int32_t cx = sx, cy = sy;
    if(sx < 0) cx = -2 * dim - sx;
    if(sy < 0) cy = -2 * dim - sy;
    const int32_t ix = cx / dim, iy = cy / dim;
    int32_t fx = abs(cx % dim), fy = abs(cy % dim);
    if((ix & 1) ^ (iy & 1)) { fx = (dim - 1) - fx; fy = (dim - 1) - fy; }
    out[0] = fx;
    out[1] = fy;
}

void orc_guide_view(orc_guide_grid* g, const float aabb[6], const float cam[3], uint32_t posBits,
                    uint32_t normalBits, uint32_t maxLevelOffset, float coneApertureDeg, uint32_t tableSize)
{
    const uint32_t base = 1u << posBits;
    double size[3];
    int mx = 0;
    for(int k = 0; k < 3; k++) size[k] = (double)(aabb[3 + k] - aabb[k]);     /* GeomSpan, then double */
    for(int k = 1; k < 3; k++)
        if(size[k] > size[mx]) mx = k;
    g->baseDelta = (float)((double)base / size[mx]);
    g->baseDim = base;
    g->normalDim = 1u << normalBits;
    g->normalDelta = (float)g->normalDim;
    g->maxLevelOffset = maxLevelOffset;
    const float aperture = (PI_F / 180.0f) * coneApertureDeg;
    g->tanConeHalfTimes2 = tanf(aperture * 0.5f) * 2.0f;
    g->tableSize = tableSize;
    g->maxEntryLimit = (uint32_t)((float)tableSize * 0.6f);
    for(int k = 0; k < 3; k++) { g->cam[k] = cam[k]; g->rmin[k] = aabb[k]; }
}

/* level from the cone width at the position (GenCode / GenCodeStochastic) */
static uint32_t base_level(const orc_guide_grid* g, const float pos[3])
{
    float d[3] = { pos[0] - g->cam[0], pos[1] - g->cam[1], pos[2] - g->cam[2] };
    const float coneWidth = g->tanConeHalfTimes2 * sqrtf(dot3(d, d));
    const uint32_t ratio = (uint32_t)lroundf(coneWidth * g->baseDelta);
    return required_bits(ratio);
}

uint64_t orc_guide_gen_code(const orc_guide_grid* g, const float pos[3], const float normal[3])
{
    const uint32_t levelMax = required_bits(g->baseDim) - 1u;
    uint32_t level = base_level(g, pos);
    level = level < levelMax ? level : levelMax;
    const float levelDelta = g->baseDelta / (float)(1u << level);
    const int32_t edge = (int32_t)(g->baseDim >> level) - 1;
    uint32_t loc[3];
    for(int k = 0; k < 3; k++)
    {
        const float f = (pos[k] - g->rmin[k]) * levelDelta;
        int32_t i = (int32_t)f;
        i = i < 0 ? 0 : (i > edge ? edge : i);
        loc[k] = (uint32_t)i;
    }
    const uint64_t mcPos = morton3_64(loc[0], loc[1], loc[2]);
    const float nZ[3] = { normal[1], normal[2], normal[0] };   /* ZUpToYUp */
    float st[2];
    orc_dir_to_conc_octa(nZ, st);
    uint32_t t[2];
    for(int k = 0; k < 2; k++)
    {
        uint32_t v = (uint32_t)(st[k] * g->normalDelta);
        t[k] = v > g->normalDim - 1u ? g->normalDim - 1u : v;
    }
    return compose_code(mcPos, morton2_32(t[0], t[1]), level);
}

uint64_t orc_guide_gen_code_stochastic(const orc_guide_grid* g, const float pos[3], const float normal[3],
                                       uint32_t* rng)
{
    const uint32_t levelMax = required_bits(g->baseDim) - 1u;
    uint32_t level = base_level(g, pos);
    uint32_t off = (uint32_t)(-log2f(1.0f - orc_guide_next_float(rng)));
    off = off < g->maxLevelOffset ? off : g->maxLevelOffset;
    level = (level + off) < levelMax ? level + off : levelMax;
    const float levelDelta = g->baseDelta / (float)(1u << level);
    const int32_t edge = (int32_t)(g->baseDim >> level) - 1;
    int32_t iv[3];
    float fv[3];
    for(int k = 0; k < 3; k++)
    {
        const float f = (pos[k] - g->rmin[k]) * levelDelta;
        float ip;
        fv[k] = modff(f, &ip);
        iv[k] = (int32_t)ip;
    }
    uint32_t loc[3];
    for(int k = 0; k < 3; k++)
    {
        int32_t i = iv[k] + (orc_guide_next_float(rng) > fv[k] ? 0 : 1);
        i = i < 0 ? 0 : (i > edge ? edge : i);
        loc[k] = (uint32_t)i;
    }
    const uint64_t mcPos = morton3_64(loc[0], loc[1], loc[2]);
    const float nZ[3] = { normal[1], normal[2], normal[0] };
    float st[2];
    orc_dir_to_conc_octa(nZ, st);
    int32_t in[2];
    for(int k = 0; k < 2; k++)
    {
        float ip;
        const float f = modff(st[k] * g->normalDelta, &ip);
        in[k] = (int32_t)ip;
        in[k] += (orc_guide_next_float(rng) > f) ? 0 : 1;
    }
    int32_t t[2] = { 0, 0 };
    if(g->normalDim - 1u != 0u) conc_octa_wrap_int(in[0], in[1], (int32_t)g->normalDim, t);
    return compose_code(mcPos, morton2_32((uint32_t)t[0], (uint32_t)t[1]), level);
}

static uint32_t slot_of(const orc_guide_grid* g, uint64_t code)
{
    const uint64_t v = hash_pcg64(code + hash_pcg64(code));
    return (uint32_t)(v >> 32) & (g->tableSize - 1u);
}

uint32_t orc_guide_search(const orc_guide_grid* g, uint64_t code)
{
    const uint32_t mask = g->tableSize - 1u, index = slot_of(g, code);
    for(uint32_t i = index;; i = (i + 1u) & mask)
    {
        if(g->codes[i] == ORC_GUIDE_EMPTY) return ORC_GUIDE_INVALID;
        if(g->codes[i] == code) return i;
        if(i == ((index - 1u) & mask)) break;
    }
    return ORC_GUIDE_INVALID;
}

uint32_t orc_guide_try_insert(orc_guide_grid* g, uint64_t code, int* inserted)
{
    *inserted = 0;
    if(g->counter >= g->maxEntryLimit) return ORC_GUIDE_INVALID;
    const uint32_t mask = g->tableSize - 1u, index = slot_of(g, code);
    for(uint32_t i = index;; i = (i + 1u) & mask)
    {
        if(g->codes[i] == code) return i;
        if(g->codes[i] == ORC_GUIDE_EMPTY)
        {
            g->codes[i] = code;
            g->counter++;
            *inserted = 1;
            return i;
        }
        if(i == ((index - 1u) & mask)) break;
    }
    return ORC_GUIDE_INVALID;
}

/* ---- Gaussian (vMF) lobe ------------------------------------------------ */
float orc_x_over_exp1m(float x)
{
    const float u = expf(x);
    if(u == 1.0f) return 1.0f;
    if(fabsf(x) < 1.0f) return logf(u) / (u - 1.0f);
    return x / (u - 1.0f);
}

orc_lobe orc_lobe_make(const float dir[3], float kappa)
{
    orc_lobe l;
    memcpy(l.dir, dir, sizeof(l.dir));
    l.kappa = kappa;
    l.alpha = orc_x_over_exp1m(-2.0f * kappa);
    return l;
}

float orc_lobe_pdf(const orc_lobe* l, const float w[3])
{
    const float d[3] = { l->dir[0] - w[0], l->dir[1] - w[1], l->dir[2] - w[2] };
    float r = expf(-0.5f * l->kappa * dot3(d, d));
    r *= l->alpha;
    r *= 0.25f / PI_F;                           /* Inv4Pi */
    return r;
}

/* ZUpToNSpace (Frisvad / Duff et al. frame, JCGT 2017) */
static void zup_to_n(const float v[3], const float n[3], float out[3])
{
    const float s = sign_pm1(n[2]);
    const float c = -1.0f / (s + n[2]);
    const float b = n[0] * n[1] * c;
    const float r0[3] = { 1.0f + s * n[0] * n[0] * c, b, n[0] };
    const float r1[3] = { s * b, s + n[1] * n[1] * c, n[1] };
    const float r2[3] = { -s * n[0], -n[1], n[2] };
    out[0] = dot3(r0, v);
    out[1] = dot3(r1, v);
    out[2] = dot3(r2, v);
}

void orc_lobe_sample(const orc_lobe* l, float xi0, float xi1, float out[3])
{
    const float T = 1.19209290e-7f / 4.0f;
    float r;
    if(l->kappa > T)
    {
        r = 1.0f / l->kappa;
        r *= log1pf(xi1 * expm1f(-2.0f * l->kappa));
    }
    else r = -2.0f * xi1;
    const float cosPhi = 1.0f + r;
    const float sinPhi = sqrtf(-fmaf(r, r, 2.0f * r));
    const float theta = 2.0f * PI_F * xi0;
    const float sinT = sinf(theta), cosT = cosf(theta);
    const float z[3] = { cosT * sinPhi, sinT * sinPhi, cosPhi };
    zup_to_n(z, l->dir, out);
}

/* ---- Markov-chain state ------------------------------------------------ */
void orc_mc_target(const orc_mc_state* s, float out[3])
{
    for(int k = 0; k < 3; k++) out[k] = (s->weight > 0.0f) ? s->target[k] / s->weight : s->target[k];
}

void orc_mc_direction(const orc_mc_state* s, const float pos[3], float out[3])
{
    float t[3];
    orc_mc_target(s, t);
    for(int k = 0; k < 3; k++) out[k] = t[k] - pos[k];
    const float d2 = dot3(out, out);
    if(d2 != 0.0f)
    {
        const float len = sqrtf(d2);
        for(int k = 0; k < 3; k++) out[k] /= len;
    }
}

float orc_mc_mean_cosine(const orc_mc_state* s, const float pos[3], uint32_t n)
{
    float t[3], d[3];
    orc_mc_target(s, t);
    for(int k = 0; k < 3; k++) d[k] = pos[k] - t[k];
    float prior = 0.2f / dot3(d, d);
    prior = prior > 0.0001f ? prior : 0.0001f;
    const float n2 = (float)(n * n);
    float c = (s->weight > 0.0f) ? (s->cosine / s->weight) : 0.0f;
    c = c < 0.0f ? 0.0f : (c > 0.999999f ? 0.999999f : c);
    return c * n2 / (n2 + prior);
}

uint32_t orc_mc_ema(orc_mc_state* s, const float pos[3], const float nt[3], float nw, uint32_t n)
{
    n = (n + 1u) < 1024u ? n + 1u : 1024u;
    const float inv = 1.0f / (float)n;
    const float a = inv > 0.01f ? inv : 0.01f;
    s->weight = lerpf_(s->weight, nw, a);
    for(int k = 0; k < 3; k++) s->target[k] = lerpf_(s->target[k], nw * nt[k], a);
    float nd[3] = { nt[0] - pos[0], nt[1] - pos[1], nt[2] - pos[2] };
    const float inl = 1.0f / sqrtf(dot3(nd, nd));
    for(int k = 0; k < 3; k++) nd[k] *= inl;
    float dir[3];
    orc_mc_direction(s, pos, dir);
    float nc = dot3(nd, dir);
    nc = nc > 0.0f ? nc : 0.0f;
    s->cosine = lerpf_(s->cosine, nw * nc, a);
    s->cosine = s->cosine < s->weight ? s->cosine : s->weight;
    return n;
}

orc_lobe orc_mc_to_lobe(const orc_mc_state* s, uint32_t n, const float pos[3])
{
    float dir[3];
    orc_mc_direction(s, pos, dir);
    const float r = orc_mc_mean_cosine(s, pos, n);
    const float r2 = r * r, r3 = r * r2;
    const float kappa = (3.0f * r - r3) / (1.0f - r2);
    return orc_lobe_make(dir, kappa);
}

void orc_irr_ema(float* irrad, uint32_t* n, float radEst)
{
    *n = (*n + 1u) < 128u ? *n + 1u : 128u;
    const float inv = 1.0f / (float)*n;
    const float t = inv > 0.01f ? inv : 0.01f;
    *irrad = lerpf_(*irrad, radEst, t);
}

/* ---- batch forms for the fixture tests (same record layouts as the MRay
 * driver's ref_guide_* functions) ---------------------------------------- */
static float x_over_exp1m_recip(float x)
{
    const float u = expf(x);
    if(u == 1.0f) return 1.0f;
    if(fabsf(x) < 1.0f) return (u - 1.0f) / logf(u);
    return (u - 1.0f) / x;
}

void orc_guide_lobe_batch(const float* in7, const float* w3, float* out8, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* q = in7 + 7 * i;
        const orc_lobe l = orc_lobe_make(q, q[3]);
        float s[3];
        orc_lobe_sample(&l, q[4], q[5], s);
        float* o = out8 + 8 * i;
        o[0] = l.alpha;
        o[1] = s[0]; o[2] = s[1]; o[3] = s[2];
        o[4] = orc_lobe_pdf(&l, s);
        o[5] = orc_lobe_pdf(&l, w3 + 3 * i);
        o[6] = orc_x_over_exp1m(-2.0f * q[3]);
        o[7] = x_over_exp1m_recip(-2.0f * q[3]);
    }
}

void orc_conc_octa_batch(const float* dir3, float* st2, const float* stIn, float* dirOut, uint32_t n)
{
    for(uint32_t i = 0; i < n; i++)
    {
        orc_dir_to_conc_octa(dir3 + 3 * i, st2 + 2 * i);
        orc_conc_octa_to_dir(stIn + 2 * i, dirOut + 3 * i);
    }
}

void orc_guide_codes_batch(const float* v, const float* in6, uint32_t* rng, uint64_t* out2, uint32_t n)
{
    orc_guide_grid g;
    memset(&g, 0, sizeof(g));
    for(int k = 0; k < 3; k++) { g.cam[k] = v[k]; g.rmin[k] = v[3 + k]; }
    g.baseDelta = v[9];
    g.baseDim = (uint32_t)v[10];
    g.normalDelta = v[11];
    g.normalDim = (uint32_t)v[12];
    g.maxLevelOffset = (uint32_t)v[13];
    g.tanConeHalfTimes2 = v[14];
    for(uint32_t i = 0; i < n; i++)
    {
        out2[2 * i] = orc_guide_gen_code(&g, in6 + 6 * i, in6 + 6 * i + 3);
        out2[2 * i + 1] = orc_guide_gen_code_stochastic(&g, in6 + 6 * i, in6 + 6 * i + 3, rng + i);
    }
}

void orc_guide_table_batch(const uint64_t* codes, uint32_t n, const uint64_t* probe, uint32_t m, uint32_t size,
                           uint32_t* slots, uint32_t* found)
{
    orc_guide_grid g;
    memset(&g, 0, sizeof(g));
    g.codes = (uint64_t*)malloc(sizeof(uint64_t) * size);
    if(!g.codes) return;
    for(uint32_t i = 0; i < size; i++) g.codes[i] = ORC_GUIDE_EMPTY;
    g.tableSize = size;
    g.maxEntryLimit = size;
    int ins;
    for(uint32_t i = 0; i < n; i++) slots[i] = orc_guide_try_insert(&g, codes[i], &ins);
    for(uint32_t i = 0; i < m; i++) found[i] = orc_guide_search(&g, probe[i]);
    free(g.codes);
}
