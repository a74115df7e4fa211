/* zsobol_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker for the GPU ZSobol
 * generator; never linked into the product).
 *
 * A plain-C restatement of MRay's ZSobol random-number group:
 *   seeds:   RNGGroupZSobol::RNGGroupZSobol      Source/Tracer/Random.cu:1149-1230
 *            (per-pixel seed = i-th output of std::mt19937(seed32), MT19937 as
 *            published by Matsumoto & Nishimura 1998, restated here)
 *   state:   ZSobol::ZSobol                      Source/Tracer/Random.cu:356-383
 *   index:   ZSobol::SampleIndex                 Source/Tracer/Random.cu:266-342
 *   output:  ZSobol::Next / Next2D / Next3D      Source/Tracer/Random.cu:385-420
 *   matrix:  BitwiseMatrixMult                   Source/Tracer/Random.cu:249-263
 *   scramble ScambleOwenFast                     Source/Tracer/Random.cu:141-150
 *   mixing:  MixBits                             Source/Tracer/Random.cu:156-165
 *   hash:    RNGFunctions::HashPCG64::Hash       Source/Tracer/Random.h:603-633
 *   list:    GenerateRNFromList / RNRequestList  Source/Tracer/Random.cu:426-470,
 *                                                Source/Tracer/Random.h:679-717
 * and MRay's independent group:
 *   seeds:   RNGGroupIndependent::RNGGroupIndependent Source/Tracer/Random.cu:661-726
 *            (the same std::mt19937(seed32) outputs, one per pixel, each
 *            through PermutedCG32::GenerateState)
 *   stream:  PermutedCG32 Step / Permute / Next     Source/Tracer/Random.h:762-810
 *   jump:    PermutedCG32::Advance                  Source/Tracer/Random.h:812-842
 *            (Brown, "Random Number Generation with Arbitrary Stride",
 *            Trans. Am. Nucl. Soc. 1994; the LCG constants are PCG's
 *            published 32-bit multiplier and increment, the output
 *            permutation PCG's RXS-M-XS)
 * The three 52-column Sobol matrices come from the Sobol recurrence (dims 0-2:
 * the reversed identity; x + 1 with m = {1}; x^2 + x + 1 with m = {1, 3}) and
 * the 24 base-4 digit permutations from the swap-recursive enumeration of the
 * permutations of {0, 1, 2, 3}; both are built here, not copied. */
#include "zsobol_oracle.h"

#include <stdlib.h>
#include <string.h>

#define ZS_WIDTH 52

static uint32_t g_mat[3][ZS_WIDTH];
static uint8_t g_perm[24][4];
static int g_ready = 0;

static void perm_rec(uint8_t* a, int k, int* n)
{
    if(k == 4) { memcpy(g_perm[(*n)++], a, 4); return; }
    for(int i = k; i < 4; i++)
    {
        uint8_t t = a[k]; a[k] = a[i]; a[i] = t;
        perm_rec(a, k + 1, n);
        t = a[k]; a[k] = a[i]; a[i] = t;
    }
}

/* Direction numbers m_k of a Sobol dimension with primitive polynomial of
 * degree s and inner coefficients a (bit j-1 = coefficient of x^(s-j)),
 * column k (1-based) = m_k placed with its top bit at bit 31 for k <= 32 and
 * shifted right by k - 32 beyond. */
static void sobol_dim(uint32_t* col, int s, uint32_t a, const uint64_t* m0)
{
    uint64_t m[ZS_WIDTH + 1];
    for(int k = 1; k <= s; k++) m[k] = m0[k - 1];
    for(int k = s + 1; k <= ZS_WIDTH; k++)
    {
        uint64_t v = m[k - s] ^ (m[k - s] << s);
        for(int j = 1; j < s; j++)
            if((a >> (s - 1 - j)) & 1u) v ^= m[k - j] << j;
        m[k] = v;
    }
    for(int k = 1; k <= ZS_WIDTH; k++)
        col[k - 1] = (k <= 32) ? (uint32_t)(m[k] << (32 - k)) : (uint32_t)(m[k] >> (k - 32));
}

static void zs_init(void)
{
    if(g_ready) return;
    for(int k = 0; k < ZS_WIDTH; k++) g_mat[0][k] = (k < 32) ? (0x80000000u >> k) : 0u;
    const uint64_t m1[1] = { 1 }, m2[2] = { 1, 3 };
    sobol_dim(g_mat[1], 1, 0u, m1);
    sobol_dim(g_mat[2], 2, 1u, m2);
    uint8_t a[4] = { 0, 1, 2, 3 };
    int n = 0;
    perm_rec(a, 0, &n);
    g_ready = 1;
}

void orc_zs_tables(uint32_t* matrices, uint8_t* perms)
{
    zs_init();
    if(matrices) memcpy(matrices, g_mat, sizeof(g_mat));
    if(perms) memcpy(perms, g_perm, sizeof(g_perm));
}

/* ---- MT19937 (the published algorithm; std::mt19937's default parameters) ---- */
typedef struct { uint32_t mt[624]; int i; } mt_state;

static void mt_seed(mt_state* s, uint32_t seed)
{
    s->mt[0] = seed;
    for(int i = 1; i < 624; i++) s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->i = 624;
}

static uint32_t mt_next(mt_state* s)
{
    if(s->i >= 624)
    {
        for(int k = 0; k < 624; k++)
        {
            uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7FFFFFFFu);
            s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
        }
        s->i = 0;
    }
    uint32_t y = s->mt[s->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

void orc_mt19937(uint32_t seed, uint32_t count, uint32_t* out)
{
    mt_state s;
    mt_seed(&s, seed);
    for(uint32_t i = 0; i < count; i++) out[i] = mt_next(&s);
}

/* ---- hashing ---- */
static uint64_t mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7FB5D329728EA185ull;
    v ^= v >> 27;
    v *= 0x81DADEF4BC2DD44Dull;
    v ^= v >> 33;
    return v;
}

static uint64_t hash_pcg64(uint64_t v)
{
    uint64_t s = v * 6364136223846793005ull + 1442695040888963407ull;
    uint64_t word = (s >> ((s >> 59) + 5u)) ^ s;
    word *= 12605985483714917081ull;
    return (word >> 43) ^ word;
}

static uint64_t hash_dim_seed(uint32_t dim, uint32_t seed)
{
    uint64_t v = 0;
    v = hash_pcg64((uint64_t)dim + v);
    v = hash_pcg64((uint64_t)seed + v);
    return v;
}

static uint32_t brev32(uint32_t v)
{
    uint32_t r = 0;
    for(int i = 0; i < 32; i++) { r = (r << 1) | (v & 1u); v >>= 1; }
    return r;
}

static uint32_t owen_fast(uint32_t v, uint32_t seed)
{
    v = brev32(v);
    v ^= v * 0x3A20ADEAu;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526C56u;
    v ^= v * 0x53A22864u;
    return v;
}

static uint32_t mat_mul(int d, uint64_t a)
{
    uint32_t r = 0;
    for(int i = 0; i < ZS_WIDTH; i++)
    {
        if(a == 0) return r;
        if(a & 1u) r ^= g_mat[d][i];
        a >>= 1;
    }
    return r;
}

static uint32_t bit_width32(uint32_t v)
{
    uint32_t n = 0;
    while(v) { n++; v >>= 1; }
    return n;
}

typedef struct { uint32_t seed; int32_t nDigits; uint32_t log2Spp; uint64_t morton; } zs_gen;

static zs_gen zs_make(uint64_t pixelMorton, uint32_t sampleIndex, uint32_t seed, uint32_t initialMaxSpp,
                      uint32_t resMaxBits)
{
    zs_gen g;
    g.seed = seed;
    uint32_t local = sampleIndex, maxSpp = initialMaxSpp;
    for(uint32_t i = 0; i < 32; i++)
    {
        uint32_t cur = initialMaxSpp << i;
        if(local < cur) break;
        local -= cur;
        maxSpp <<= 1;
    }
    g.log2Spp = bit_width32(maxSpp) - 1u;
    uint32_t log4 = (g.log2Spp + 1u) / 2u;
    g.nDigits = (int32_t)(resMaxBits + log4);
    g.morton = (pixelMorton << g.log2Spp) | local;
    return g;
}

static uint64_t zs_index(const zs_gen* g, uint32_t dim)
{
    const uint32_t mixer = 0x55555555u * dim;
    uint64_t idx = 0;
    const int odd = (int)(g->log2Spp & 1u);
    const int32_t last = odd ? 1 : 0;
    for(int32_t i = g->nDigits - 1; i >= last; i--)
    {
        uint32_t shift = (uint32_t)(2 * i - (odd ? 1 : 0));
        uint32_t digit = (uint32_t)((g->morton >> shift) & 3u);
        uint64_t higher = g->morton >> (shift + 2u);
        uint32_t p = (uint32_t)((mix_bits(higher ^ (uint64_t)mixer) >> 24) % 24u);
        digit = g_perm[p][digit];
        idx |= (uint64_t)digit << shift;
    }
    if(odd)
    {
        uint32_t digit = (uint32_t)(g->morton & 1u);
        idx |= (uint64_t)(digit ^ (uint32_t)(mix_bits((g->morton >> 1) ^ (uint64_t)mixer) & 1u));
    }
    return idx;
}

static uint64_t morton2(uint32_t x, uint32_t y)
{
    uint64_t r = 0;
    for(int b = 0; b < 32; b++)
        r |= ((uint64_t)((x >> b) & 1u) << (2 * b)) | ((uint64_t)((y >> b) & 1u) << (2 * b + 1));
    return r;
}

uint32_t orc_zs_res_max_bits(uint32_t width, uint32_t height)
{
    uint32_t m = width > height ? width : height;
    uint32_t p = (m <= 1u) ? 1u : (1u << bit_width32(m - 1u));
    return bit_width32(p) - 1u;
}

void orc_zs_seeds(uint32_t width, uint32_t height, uint64_t seed, uint32_t* out)
{
    orc_mt19937((uint32_t)((seed >> 32) ^ (seed & 0xFFFFFFFFull)), width * height, out);
}

int orc_zs_generate(uint32_t width, uint32_t height, const uint32_t* seeds, uint32_t initialMaxSpp,
                    uint32_t sampleIndex, uint32_t dimStart, uint64_t requests, uint32_t requestCount,
                    uint32_t* out)
{
    if(!seeds || !out || initialMaxSpp == 0 || requestCount > 32) return -1;
    zs_init();
    const uint32_t resBits = orc_zs_res_max_bits(width, height);
    const uint32_t n = width * height;
    for(uint32_t i = 0; i < n; i++)
    {
        zs_gen g = zs_make(morton2(i % width, i / width), sampleIndex, seeds[i], initialMaxSpp, resBits);
        uint32_t o = 0;
        for(uint32_t r = 0; r < requestCount; r++)
        {
            const uint32_t d = (uint32_t)((requests >> (2 * r)) & 3u);
            const uint32_t dim = dimStart + o;
            if(d == 0) continue;
            const uint64_t a = zs_index(&g, dim);
            const uint64_t h = hash_dim_seed(dim, g.seed);
            if(d == 1)
                out[i + (size_t)n * o] = owen_fast(mat_mul(0, a), (uint32_t)h);
            else if(d == 2)
            {
                out[i + (size_t)n * o] = owen_fast(mat_mul(0, a), (uint32_t)(h & 0xFFFFFFFFull));
                out[i + (size_t)n * (o + 1)] = owen_fast(mat_mul(1, a), (uint32_t)(h >> 32));
            }
            else
            {
                const uint64_t M = (1ull << 21) - 1ull;
                out[i + (size_t)n * o] = owen_fast(mat_mul(0, a), (uint32_t)(h & M));
                out[i + (size_t)n * (o + 1)] = owen_fast(mat_mul(1, a), (uint32_t)((h >> 21) & M));
                out[i + (size_t)n * (o + 2)] = owen_fast(mat_mul(2, a), (uint32_t)(h >> 42));
            }
            o += d;
        }
    }
    return 0;
}

uint32_t orc_zs_number(uint32_t px, uint32_t py, uint32_t seed, uint32_t sampleIndex, uint32_t initialMaxSpp,
                       uint32_t resMaxBits, uint32_t dim, uint32_t size, uint32_t comp, int owen)
{
    zs_init();
    zs_gen g = zs_make(morton2(px, py), sampleIndex, seed, initialMaxSpp, resMaxBits);
    const uint64_t a = zs_index(&g, dim);
    const uint64_t h = hash_dim_seed(dim, seed);
    uint32_t scr;
    if(size == 1u) scr = (uint32_t)h;
    else if(size == 2u) scr = comp ? (uint32_t)(h >> 32) : (uint32_t)h;
    else scr = (comp == 0u) ? (uint32_t)(h & 0x1FFFFFull)
             : (comp == 1u) ? (uint32_t)((h >> 21) & 0x1FFFFFull) : (uint32_t)(h >> 42);
    const uint32_t v = owen_fast(mat_mul((int)comp, a), scr);
    return owen ? brev32(v) : v;
}

/* ---- independent group: PCG32 ------------------------------------------ */
#define PCG_MULT 747796405u
#define PCG_INC  2891336453u

static uint32_t pcg_step(uint32_t r) { return r * PCG_MULT + PCG_INC; }

uint32_t orc_pcg32_state(uint32_t seed)
{
    return pcg_step(pcg_step(0u) + seed);
}

uint32_t orc_pcg32_advance(uint32_t state, uint32_t delta)
{
    /* Step^delta as one affine map a*x + c, composed from the maps of
     * Step^(2^i) for the set bits of delta. */
    uint32_t a = 1u, c = 0u, m = PCG_MULT, k = PCG_INC;
    for(; delta; delta >>= 1)
    {
        if(delta & 1u) { a *= m; c = c * m + k; }
        k = (m + 1u) * k;
        m *= m;
    }
    return a * state + c;
}

uint32_t orc_pcg32_permute(uint32_t s)
{
    const uint32_t x = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    return (x >> 22) ^ x;
}

void orc_pcg32_numbers(const uint32_t* seeds, const uint32_t* delta, uint32_t count, uint32_t* out)
{
    for(uint32_t i = 0; i < count; i++)
        out[i] = orc_pcg32_permute(orc_pcg32_advance(orc_pcg32_state(seeds[i]), delta[i]));
}
