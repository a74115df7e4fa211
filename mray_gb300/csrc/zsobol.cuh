// zsobol.cuh -- device functions of MRay's ZSobol generator, shared by the
// standalone generator (zsobol.cu) and the path tracer's sampler (pt.cu).
//
// Restates Source/Tracer/Random.cu: ScambleOwenFast (141-150), MixBits
// (156-165), BitwiseMatrixMult (249-263), ZSobol::SampleIndex (266-342),
// ZSobol::ZSobol (356-383), Next / Next2D / Next3D (385-420); and
// HashPCG64::Hash (Source/Tracer/Random.h:603-633).  `mat` holds the three
// 52-column Sobol matrices, `perm[d]` element d of the 24 digit permutations
// (2 bits each).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mrg {

constexpr int kZsWidth = 52;
constexpr int kZsTableWords = 3 * kZsWidth + 8;   // matrices, then 4 x uint64 permutations

// Host: fills the tables (kZsTableWords words) from the Sobol recurrence and
// the swap enumeration of the permutations of {0, 1, 2, 3}.
void zsobol_tables(uint32_t* out);

#if defined(__CUDACC__)

__device__ __forceinline__ uint64_t zs_mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7FB5D329728EA185ull;
    v ^= v >> 27;
    v *= 0x81DADEF4BC2DD44Dull;
    v ^= v >> 33;
    return v;
}

__device__ __forceinline__ uint64_t zs_hash_pcg64(uint64_t v)
{
    const uint64_t s = v * 6364136223846793005ull + 1442695040888963407ull;
    uint64_t word = (s >> ((s >> 59) + 5u)) ^ s;
    word *= 12605985483714917081ull;
    return (word >> 43) ^ word;
}

__device__ __forceinline__ uint32_t zs_owen_fast(uint32_t v, uint32_t seed)
{
    v = __brev(v);
    v ^= v * 0x3A20ADEAu;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526C56u;
    v ^= v * 0x53A22864u;
    return v;
}

__device__ __forceinline__ uint32_t zs_mat_mul(const uint32_t* mat, int d, uint64_t a)
{
    uint32_t r = 0;
    for(int i = 0; i < kZsWidth && a != 0; i++, a >>= 1)
        if(a & 1u) r ^= mat[d * kZsWidth + i];
    return r;
}

__device__ __forceinline__ uint64_t zs_expand2(uint32_t v)
{
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

struct ZsGen
{
    uint64_t morton;
    uint32_t log2Spp;
    int32_t  nDigits;
    uint32_t seed;
};

__device__ __forceinline__ ZsGen zs_make(uint32_t px, uint32_t py, uint32_t seed, uint32_t sampleIndex,
                                         uint32_t initialMaxSpp, uint32_t resMaxBits)
{
    ZsGen g;
    uint32_t local = sampleIndex, maxSpp = initialMaxSpp;
    for(uint32_t r = 0; r < 32u; r++)
    {
        const uint32_t cur = initialMaxSpp << r;
        if(local < cur) break;
        local -= cur;
        maxSpp <<= 1;
    }
    g.log2Spp = 31u - __clz(maxSpp);
    g.nDigits = (int32_t)(resMaxBits + (g.log2Spp + 1u) / 2u);
    g.morton = ((zs_expand2(px) | (zs_expand2(py) << 1)) << g.log2Spp) | local;
    g.seed = seed;
    return g;
}

__device__ __forceinline__ uint64_t zs_sample_index(const ZsGen& g, const uint64_t* perm, uint32_t dim)
{
    const uint32_t mixer = 0x55555555u * dim;
    const bool odd = (g.log2Spp & 1u) != 0u;
    uint64_t a = 0;
    for(int32_t q = g.nDigits - 1; q >= (odd ? 1 : 0); q--)
    {
        const uint32_t shift = (uint32_t)(2 * q - (odd ? 1 : 0));
        const uint32_t digit = (uint32_t)((g.morton >> shift) & 3u);
        const uint32_t p = (uint32_t)((zs_mix_bits((g.morton >> (shift + 2u)) ^ (uint64_t)mixer) >> 24) % 24u);
        a |= ((perm[digit] >> (2u * p)) & 3ull) << shift;
    }
    if(odd) a |= (g.morton & 1ull) ^ (zs_mix_bits((g.morton >> 1) ^ (uint64_t)mixer) & 1ull);
    return a;
}

__device__ __forceinline__ uint64_t zs_hash(uint32_t dim, uint32_t seed)
{
    return zs_hash_pcg64((uint64_t)seed + zs_hash_pcg64((uint64_t)dim));
}

// Component `comp` of the `size`-number request at dimension `dim`.  With
// `owen` the scrambled value is bit-reversed back (the Laine-Karras form of
// Owen scrambling, which keeps the Sobol points' stratification); MRay's
// ScambleOwenFast leaves it reversed.
__device__ __forceinline__ uint32_t zs_number(const ZsGen& g, const uint32_t* mat, const uint64_t* perm,
                                              uint32_t dim, uint32_t size, uint32_t comp, bool owen = false)
{
    const uint64_t a = zs_sample_index(g, perm, dim);
    const uint64_t h = zs_hash(dim, g.seed);
    uint32_t scr;
    if(size == 1u) scr = (uint32_t)h;
    else if(size == 2u) scr = comp ? (uint32_t)(h >> 32) : (uint32_t)h;
    else scr = (comp == 0u) ? (uint32_t)(h & 0x1FFFFFull)
             : (comp == 1u) ? (uint32_t)((h >> 21) & 0x1FFFFFull) : (uint32_t)(h >> 42);
    const uint32_t v = zs_owen_fast(zs_mat_mul(mat, (int)comp, a), scr);
    return owen ? __brev(v) : v;
}

// Components 0 .. size-1 of the request at `dim` (sample index and hash
// computed once); each equals zs_number's result for that component.
__device__ __forceinline__ void zs_numbers(const ZsGen& g, const uint32_t* mat, const uint64_t* perm, uint32_t dim,
                                           uint32_t size, uint32_t* out, bool owen = false)
{
    const uint64_t a = zs_sample_index(g, perm, dim);
    const uint64_t h = zs_hash(dim, g.seed);
    for(uint32_t comp = 0; comp < size; comp++)
    {
        uint32_t scr;
        if(size == 1u) scr = (uint32_t)h;
        else if(size == 2u) scr = comp ? (uint32_t)(h >> 32) : (uint32_t)h;
        else scr = (comp == 0u) ? (uint32_t)(h & 0x1FFFFFull)
                 : (comp == 1u) ? (uint32_t)((h >> 21) & 0x1FFFFFull) : (uint32_t)(h >> 42);
        const uint32_t v = zs_owen_fast(zs_mat_mul(mat, (int)comp, a), scr);
        out[comp] = owen ? __brev(v) : v;
    }
}

// RNGFunctions::ToFloat01<float, uint32_t> (Source/Tracer/Random.h:100-119).
__device__ __forceinline__ float zs_to_float01(uint32_t v)
{
    return fminf(__fmul_rn(__uint2float_rn(v), 2.3283064365386963e-10f), __uint_as_float(0x3F7FFFFFu));
}

#endif // __CUDACC__

} // namespace mrg
