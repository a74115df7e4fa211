// zsobol.cu -- MRay's ZSobol random-number group on the GPU.
//
// Restates, for one sample of every pixel of a width x height image:
//   RNGGroupZSobol seeds          Source/Tracer/Random.cu:1149-1230 (std::mt19937(seed32))
//   ZSobol::ZSobol                Source/Tracer/Random.cu:356-383  (sample rotation, digits)
//   ZSobol::SampleIndex           Source/Tracer/Random.cu:266-342  (base-4 digit permutations)
//   ZSobol::Next / Next2D / Next3D Source/Tracer/Random.cu:385-420
//   BitwiseMatrixMult, ScambleOwenFast, MixBits  Source/Tracer/Random.cu:141-165, 249-263
//   HashPCG64::Hash               Source/Tracer/Random.h:603-633
//   GenerateRNFromList            Source/Tracer/Random.cu:426-470 (strided output)
// The Sobol matrices (dims 0-2) are built from the Sobol recurrence and the 24
// digit permutations from the swap-recursive enumeration of {0, 1, 2, 3}.
// One thread per pixel; integer arithmetic only, so results are bit-exact.
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <cuda_runtime.h>

#include "mray_gb300.h"

namespace mrg {
mrg_status set_error(mrg_status s, const std::string& msg);
}

namespace {

constexpr int kZsWidth = 52;

struct ZsTables
{
    uint32_t mat[3][kZsWidth];
    uint64_t perm[4];   // perm[d] bits 2p..2p+1: element d of permutation p
};

__constant__ ZsTables c_zs;

void sobol_dim(uint32_t* col, int s, uint32_t a, const uint64_t* m0)
{
    uint64_t m[kZsWidth + 1];
    for(int k = 1; k <= s; k++) m[k] = m0[k - 1];
    for(int k = s + 1; k <= kZsWidth; k++)
    {
        uint64_t v = m[k - s] ^ (m[k - s] << s);
        for(int j = 1; j < s; j++)
            if((a >> (s - 1 - j)) & 1u) v ^= m[k - j] << j;
        m[k] = v;
    }
    for(int k = 1; k <= kZsWidth; k++)
        col[k - 1] = (k <= 32) ? (uint32_t)(m[k] << (32 - k)) : (uint32_t)(m[k] >> (k - 32));
}

void perms(uint8_t* a, int k, int& n, uint8_t (*out)[4])
{
    if(k == 4) { std::memcpy(out[n++], a, 4); return; }
    for(int i = k; i < 4; i++)
    {
        std::swap(a[k], a[i]);
        perms(a, k + 1, n, out);
        std::swap(a[k], a[i]);
    }
}

ZsTables make_tables()
{
    ZsTables t{};
    for(int k = 0; k < kZsWidth; k++) t.mat[0][k] = (k < 32) ? (0x80000000u >> k) : 0u;
    const uint64_t m1[1] = { 1 }, m2[2] = { 1, 3 };
    sobol_dim(t.mat[1], 1, 0u, m1);
    sobol_dim(t.mat[2], 2, 1u, m2);
    uint8_t a[4] = { 0, 1, 2, 3 }, p[24][4];
    int n = 0;
    perms(a, 0, n, p);
    for(int d = 0; d < 4; d++)
        for(int q = 0; q < 24; q++) t.perm[d] |= (uint64_t)p[q][d] << (2 * q);
    return t;
}

__device__ __forceinline__ uint64_t mix_bits(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7FB5D329728EA185ull;
    v ^= v >> 27;
    v *= 0x81DADEF4BC2DD44Dull;
    v ^= v >> 33;
    return v;
}

__device__ __forceinline__ uint64_t hash_pcg64(uint64_t v)
{
    const uint64_t s = v * 6364136223846793005ull + 1442695040888963407ull;
    uint64_t word = (s >> ((s >> 59) + 5u)) ^ s;
    word *= 12605985483714917081ull;
    return (word >> 43) ^ word;
}

__device__ __forceinline__ uint32_t owen_fast(uint32_t v, uint32_t seed)
{
    v = __brev(v);
    v ^= v * 0x3A20ADEAu;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526C56u;
    v ^= v * 0x53A22864u;
    return v;
}

__device__ __forceinline__ uint32_t mat_mul(int d, uint64_t a)
{
    uint32_t r = 0;
    for(int i = 0; i < kZsWidth && a != 0; i++, a >>= 1)
        if(a & 1u) r ^= c_zs.mat[d][i];
    return r;
}

__device__ __forceinline__ uint64_t expand2(uint32_t v)
{
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

__global__ void k_zsobol(uint32_t width, uint32_t n, const uint32_t* __restrict__ seeds, uint32_t initialMaxSpp,
                         uint32_t resMaxBits, uint32_t sampleIndex, uint32_t dimStart, uint64_t requests,
                         uint32_t requestCount, uint32_t* __restrict__ out)
{
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t seed = seeds[i];
        const uint64_t pixelMorton = expand2(i % width) | (expand2(i / width) << 1);
        // sample rotation: indices past the initial count fall in doubled blocks
        uint32_t local = sampleIndex, maxSpp = initialMaxSpp;
        for(uint32_t r = 0; r < 32u; r++)
        {
            const uint32_t cur = initialMaxSpp << r;
            if(local < cur) break;
            local -= cur;
            maxSpp <<= 1;
        }
        const uint32_t log2Spp = 31u - __clz(maxSpp);
        const int32_t nDigits = (int32_t)(resMaxBits + (log2Spp + 1u) / 2u);
        const uint64_t morton = (pixelMorton << log2Spp) | local;
        const bool odd = (log2Spp & 1u) != 0u;
        uint32_t o = 0;
        for(uint32_t r = 0; r < requestCount; r++)
        {
            const uint32_t d = (uint32_t)((requests >> (2 * r)) & 3u);
            if(d == 0u) continue;
            const uint32_t dim = dimStart + o;
            const uint32_t mixer = 0x55555555u * dim;
            uint64_t a = 0;
            for(int32_t q = nDigits - 1; q >= (odd ? 1 : 0); q--)
            {
                const uint32_t shift = (uint32_t)(2 * q - (odd ? 1 : 0));
                const uint32_t digit = (uint32_t)((morton >> shift) & 3u);
                const uint32_t p = (uint32_t)((mix_bits((morton >> (shift + 2u)) ^ (uint64_t)mixer) >> 24) % 24u);
                a |= ((c_zs.perm[digit] >> (2u * p)) & 3ull) << shift;
            }
            if(odd) a |= (morton & 1ull) ^ (mix_bits((morton >> 1) ^ (uint64_t)mixer) & 1ull);
            const uint64_t h = hash_pcg64((uint64_t)seed + hash_pcg64((uint64_t)dim));
            uint32_t* dst = out + i + (size_t)n * o;
            if(d == 1u) dst[0] = owen_fast(mat_mul(0, a), (uint32_t)h);
            else if(d == 2u)
            {
                dst[0] = owen_fast(mat_mul(0, a), (uint32_t)h);
                dst[n] = owen_fast(mat_mul(1, a), (uint32_t)(h >> 32));
            }
            else
            {
                const uint64_t M = (1ull << 21) - 1ull;
                dst[0] = owen_fast(mat_mul(0, a), (uint32_t)(h & M));
                dst[n] = owen_fast(mat_mul(1, a), (uint32_t)((h >> 21) & M));
                dst[2 * (size_t)n] = owen_fast(mat_mul(2, a), (uint32_t)(h >> 42));
            }
            o += d;
        }
    }
}

uint32_t bit_width(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

} // namespace

extern "C" {

mrg_status mrg_zsobol_seeds(uint32_t width, uint32_t height, uint64_t seed, uint32_t* h_seeds)
{
    if(!h_seeds || width == 0 || height == 0)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_zsobol_seeds: empty image or null pointer");
    std::mt19937 rng((uint32_t)((seed >> 32) ^ (seed & 0xFFFFFFFFull)));
    const size_t n = (size_t)width * height;
    for(size_t i = 0; i < n; i++) h_seeds[i] = (uint32_t)rng();
    return MRG_OK;
}

mrg_status mrg_zsobol_generate(uint32_t width, uint32_t height, const uint32_t* d_seeds, uint32_t initial_max_spp,
                               uint32_t sample_index, uint32_t dim_start, uint64_t requests,
                               uint32_t request_count, uint32_t* d_out, void* stream)
{
    if(!d_seeds || !d_out || width == 0 || height == 0 || initial_max_spp == 0 || request_count > 32u ||
       (uint64_t)width * height > 0xFFFFFFFFull)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_zsobol_generate: bad arguments");
    static bool uploaded = false;
    static int uploadedDevice = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if(e == cudaSuccess && (!uploaded || uploadedDevice != dev))
    {
        const ZsTables t = make_tables();
        e = cudaMemcpyToSymbol(c_zs, &t, sizeof(t));
        uploaded = (e == cudaSuccess);
        uploadedDevice = dev;
    }
    if(e != cudaSuccess) return mrg::set_error(MRG_ERR_CUDA, std::string("mrg_zsobol_generate: ") + cudaGetErrorString(e));
    const uint32_t m = width > height ? width : height;
    const uint32_t pow2 = (m <= 1u) ? 1u : (1u << bit_width(m - 1u));
    const uint32_t resMaxBits = bit_width(pow2) - 1u;
    const uint32_t n = width * height;
    const unsigned blocks = (n + 255u) / 256u;
    k_zsobol<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(width, n, d_seeds, initial_max_spp, resMaxBits,
                                                                   sample_index, dim_start, requests, request_count,
                                                                   d_out);
    e = cudaGetLastError();
    if(e != cudaSuccess) return mrg::set_error(MRG_ERR_CUDA, std::string("mrg_zsobol_generate: ") + cudaGetErrorString(e));
    return MRG_OK;
}

} // extern "C"
