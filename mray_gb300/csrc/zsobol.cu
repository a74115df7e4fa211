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
// The device functions are in zsobol.cuh (shared with the path tracer).
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <cuda_runtime.h>

#include "mray_gb300.h"
#include "zsobol.cuh"

namespace mrg {
mrg_status set_error(mrg_status s, const std::string& msg);
}

namespace {

__constant__ __align__(16) uint32_t c_zs[mrg::kZsTableWords];

void sobol_dim(uint32_t* col, int s, uint32_t a, const uint64_t* m0)
{
    uint64_t m[mrg::kZsWidth + 1];
    for(int k = 1; k <= s; k++) m[k] = m0[k - 1];
    for(int k = s + 1; k <= mrg::kZsWidth; k++)
    {
        uint64_t v = m[k - s] ^ (m[k - s] << s);
        for(int j = 1; j < s; j++)
            if((a >> (s - 1 - j)) & 1u) v ^= m[k - j] << j;
        m[k] = v;
    }
    for(int k = 1; k <= mrg::kZsWidth; k++)
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

__global__ void k_zsobol(uint32_t width, uint32_t n, const uint32_t* __restrict__ seeds, uint32_t initialMaxSpp,
                         uint32_t resMaxBits, uint32_t sampleIndex, uint32_t dimStart, uint64_t requests,
                         uint32_t requestCount, uint32_t* __restrict__ out)
{
    const uint32_t* mat = c_zs;
    const uint64_t* perm = reinterpret_cast<const uint64_t*>(c_zs + 3 * mrg::kZsWidth);
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const mrg::ZsGen g = mrg::zs_make(i % width, i / width, seeds[i], sampleIndex, initialMaxSpp, resMaxBits);
        uint32_t o = 0;
        for(uint32_t r = 0; r < requestCount; r++)
        {
            const uint32_t d = (uint32_t)((requests >> (2 * r)) & 3u);
            if(d == 0u) continue;
            const uint32_t dim = dimStart + o;
            for(uint32_t c = 0; c < d; c++)
                out[i + (size_t)n * (o + c)] = mrg::zs_number(g, mat, perm, dim, d, c);
            o += d;
        }
    }
}

uint32_t bit_width(uint32_t v) { return v ? 32u - (uint32_t)__builtin_clz(v) : 0u; }

} // namespace

namespace mrg {

void zsobol_tables(uint32_t* out)
{
    std::memset(out, 0, sizeof(uint32_t) * kZsTableWords);
    for(int k = 0; k < kZsWidth; k++) out[k] = (k < 32) ? (0x80000000u >> k) : 0u;
    const uint64_t m1[1] = { 1 }, m2[2] = { 1, 3 };
    sobol_dim(out + kZsWidth, 1, 0u, m1);
    sobol_dim(out + 2 * kZsWidth, 2, 1u, m2);
    uint8_t a[4] = { 0, 1, 2, 3 }, p[24][4];
    int n = 0;
    perms(a, 0, n, p);
    uint64_t packed[4] = { 0, 0, 0, 0 };
    for(int d = 0; d < 4; d++)
        for(int q = 0; q < 24; q++) packed[d] |= (uint64_t)p[q][d] << (2 * q);
    std::memcpy(out + 3 * kZsWidth, packed, sizeof(packed));
}

} // namespace mrg

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
    static bool uploaded[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if(e == cudaSuccess && dev >= 0 && dev < 64 && !uploaded[dev])
    {
        uint32_t t[mrg::kZsTableWords];
        mrg::zsobol_tables(t);
        e = cudaMemcpyToSymbol(c_zs, t, sizeof(t));
        uploaded[dev] = (e == cudaSuccess);
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
