// nrc.cu -- radiance cache kernels: multiresolution hash-grid encoding
// (Mueller et al. 2022, "Instant Neural Graphics Primitives"), a fully fused
// 64-wide MLP on BF16 tensor cores (Mueller et al. 2021, "Real-time Neural
// Radiance Caching for Path Tracing"), its backward pass, weight gradients
// and Adam.  No reference counterpart: MRay has no learned cache.
//
// The MLP runs one warp per 16 samples: a layer is 4 (k) x 8 (n) BF16
// mma.m16n8k16 tiles with FP32 accumulation, and the accumulator fragment of
// one layer is, register for register, the A fragment of the next (the row /
// column ownership of m16n8 C tiles matches m16k16 A tiles), so activations
// never leave registers between layers.  Weights live in shared memory with
// rows padded to 72 elements (conflict-free fragment loads).
#include "mrg_nrc.h"
#include "mrg_launch.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace mrg {

namespace {

constexpr int kPad = 72;                      // padded row of 64 bf16
constexpr int kPadT4 = 24;                    // padded row of the output layer's W^T (16 bf16)
constexpr int kHiddenRows = kNrcHidden * kNrcWidth;   // rows of the hidden weight matrices
constexpr int kActs = kNrcHidden + 1;         // stored activations per training sample: x0, a1 ..
constexpr int kG16Row = kNrcLayers * kNrcWidth;  // bf16 per sample of the gradient rows
static_assert(kActs == kNrcLayers, "activation and gradient rows share one tensor-map shape");

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_to_f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t lds32(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// ---------------------------------------------------------------------------
// Encoding
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t grid_index(const NrcGrid& G, uint32_t l, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t mask = (1u << G.log2Table) - 1u;
    if(G.dense[l])
    {
        const uint32_t r = G.res[l];
        return (x + y * r + z * r * r) & mask;
    }
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & mask;
}

struct LevelPos
{
    uint32_t x, y, z;
    float fx, fy, fz;
};

__device__ __forceinline__ LevelPos level_pos(const NrcGrid& G, uint32_t l, float ux, float uy, float uz)
{
    const float s = G.scale[l];
    const float px = ux * s + 0.5f, py = uy * s + 0.5f, pz = uz * s + 0.5f;
    const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
    LevelPos p;
    p.x = (uint32_t)bx; p.y = (uint32_t)by; p.z = (uint32_t)bz;
    p.fx = px - bx; p.fy = py - by; p.fz = pz - bz;
    return p;
}

__device__ __forceinline__ void normalized_pos(const NrcGrid& G, float4 in0, float& ux, float& uy, float& uz)
{
    ux = fminf(fmaxf((in0.x - G.aabbMin[0]) * G.aabbInv[0], 0.0f), 1.0f);
    uy = fminf(fmaxf((in0.y - G.aabbMin[1]) * G.aabbInv[1], 0.0f), 1.0f);
    uz = fminf(fmaxf((in0.z - G.aabbMin[2]) * G.aabbInv[2], 0.0f), 1.0f);
}

// Real spherical harmonics up to degree 3 (16 coefficients) of a unit vector.
__device__ __forceinline__ void sh16(float x, float y, float z, float* o)
{
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (-3.0f * xx + yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * zz);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * zz);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (-xx + 3.0f * yy);
}

// Writes the 64 input features of sample `s` (valid) into the warp's bf16
// tile: lane (s, half) encodes levels [8 half, 8 half + 8) and half 0 the
// direction harmonics, half 1 the normal, albedo, roughness and constants.
__device__ void encode_sample(const NrcState& S, const float4* in, bool valid, uint32_t half, uint16_t* row)
{
    const NrcGrid& G = S.grid;
    float4 i0 = make_float4(0, 0, 0, 0), i1 = i0, i2 = i0, i3 = i0;
    if(valid) { i0 = in[0]; i1 = in[1]; i2 = in[2]; i3 = in[3]; }
    float ux, uy, uz;
    normalized_pos(G, i0, ux, uy, uz);
    const uint32_t T = 1u << G.log2Table;
#pragma unroll 2
    for(uint32_t q = 0; q < 8; q++)
    {
        const uint32_t l = 8u * half + q;
        float f0 = 0.0f, f1 = 0.0f;
        if(valid && l < G.levels)
        {
            const LevelPos p = level_pos(G, l, ux, uy, uz);
            const __half2* tab = reinterpret_cast<const __half2*>(S.t16) + (size_t)l * T;
#pragma unroll
            for(uint32_t c = 0; c < 8; c++)
            {
                const uint32_t cx = c & 1u, cy = (c >> 1) & 1u, cz = (c >> 2) & 1u;
                const float w = (cx ? p.fx : 1.0f - p.fx) * (cy ? p.fy : 1.0f - p.fy) * (cz ? p.fz : 1.0f - p.fz);
                const float2 v = __half22float2(__ldg(tab + grid_index(G, l, p.x + cx, p.y + cy, p.z + cz)));
                f0 += w * v.x;
                f1 += w * v.y;
            }
        }
        *reinterpret_cast<uint32_t*>(row + 2 * l) = pack_bf16(f0, f1);
    }
    float v[16];
    if(half == 0u)
    {
        sh16(i1.x, i1.y, i1.z, v);
        if(!valid) for(int k = 0; k < 16; k++) v[k] = 0.0f;
#pragma unroll
        for(int k = 0; k < 16; k += 2) *reinterpret_cast<uint32_t*>(row + 32 + k) = pack_bf16(v[k], v[k + 1]);
    }
    else
    {
        v[0] = (i2.x + 1.0f) * 0.5f; v[1] = (i2.y + 1.0f) * 0.5f; v[2] = (i2.z + 1.0f) * 0.5f;
        v[3] = i3.x; v[4] = i3.y; v[5] = i3.z; v[6] = i0.w; v[7] = 1.0f;
        for(int k = 8; k < 16; k++) v[k] = 0.0f;
        if(!valid) for(int k = 0; k < 16; k++) v[k] = 0.0f;
#pragma unroll
        for(int k = 0; k < 16; k += 2) *reinterpret_cast<uint32_t*>(row + 48 + k) = pack_bf16(v[k], v[k + 1]);
    }
}

// ---------------------------------------------------------------------------
// Forward: inference (out) or training (stores activations and outputs)
// ---------------------------------------------------------------------------
// WARPS warps per CTA share one shared-memory copy of the weights; more warps
// per CTA keep more hash-grid gathers in flight per SM.
template<bool TRAIN, bool LIST, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_nrc_forward(NrcState S, const float4* __restrict__ inputs, const uint32_t* __restrict__ list,
              const uint32_t* nDevice, uint32_t nMax, float4* __restrict__ out)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t* sW = reinterpret_cast<uint16_t*>(smem);                       // (256 + 16) x kPad
    uint16_t* sX = sW + (kHiddenRows + kNrcOut) * kPad;                      // WARPS x 16 x kPad
    float* sO = reinterpret_cast<float*>(sX + WARPS * 16 * kPad);            // WARPS x 16 x 4
    for(uint32_t i = threadIdx.x; i < (uint32_t)kNrcWeightCount; i += WARPS * 32)
        sW[(i / kNrcWidth) * kPad + (i % kNrcWidth)] = S.w16[i];
    __syncthreads();
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    uint16_t* xw = sX + warp * 16 * kPad;
    float* ow = sO + warp * 64;
    for(uint32_t base = (blockIdx.x * WARPS + warp) * 16u; base < n; base += gridDim.x * WARPS * 16u)
    {
        // ---- encode 16 samples ----
        {
            const uint32_t s = lane & 15u, half = lane >> 4;
            const uint32_t e = base + s;
            const bool valid = e < n;
            const uint32_t src = valid ? (LIST ? list[e] : e) : 0u;
            encode_sample(S, inputs + (size_t)src * 4, valid, half, xw + s * kPad);
        }
        __syncwarp();
        uint32_t a[4][4];
#pragma unroll
        for(int kt = 0; kt < 4; kt++)
        {
            a[kt][0] = lds32(xw + g * kPad + 16 * kt + 2 * t);
            a[kt][1] = lds32(xw + (g + 8) * kPad + 16 * kt + 2 * t);
            a[kt][2] = lds32(xw + g * kPad + 16 * kt + 8 + 2 * t);
            a[kt][3] = lds32(xw + (g + 8) * kPad + 16 * kt + 8 + 2 * t);
        }
        if(TRAIN)
        {
            // x0 rows as the fragments hold them
#pragma unroll
            for(int kt = 0; kt < 4; kt++)
            {
                const uint32_t r0 = base + g, r1 = base + g + 8;
                uint32_t* A = reinterpret_cast<uint32_t*>(S.acts);
                if(r0 < n)
                {
                    A[((size_t)r0 * kActs * kNrcWidth + 16 * kt + 2 * t) / 2] = a[kt][0];
                    A[((size_t)r0 * kActs * kNrcWidth + 16 * kt + 8 + 2 * t) / 2] = a[kt][2];
                }
                if(r1 < n)
                {
                    A[((size_t)r1 * kActs * kNrcWidth + 16 * kt + 2 * t) / 2] = a[kt][1];
                    A[((size_t)r1 * kActs * kNrcWidth + 16 * kt + 8 + 2 * t) / 2] = a[kt][3];
                }
            }
        }
        __syncwarp();
        // ---- hidden layers ----
#pragma unroll 1
        for(int layer = 0; layer < kNrcHidden; layer++)
        {
            const uint16_t* W = sW + layer * kNrcWidth * kPad;
            float acc[8][4];
#pragma unroll
            for(int nt = 0; nt < 8; nt++)
            {
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
                for(int kt = 0; kt < 4; kt++)
                {
                    const uint16_t* wr = W + (8 * nt + g) * kPad + 16 * kt + 2 * t;
                    mma_bf16(acc[nt], a[kt], lds32(wr), lds32(wr + 8));
                }
            }
#pragma unroll
            for(int kt = 0; kt < 4; kt++)
            {
                a[kt][0] = pack_bf16(fmaxf(acc[2 * kt][0], 0.0f), fmaxf(acc[2 * kt][1], 0.0f));
                a[kt][1] = pack_bf16(fmaxf(acc[2 * kt][2], 0.0f), fmaxf(acc[2 * kt][3], 0.0f));
                a[kt][2] = pack_bf16(fmaxf(acc[2 * kt + 1][0], 0.0f), fmaxf(acc[2 * kt + 1][1], 0.0f));
                a[kt][3] = pack_bf16(fmaxf(acc[2 * kt + 1][2], 0.0f), fmaxf(acc[2 * kt + 1][3], 0.0f));
            }
            if(TRAIN)
            {
                uint32_t* A = reinterpret_cast<uint32_t*>(S.acts);
                const size_t off = (size_t)(layer + 1) * kNrcWidth;
#pragma unroll
                for(int kt = 0; kt < 4; kt++)
                {
                    const uint32_t r0 = base + g, r1 = base + g + 8;
                    if(r0 < n)
                    {
                        A[((size_t)r0 * kActs * kNrcWidth + off + 16 * kt + 2 * t) / 2] = a[kt][0];
                        A[((size_t)r0 * kActs * kNrcWidth + off + 16 * kt + 8 + 2 * t) / 2] = a[kt][2];
                    }
                    if(r1 < n)
                    {
                        A[((size_t)r1 * kActs * kNrcWidth + off + 16 * kt + 2 * t) / 2] = a[kt][1];
                        A[((size_t)r1 * kActs * kNrcWidth + off + 16 * kt + 8 + 2 * t) / 2] = a[kt][3];
                    }
                }
            }
        }
        // ---- output layer (16 rows; the first 3 are RGB) ----
        float o[2][4];
#pragma unroll
        for(int nt = 0; nt < 2; nt++)
        {
            o[nt][0] = o[nt][1] = o[nt][2] = o[nt][3] = 0.0f;
#pragma unroll
            for(int kt = 0; kt < 4; kt++)
            {
                const uint16_t* wr = sW + (kHiddenRows + 8 * nt + g) * kPad + 16 * kt + 2 * t;
                mma_bf16(o[nt], a[kt], lds32(wr), lds32(wr + 8));
            }
        }
        // columns 0..3 of rows g, g + 8 sit in n-tile 0 with t in {0, 1}
        if(t < 2u)
        {
            ow[g * 4 + 2 * t] = o[0][0];
            ow[g * 4 + 2 * t + 1] = o[0][1];
            ow[(g + 8) * 4 + 2 * t] = o[0][2];
            ow[(g + 8) * 4 + 2 * t + 1] = o[0][3];
        }
        __syncwarp();
        if(lane < 16u && base + lane < n)
        {
            const uint32_t e = base + lane;
            const float4 r = make_float4(ow[lane * 4], ow[lane * 4 + 1], ow[lane * 4 + 2], 0.0f);
            out[LIST ? list[e] : e] = r;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Backward: relative L2 loss, deltas through the MLP, hash-grid scatter
// ---------------------------------------------------------------------------
template<int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_nrc_backward(NrcState S, const float4* __restrict__ inputs, const float4* __restrict__ y,
               const float4* __restrict__ targets, const uint32_t* nDevice, uint32_t nMax)
{
    extern __shared__ __align__(16) uint8_t smem[];
    // transposed weights: hidden W0^T..W4^T [64 in][64 out], output W5^T [64 in][16 out]
    uint16_t* sT = reinterpret_cast<uint16_t*>(smem);                        // 4 x 64 x kPad
    uint16_t* sT4 = sT + kHiddenRows * kPad;                                  // 64 x kPadT4
    float* sG = reinterpret_cast<float*>(sT4 + kNrcWidth * kPadT4);           // WARPS x 16 x 33
    for(uint32_t i = threadIdx.x; i < (uint32_t)(kHiddenRows * kNrcWidth); i += WARPS * 32)
    {
        const uint32_t layer = i / (kNrcWidth * kNrcWidth), r = (i / kNrcWidth) % kNrcWidth, c = i % kNrcWidth;
        // W[layer][out = r][in = c] -> T[layer][in = c][out = r]
        sT[(layer * kNrcWidth + c) * kPad + r] = S.w16[i];
    }
    for(uint32_t i = threadIdx.x; i < (uint32_t)(kNrcOut * kNrcWidth); i += WARPS * 32)
    {
        const uint32_t r = i / kNrcWidth, c = i % kNrcWidth;
        sT4[c * kPadT4 + r] = S.w16[kHiddenRows * kNrcWidth + i];
    }
    __syncthreads();
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    if(n == 0u) return;
    const float invN = 1.0f / (float)n;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    float* gw = sG + warp * 16 * 33;
    float lossAcc = 0.0f;
    for(uint32_t base = (blockIdx.x * WARPS + warp) * 16u; base < n; base += gridDim.x * WARPS * 16u)
    {
        const uint32_t r0 = base + g, r1 = base + g + 8;
        const bool v0 = r0 < n, v1 = r1 < n;
        // ---- dLoss/dy for the 16 x 16 output tile (C layout), relative L2 ----
        float gy[2][4];
#pragma unroll
        for(int nt = 0; nt < 2; nt++)
            for(int q = 0; q < 4; q++) gy[nt][q] = 0.0f;
        if(t < 2u)
        {
            const float4 ya = v0 ? y[r0] : make_float4(0, 0, 0, 0), ta = v0 ? targets[r0] : make_float4(0, 0, 0, 0);
            const float4 yb = v1 ? y[r1] : make_float4(0, 0, 0, 0), tb = v1 ? targets[r1] : make_float4(0, 0, 0, 0);
            const float yav[3] = { ya.x, ya.y, ya.z }, tav[3] = { ta.x, ta.y, ta.z };
            const float ybv[3] = { yb.x, yb.y, yb.z }, tbv[3] = { tb.x, tb.y, tb.z };
#pragma unroll
            for(int j = 0; j < 2; j++)
            {
                const int c = 2 * (int)t + j;
                if(c < 3)
                {
                    if(v0)
                    {
                        const float d = yav[c] - tav[c], den = yav[c] * yav[c] + 0.01f;
                        gy[0][j] = 2.0f * d / den * invN;
                        lossAcc += d * d / den;
                    }
                    if(v1)
                    {
                        const float d = ybv[c] - tbv[c], den = ybv[c] * ybv[c] + 0.01f;
                        gy[0][2 + j] = 2.0f * d / den * invN;
                        lossAcc += d * d / den;
                    }
                }
            }
        }
        uint32_t a[4][4];
        a[0][0] = pack_bf16(gy[0][0], gy[0][1]);
        a[0][1] = pack_bf16(gy[0][2], gy[0][3]);
        a[0][2] = pack_bf16(gy[1][0], gy[1][1]);
        a[0][3] = pack_bf16(gy[1][2], gy[1][3]);
        // bf16 dL/dy rows for the output layer's dW = gy^T a5 (slot kNrcHidden, columns 0..15)
        uint32_t* G16 = reinterpret_cast<uint32_t*>(S.g16);
        if(v0) { G16[((size_t)r0 * kG16Row + kNrcHidden * kNrcWidth + 2 * t) / 2] = a[0][0];
                 G16[((size_t)r0 * kG16Row + kNrcHidden * kNrcWidth + 8 + 2 * t) / 2] = a[0][2]; }
        if(v1) { G16[((size_t)r1 * kG16Row + kNrcHidden * kNrcWidth + 2 * t) / 2] = a[0][1];
                 G16[((size_t)r1 * kG16Row + kNrcHidden * kNrcWidth + 8 + 2 * t) / 2] = a[0][3]; }
        // ---- g_a5 = gy W5 (k = 16) ----
        float acc[8][4];
#pragma unroll
        for(int nt = 0; nt < 8; nt++)
        {
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
            const uint16_t* wr = sT4 + (8 * nt + g) * kPadT4 + 2 * t;
            mma_bf16(acc[nt], a[0], lds32(wr), lds32(wr + 8));
        }
        const uint16_t* acts = S.acts;
#pragma unroll 1
        for(int layer = kNrcHidden - 1; layer >= 0; layer--)
        {
            // mask with the ReLU of activation a_{layer+1} (stored at index layer + 1)
            const size_t aoff = (size_t)(layer + 1) * kNrcWidth;
#pragma unroll
            for(int nt = 0; nt < 8; nt++)
            {
                const int c = 8 * nt + 2 * (int)t;
                float m0 = 0, m1 = 0, m2 = 0, m3 = 0;
                if(v0)
                {
                    const uint32_t p = *reinterpret_cast<const uint32_t*>(acts + (size_t)r0 * kActs * kNrcWidth + aoff + c);
                    m0 = bf16_to_f((uint16_t)(p & 0xFFFFu)) > 0.0f ? 1.0f : 0.0f;
                    m1 = bf16_to_f((uint16_t)(p >> 16)) > 0.0f ? 1.0f : 0.0f;
                }
                if(v1)
                {
                    const uint32_t p = *reinterpret_cast<const uint32_t*>(acts + (size_t)r1 * kActs * kNrcWidth + aoff + c);
                    m2 = bf16_to_f((uint16_t)(p & 0xFFFFu)) > 0.0f ? 1.0f : 0.0f;
                    m3 = bf16_to_f((uint16_t)(p >> 16)) > 0.0f ? 1.0f : 0.0f;
                }
                acc[nt][0] *= m0; acc[nt][1] *= m1; acc[nt][2] *= m2; acc[nt][3] *= m3;
            }
            // bf16 g_z{layer+1}: the A fragments of g_a_layer below and the rows of
            // dW_layer = g_z{layer+1}^T a_layer (slot `layer`)
#pragma unroll
            for(int kt = 0; kt < 4; kt++)
            {
                a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
                a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
                a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
                a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
                const size_t col = (size_t)layer * kNrcWidth + 16 * kt + 2 * t;
                if(v0) { G16[((size_t)r0 * kG16Row + col) / 2] = a[kt][0]; G16[((size_t)r0 * kG16Row + col + 8) / 2] = a[kt][2]; }
                if(v1) { G16[((size_t)r1 * kG16Row + col) / 2] = a[kt][1]; G16[((size_t)r1 * kG16Row + col + 8) / 2] = a[kt][3]; }
            }
            // g_a_layer = g_z{layer+1} W_layer; at layer 0 only the hash columns (0..31) are needed
            const uint16_t* T = sT + layer * kNrcWidth * kPad;
            const int nts = (layer == 0) ? 4 : 8;
#pragma unroll
            for(int nt = 0; nt < 8; nt++)
            {
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
                if(nt < nts)
                {
#pragma unroll
                    for(int kt = 0; kt < 4; kt++)
                    {
                        const uint16_t* wr = T + (8 * nt + g) * kPad + 16 * kt + 2 * t;
                        mma_bf16(acc[nt], a[kt], lds32(wr), lds32(wr + 8));
                    }
                }
            }
        }
        // ---- hash-grid scatter: dTable += w_corner * g_x0[hash feature] ----
#pragma unroll
        for(int nt = 0; nt < 4; nt++)
        {
            const int c = 8 * nt + 2 * (int)t;
            gw[g * 33 + c] = acc[nt][0]; gw[g * 33 + c + 1] = acc[nt][1];
            gw[(g + 8) * 33 + c] = acc[nt][2]; gw[(g + 8) * 33 + c + 1] = acc[nt][3];
        }
        __syncwarp();
        {
            const uint32_t s = lane & 15u, half = lane >> 4;
            const uint32_t e = base + s;
            if(e < n)
            {
                const NrcGrid& G = S.grid;
                float ux, uy, uz;
                normalized_pos(G, inputs[(size_t)e * 4], ux, uy, uz);
                const uint32_t T = 1u << G.log2Table;
                for(uint32_t q = 0; q < 8; q++)
                {
                    const uint32_t l = 8u * half + q;
                    if(l >= G.levels) break;
                    const float d0 = gw[s * 33 + 2 * l], d1 = gw[s * 33 + 2 * l + 1];
                    const LevelPos p = level_pos(G, l, ux, uy, uz);
                    float* tab = S.gT + (size_t)l * T * 2;
#pragma unroll
                    for(uint32_t c = 0; c < 8; c++)
                    {
                        const uint32_t cx = c & 1u, cy = (c >> 1) & 1u, cz = (c >> 2) & 1u;
                        const float w = (cx ? p.fx : 1.0f - p.fx) * (cy ? p.fy : 1.0f - p.fy) * (cz ? p.fz : 1.0f - p.fz);
                        const uint32_t idx = grid_index(G, l, p.x + cx, p.y + cy, p.z + cz);
                        atomicAdd(tab + 2 * (size_t)idx, w * d0);
                        atomicAdd(tab + 2 * (size_t)idx + 1, w * d1);
                    }
                }
            }
        }
        __syncwarp();
    }
    // loss (mean over samples of the summed relative L2 of RGB)
    for(int o = 16; o > 0; o >>= 1) lossAcc += __shfl_xor_sync(0xFFFFFFFFu, lossAcc, o);
    if(lane == 0u && lossAcc != 0.0f) atomicAdd(S.loss, lossAcc * invN);
}

// ---------------------------------------------------------------------------
// Weight gradients on the 5th-generation tensor cores:
//   dW_l[o][i] = sum_b G_l[b][o] A_l[b][i]
// for all six layers at once.  The batch is the reduction dimension: each CTA
// takes chunks of 128 samples (blockIdx.x, + gridDim.x, ...), and for every
// (chunk, layer) item a TMA pair brings the G_l and A_l tiles (128 rows x 64
// bf16, 128-byte swizzled) into one of four shared-memory stages.  One thread
// issues tcgen05.mma (kind::f16, M = 64 outputs o, N = 64 inputs i, K = 16
// samples, both operands MN-major) into the layer's 64 TMEM columns; a
// tcgen05.commit frees the stage.  At the end every warp reads its TMEM lane
// quarter (an M = 64 accumulator keeps row r in lane 32 (r / 16) + r % 16) and
// writes the CTA's partial sums; k_nrc_wgrad_sum adds the partials into gW in
// a fixed order, so the weight gradient is deterministic.
// Every mbarrier wait is bounded by a clock deadline; one that runs out sets
// kNrcWaitTimeout in S.err and the CTA drains its copies, frees its TMEM and
// returns.
// ---------------------------------------------------------------------------
constexpr uint32_t kWgRows = 128;                        // samples per chunk
constexpr uint32_t kWgStages = 4;
constexpr uint32_t kWgTileBytes = kWgRows * kNrcWidth * 2;   // 16 KB
constexpr uint32_t kWgStageBytes = 2 * kWgTileBytes;
constexpr size_t kWgSmem = (size_t)kWgStages * kWgStageBytes + 1024;   // + alignment to 1024 B
constexpr uint32_t kWgTmemCols = 512;                    // kNrcLayers x 64 fp32 columns, power of two
static_assert(kNrcLayers * kNrcWidth <= (int)kWgTmemCols, "layer accumulators exceed the TMEM allocation");
constexpr uint32_t kWgThreads = 128;
constexpr long long kWgWaitCycles = 2000000000ll;        // ~1 s at 2 GHz
// tcgen05 instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16
// (bits 7-9 = 1), B bf16 (bits 10-12 = 1), A and B MN-major (bits 15, 16),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kWgIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                              ((64u >> 3) << 17) | ((64u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of an MN-major operand tile with a 128-byte
// swizzle: start address >> 4 (bits 0-13), 8-row groups 1024 B apart (stride
// byte offset, bits 32-45), descriptor version 1 (bit 46), swizzle mode 2 =
// 128 B (bits 61-63).  The tile is one 64-element atom wide along M/N, so the
// leading byte offset is unused (0).
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(1024u >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long deadline)
{
    for(;;)
    {
        uint32_t ok;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if(ok) return true;
        if(clock64() > deadline) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }"
                 :: "r"(dTmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(kWgThreads, 1)
k_nrc_wgrad_tc(const __grid_constant__ CUtensorMap tmG, const __grid_constant__ CUtensorMap tmA,
               const uint32_t* __restrict__ nDevice, uint32_t nMax, float* __restrict__ part,
               uint32_t* __restrict__ err, uint32_t stallItem)
{
    extern __shared__ uint8_t wgRaw[];
    uint8_t* tiles = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(wgRaw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[kWgStages], empty[kWgStages], done;
    __shared__ uint32_t tmemSlot, aborted, issued, consumed, skipped;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    const uint32_t chunks = (n + kWgRows - 1) / kWgRows;
    const uint32_t myChunks = blockIdx.x < chunks ? (chunks - 1 - blockIdx.x) / gridDim.x + 1 : 0u;
    const uint32_t items = myChunks * kNrcLayers;
    if(items == 0u) return;

    if(tid == 0u)
    {
        for(uint32_t s = 0; s < kWgStages; s++)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        aborted = 0u; issued = 0u; consumed = 0u; skipped = 0xFFFFFFFFu;
    }
    if(warp == 0u)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmemSlot)), "r"(kWgTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmemSlot;
    const long long deadline = clock64() + kWgWaitCycles;

    if(warp == 0u && lane == 0u)
    {
        // producer: TMA pairs into the stages
        for(uint32_t it = 0; it < items; it++)
        {
            const uint32_t s = it % kWgStages, round = it / kWgStages;
            if(!mbar_wait(smem_u32(&empty[s]), (round & 1u) ^ 1u, deadline)) { atomicExch(&aborted, 1u); break; }
            if(*reinterpret_cast<volatile uint32_t*>(&aborted)) break;
            if(it == stallItem && blockIdx.x == 0u)
            {
                // test hook: this stage's copy is never issued, so the MMA
                // warp's bounded wait on it runs out (no fault, no trap)
                *reinterpret_cast<volatile uint32_t*>(&skipped) = it;
                continue;
            }
            const uint32_t chunk = blockIdx.x + (it / kNrcLayers) * gridDim.x, layer = it % kNrcLayers;
            const uint32_t dst = smem_u32(tiles + s * kWgStageBytes), bar = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(kWgStageBytes) : "memory");
            tma_load_2d(dst, &tmG, (int)(layer * kNrcWidth), (int)(chunk * kWgRows), bar);
            tma_load_2d(dst + kWgTileBytes, &tmA, (int)(layer * kNrcWidth), (int)(chunk * kWgRows), bar);
            *reinterpret_cast<volatile uint32_t*>(&issued) = it + 1u;
        }
    }
    else if(warp == 1u)
    {
        // MMA issuer: the warp waits and clears ragged rows, lane 0 issues
        uint32_t it = 0;
        for(; it < items; it++)
        {
            const uint32_t s = it % kWgStages, round = it / kWgStages;
            // warp-uniform: every lane leaves together if any lane's wait ran out
            const bool landed = mbar_wait(smem_u32(&full[s]), round & 1u, deadline);
            if(!__all_sync(0xFFFFFFFFu, landed)) { if(lane == 0u) atomicExch(&aborted, 1u); break; }
            const uint32_t chunk = blockIdx.x + (it / kNrcLayers) * gridDim.x, layer = it % kNrcLayers;
            uint8_t* st = tiles + s * kWgStageBytes;
            const uint32_t rows = min(kWgRows, n - chunk * kWgRows);
            if(rows < kWgRows)
            {
                // rows past the batch hold stale samples: zero them in both tiles
                const uint32_t units = (kWgRows - rows) * 8u;     // 16-byte units per tile
                for(uint32_t q = lane; q < 2u * units; q += 32u)
                {
                    const uint32_t t = q / units, u = q % units;
                    *reinterpret_cast<uint4*>(st + t * kWgTileBytes + rows * 128u + u * 16u) = make_uint4(0, 0, 0, 0);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if(lane == 0u)
            {
                const uint32_t aG = smem_u32(st), aA = aG + kWgTileBytes;
#pragma unroll
                for(uint32_t k = 0; k < kWgRows / 16u; k++)
                    umma_f16(tmem + layer * kNrcWidth, umma_desc(aG + k * 2048u), umma_desc(aA + k * 2048u), kWgIdesc,
                             (it >= (uint32_t)kNrcLayers || k > 0u) ? 1u : 0u);
                umma_commit(smem_u32(&empty[s]));
            }
            __syncwarp();
        }
        if(lane == 0u)
        {
            *reinterpret_cast<volatile uint32_t*>(&consumed) = it;
            umma_commit(smem_u32(&done));   // arrives once every MMA issued above has completed
        }
    }
    __syncthreads();
    const bool finished = mbar_wait(smem_u32(&done), 0u, deadline + kWgWaitCycles);
    const bool ok = finished && !*reinterpret_cast<volatile uint32_t*>(&aborted);
    if(!ok)
    {
        if(tid == 0u)
        {
            atomicOr(err, kNrcWaitTimeout);
            // copies issued but never consumed may still be landing: wait for them
            for(uint32_t it = consumed; it < issued; it++)
                if(it != skipped)
                    mbar_wait(smem_u32(&full[it % kWgStages]), (it / kWgStages) & 1u, clock64() + kWgWaitCycles);
        }
    }
    else
    {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        float* dst = part + (size_t)blockIdx.x * kNrcWeightCount;
        const uint32_t row = 16u * warp + lane;          // lanes 0..15 of each quarter hold rows
        for(uint32_t layer = 0; layer < (uint32_t)kNrcLayers; layer++)
        {
            const uint32_t rows = (layer == (uint32_t)kNrcHidden) ? (uint32_t)kNrcOut : (uint32_t)kNrcWidth;
#pragma unroll
            for(uint32_t c = 0; c < (uint32_t)kNrcWidth; c += 16u)
            {
                uint32_t r[16];
                tmem_ld16(tmem + ((32u * warp) << 16) + layer * kNrcWidth + c, r);
                if(lane < 16u && row < rows)
                {
                    float4* o = reinterpret_cast<float4*>(dst + (size_t)layer * kNrcWidth * kNrcWidth +
                                                          (size_t)row * kNrcWidth + c);
#pragma unroll
                    for(int q = 0; q < 4; q++)
                        o[q] = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]),
                                           __uint_as_float(r[4 * q + 2]), __uint_as_float(r[4 * q + 3]));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if(warp == 0u)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kWgTmemCols) : "memory");
}

// gW[i] += sum over the CTAs that had work, in CTA order.
__global__ void k_nrc_wgrad_sum(const float* __restrict__ part, const uint32_t* __restrict__ nDevice, uint32_t nMax,
                                uint32_t ctas, float* __restrict__ gW)
{
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    const uint32_t used = min(ctas, (n + kWgRows - 1) / kWgRows);
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (uint32_t)kNrcWeightCount; i += gridDim.x * blockDim.x)
    {
        float acc = 0.0f;
        for(uint32_t c = 0; c < used; c++) acc += part[(size_t)c * kNrcWeightCount + i];
        gW[i] += acc;
    }
}

// ---------------------------------------------------------------------------
// Adam (resets the gradient, refreshes the low-precision copy)
// ---------------------------------------------------------------------------
template<bool HALF>
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, float* __restrict__ gr,
                       uint16_t* __restrict__ copy, size_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for(size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        const float gi = gr[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        gr[i] = 0.0f;
        if(HALF) { __half h = __float2half_rn(wi); copy[i] = *reinterpret_cast<uint16_t*>(&h); }
        else { __nv_bfloat16 h = __float2bfloat16_rn(wi); copy[i] = *reinterpret_cast<uint16_t*>(&h); }
    }
}

template<bool HALF>
__global__ void k_copy_params(const float* __restrict__ w, uint16_t* __restrict__ copy, size_t n)
{
    for(size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    {
        if(HALF) { __half h = __float2half_rn(w[i]); copy[i] = *reinterpret_cast<uint16_t*>(&h); }
        else { __nv_bfloat16 h = __float2bfloat16_rn(w[i]); copy[i] = *reinterpret_cast<uint16_t*>(&h); }
    }
}

#ifndef MRG_NRC_QUERY_WARPS
#define MRG_NRC_QUERY_WARPS 16       // warps per CTA of the inference forward
#endif
constexpr size_t fwd_smem(int warps)
{
    return (size_t)(kHiddenRows + kNrcOut) * kPad * 2 + (size_t)warps * 16 * kPad * 2 + (size_t)warps * 64 * 4;
}
#ifndef MRG_NRC_TRAIN_WARPS
#define MRG_NRC_TRAIN_WARPS 16       // warps per CTA of the training forward and backward
#endif
constexpr size_t bwd_smem(int warps)
{
    return (size_t)kHiddenRows * kPad * 2 + (size_t)kNrcWidth * kPadT4 * 2 + (size_t)warps * 16 * 33 * 4;
}

template<bool TRAIN, bool LIST>
cudaError_t launch_forward(const NrcState& S, const float4* in, const uint32_t* list, const uint32_t* nDevice,
                           uint32_t nMax, float4* out, int smCount, cudaStream_t st)
{
    // warps per CTA: MRG_NRC_TRAIN_WARPS for training batches, MRG_NRC_QUERY_WARPS for inference
    constexpr int W = TRAIN ? MRG_NRC_TRAIN_WARPS : MRG_NRC_QUERY_WARPS;
    constexpr size_t smem = fwd_smem(W);
    static int perSMOf[kMaxDevices] = {};          // 0: not configured on that device yet
    int& perSM = perSMOf[launch_device()];
    if(perSM == 0)
    {
        cudaError_t e = cudaFuncSetAttribute(k_nrc_forward<TRAIN, LIST, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if(e != cudaSuccess) return e;
        int b = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_nrc_forward<TRAIN, LIST, W>, W * 32, smem) != cudaSuccess ||
           b < 1)
            b = 1;
        perSM = b;
    }
    const uint32_t tiles = (nMax + 16 * W - 1) / (16 * W);
    const uint32_t grid = std::max(1u, std::min(tiles, (uint32_t)smCount * (uint32_t)perSM * 2u));
    k_nrc_forward<TRAIN, LIST, W><<<grid, W * 32, smem, st>>>(S, in, list, nDevice, nMax, out);
    return cudaGetLastError();
}

} // namespace

size_t nrc_table_entries(const NrcGrid& g) { return (size_t)g.levels << g.log2Table; }

void nrc_make_grid(NrcGrid& g, uint32_t levels, uint32_t log2Table, uint32_t baseRes, uint32_t maxRes,
                   const float aabb[6])
{
    g.levels = levels;
    g.featuresPerLevel = 2;
    g.log2Table = log2Table;
    const double lb = (levels > 1) ? (std::log2((double)maxRes) - std::log2((double)baseRes)) / (levels - 1) : 0.0;
    const uint64_t T = 1ull << log2Table;
    for(uint32_t l = 0; l < 32; l++)
    {
        const double sc = (l < levels) ? std::exp2(l * lb) * baseRes - 1.0 : 0.0;
        g.scale[l] = (float)sc;
        const uint64_t r = (uint64_t)std::ceil((double)g.scale[l]) + 2ull;
        g.res[l] = (uint32_t)r;
        g.dense[l] = (r * r * r <= T) ? 1u : 0u;
    }
    for(int k = 0; k < 3; k++)
    {
        g.aabbMin[k] = aabb[k];
        const float ext = aabb[3 + k] - aabb[k];
        g.aabbInv[k] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
}

cudaError_t nrc_query(const NrcState& S, const float4* inputs, const uint32_t* nDevice, uint32_t nMax,
                      float4* out, int smCount, cudaStream_t st)
{
    return launch_forward<false, false>(S, inputs, nullptr, nDevice, nMax, out, smCount, st);
}

cudaError_t nrc_query_list(const NrcState& S, const float4* inputs, const uint32_t* list, const uint32_t* count,
                           uint32_t nMax, float4* out, int smCount, cudaStream_t st)
{
    return launch_forward<false, true>(S, inputs, list, count, nMax, out, smCount, st);
}

cudaError_t nrc_train(NrcState& S, const float4* inputs, const float4* targets, const uint32_t* nDevice,
                      uint32_t nMax, int smCount, cudaStream_t st)
{
    cudaError_t e = nrc_gradients(S, inputs, targets, nDevice, nMax, smCount, st);
    if(e != cudaSuccess) return e;
    S.step += 1;
    const float c1 = 1.0f / (1.0f - std::pow(S.beta1, (float)S.step));
    const float c2 = 1.0f / (1.0f - std::pow(S.beta2, (float)S.step));
    k_adam<false><<<64, 256, 0, st>>>(S.w32, S.mW, S.vW, S.gW, S.w16, (size_t)kNrcWeightCount, S.lr, S.beta1,
                                      S.beta2, S.eps, c1, c2);
    const size_t nt = nrc_table_entries(S.grid) * 2;
    k_adam<true><<<(unsigned)smCount * 8u, 256, 0, st>>>(S.t32, S.mT, S.vT, S.gT, S.t16, nt, S.lr, S.beta1,
                                                         S.beta2, S.eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t nrc_gradients(NrcState& S, const float4* inputs, const float4* targets, const uint32_t* nDevice,
                          uint32_t nMax, int smCount, cudaStream_t st)
{
    if(nMax > S.cap) return cudaErrorInvalidValue;
    constexpr int W = MRG_NRC_TRAIN_WARPS;
    constexpr size_t bsmem = bwd_smem(W);
    static int perSMOf[kMaxDevices] = {};          // 0: not configured on that device yet
    const int dev = launch_device();
    int& perSM = perSMOf[dev];
    if(perSM == 0)
    {
        cudaError_t e = cudaFuncSetAttribute(k_nrc_backward<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsmem);
        if(e != cudaSuccess) return e;
        int b = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_nrc_backward<W>, W * 32, bsmem) != cudaSuccess || b < 1)
            b = 1;
        perSM = b;
    }
    cudaError_t e = cudaMemsetAsync(S.loss, 0, sizeof(float), st);
    // the forward stores the activations and the outputs of the batch
    if(e == cudaSuccess) e = launch_forward<true, false>(S, inputs, nullptr, nDevice, nMax, S.y, smCount, st);
    const uint32_t tiles = (nMax + 16 * W - 1) / (16 * W);
    const uint32_t grid = std::max(1u, std::min(tiles, (uint32_t)smCount * (uint32_t)perSM * 2u));
    if(e == cudaSuccess)
    {
        k_nrc_backward<W><<<grid, W * 32, bsmem, st>>>(S, inputs, S.y, targets, nDevice, nMax);
        e = cudaGetLastError();
    }
    static bool wgConfigured[kMaxDevices] = {};
    if(e == cudaSuccess && !wgConfigured[dev])
    {
        e = cudaFuncSetAttribute(k_nrc_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWgSmem);
        wgConfigured[dev] = e == cudaSuccess;
    }
    const uint32_t ctas = std::max(1u, std::min(S.partCtas, (nMax + kWgRows - 1) / kWgRows));
    if(e == cudaSuccess)
    {
        // MRG_TEST_WGRAD_STALL=1 (tests only): CTA 0 never issues its first copy
        const char* stall = std::getenv("MRG_TEST_WGRAD_STALL");
        const uint32_t stallItem = (stall && stall[0] == '1') ? 0u : 0xFFFFFFFFu;
        k_nrc_wgrad_tc<<<ctas, kWgThreads, kWgSmem, st>>>(S.tmG16, S.tmActs, nDevice, nMax, S.wgPart, S.err,
                                                         stallItem);
        e = cudaGetLastError();
    }
    if(e == cudaSuccess)
    {
        k_nrc_wgrad_sum<<<(kNrcWeightCount + 255) / 256, 256, 0, st>>>(S.wgPart, nDevice, nMax, ctas, S.gW);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t nrc_make_tensor_maps(NrcState& S)
{
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = nullptr;
    if(!encode)
    {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if(e != cudaSuccess) return e;
        if(q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        encode = reinterpret_cast<Encode>(fn);
    }
    // [cap rows][5 x 64 bf16]: rows 640 B apart; a box is 64 bf16 (128 B, one
    // swizzle span) by kWgRows rows; rows past cap read as zero.
    const cuuint64_t dims[2] = { (cuuint64_t)kG16Row, (cuuint64_t)S.cap };
    const cuuint64_t strides[1] = { (cuuint64_t)kG16Row * 2 };
    const cuuint32_t box[2] = { (cuuint32_t)kNrcWidth, kWgRows };
    const cuuint32_t elem[2] = { 1, 1 };
    void* bases[2] = { S.g16, S.acts };
    CUtensorMap* maps[2] = { &S.tmG16, &S.tmActs };
    for(int k = 0; k < 2; k++)
        if(encode(maps[k], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, bases[k], dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t nrc_sync_copies(const NrcState& S, cudaStream_t st)
{
    k_copy_params<false><<<64, 256, 0, st>>>(S.w32, S.w16, (size_t)kNrcWeightCount);
    k_copy_params<true><<<1024, 256, 0, st>>>(S.t32, S.t16, nrc_table_entries(S.grid) * 2);
    return cudaGetLastError();
}

} // namespace mrg
