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

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

namespace mrg {

namespace {

constexpr int kTPB = 128;                     // 4 warps
constexpr int kWarps = kTPB / 32;
constexpr int kPad = 72;                      // padded row of 64 bf16
constexpr int kPadT4 = 24;                    // padded row of W4^T (16 bf16)
constexpr int kHiddenRows = 4 * kNrcWidth;    // rows of W0..W3
constexpr int kActs = 5;                      // stored activations per training sample

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
template<bool TRAIN, bool LIST>
__global__ void __launch_bounds__(kTPB)
k_nrc_forward(NrcState S, const float4* __restrict__ inputs, const uint32_t* __restrict__ list,
              const uint32_t* nDevice, uint32_t nMax, float4* __restrict__ out)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint16_t* sW = reinterpret_cast<uint16_t*>(smem);                       // (256 + 16) x kPad
    uint16_t* sX = sW + (kHiddenRows + kNrcOut) * kPad;                      // kWarps x 16 x kPad
    float* sO = reinterpret_cast<float*>(sX + kWarps * 16 * kPad);           // kWarps x 16 x 4
    for(uint32_t i = threadIdx.x; i < (uint32_t)kNrcWeightCount; i += kTPB)
        sW[(i / kNrcWidth) * kPad + (i % kNrcWidth)] = S.w16[i];
    __syncthreads();
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t g = lane >> 2, t = lane & 3u;
    uint16_t* xw = sX + warp * 16 * kPad;
    float* ow = sO + warp * 64;
    for(uint32_t base = (blockIdx.x * kWarps + warp) * 16u; base < n; base += gridDim.x * kWarps * 16u)
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
        // ---- 4 hidden layers ----
#pragma unroll 1
        for(int layer = 0; layer < 4; layer++)
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
__global__ void __launch_bounds__(kTPB)
k_nrc_backward(NrcState S, const float4* __restrict__ inputs, const float4* __restrict__ y,
               const float4* __restrict__ targets, const uint32_t* nDevice, uint32_t nMax)
{
    extern __shared__ __align__(16) uint8_t smem[];
    // transposed weights: W0^T..W3^T [64 in][64 out] and W4^T [64 in][16 out]
    uint16_t* sT = reinterpret_cast<uint16_t*>(smem);                        // 4 x 64 x kPad
    uint16_t* sT4 = sT + kHiddenRows * kPad;                                  // 64 x kPadT4
    float* sG = reinterpret_cast<float*>(sT4 + kNrcWidth * kPadT4);           // kWarps x 16 x 33
    for(uint32_t i = threadIdx.x; i < (uint32_t)(kHiddenRows * kNrcWidth); i += kTPB)
    {
        const uint32_t layer = i / (kNrcWidth * kNrcWidth), r = (i / kNrcWidth) % kNrcWidth, c = i % kNrcWidth;
        // W[layer][out = r][in = c] -> T[layer][in = c][out = r]
        sT[(layer * kNrcWidth + c) * kPad + r] = S.w16[i];
    }
    for(uint32_t i = threadIdx.x; i < (uint32_t)(kNrcOut * kNrcWidth); i += kTPB)
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
    for(uint32_t base = (blockIdx.x * kWarps + warp) * 16u; base < n; base += gridDim.x * kWarps * 16u)
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
        // store gy rows (dW4 = gy x a4)
        if(v0) { S.gy[(size_t)r0 * 16 + 2 * t] = gy[0][0]; S.gy[(size_t)r0 * 16 + 2 * t + 1] = gy[0][1];
                 S.gy[(size_t)r0 * 16 + 8 + 2 * t] = gy[1][0]; S.gy[(size_t)r0 * 16 + 9 + 2 * t] = gy[1][1]; }
        if(v1) { S.gy[(size_t)r1 * 16 + 2 * t] = gy[0][2]; S.gy[(size_t)r1 * 16 + 2 * t + 1] = gy[0][3];
                 S.gy[(size_t)r1 * 16 + 8 + 2 * t] = gy[1][2]; S.gy[(size_t)r1 * 16 + 9 + 2 * t] = gy[1][3]; }
        uint32_t a[4][4];
        a[0][0] = pack_bf16(gy[0][0], gy[0][1]);
        a[0][1] = pack_bf16(gy[0][2], gy[0][3]);
        a[0][2] = pack_bf16(gy[1][0], gy[1][1]);
        a[0][3] = pack_bf16(gy[1][2], gy[1][3]);
        // ---- g_a4 = gy W4 (k = 16) ----
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
        for(int layer = 3; layer >= 0; layer--)
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
                // store g_z{layer+1} (dW_layer = g_z{layer+1} x a_layer)
                float* G = S.gz + (size_t)layer * kNrcWidth;
                if(v0) { G[(size_t)r0 * 4 * kNrcWidth + c] = acc[nt][0]; G[(size_t)r0 * 4 * kNrcWidth + c + 1] = acc[nt][1]; }
                if(v1) { G[(size_t)r1 * 4 * kNrcWidth + c] = acc[nt][2]; G[(size_t)r1 * 4 * kNrcWidth + c + 1] = acc[nt][3]; }
            }
#pragma unroll
            for(int kt = 0; kt < 4; kt++)
            {
                a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
                a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
                a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
                a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
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
// Weight gradients: dW_l[o][i] = sum_b G[b][o] A[b][i] on CUDA cores
// ---------------------------------------------------------------------------
constexpr int kWgTile = 32;

__global__ void __launch_bounds__(256)
k_nrc_wgrad(NrcState S, const uint32_t* nDevice, uint32_t nMax, uint32_t chunk)
{
    __shared__ float sGt[kWgTile][kNrcWidth];
    __shared__ float sAt[kWgTile][kNrcWidth + 1];
    const uint32_t layer = blockIdx.y;
    const uint32_t n = nDevice ? min(*nDevice, nMax) : nMax;
    const uint32_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    if(b0 >= b1) return;
    const uint32_t rows = (layer == 4) ? kNrcOut : kNrcWidth;
    const uint32_t o = threadIdx.x >> 2, i0 = (threadIdx.x & 3u) * 16u;
    float acc[16];
#pragma unroll
    for(int j = 0; j < 16; j++) acc[j] = 0.0f;
    for(uint32_t b = b0; b < b1; b += kWgTile)
    {
        const uint32_t m = min((uint32_t)kWgTile, b1 - b);
        for(uint32_t k = threadIdx.x; k < (uint32_t)kWgTile * kNrcWidth; k += 256)
        {
            const uint32_t r = k / kNrcWidth, c = k % kNrcWidth;
            float gv = 0.0f, av = 0.0f;
            if(r < m)
            {
                const size_t s = b + r;
                if(layer == 4) gv = (c < (uint32_t)kNrcOut) ? S.gy[s * 16 + c] : 0.0f;
                else gv = S.gz[s * 4 * kNrcWidth + (size_t)layer * kNrcWidth + c];
                av = bf16_to_f(S.acts[s * kActs * kNrcWidth + (size_t)layer * kNrcWidth + c]);
            }
            sGt[r][c] = gv;
            sAt[r][c] = av;
        }
        __syncthreads();
        if(o < rows)
            for(uint32_t r = 0; r < m; r++)
            {
                const float gv = sGt[r][o];
#pragma unroll
                for(int j = 0; j < 16; j++) acc[j] += gv * sAt[r][i0 + j];
            }
        __syncthreads();
    }
    if(o < rows)
    {
        float* dst = S.gW + (size_t)layer * kNrcWidth * kNrcWidth + (size_t)o * kNrcWidth + i0;
#pragma unroll
        for(int j = 0; j < 16; j++) atomicAdd(dst + j, acc[j]);
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

constexpr size_t kFwdSmem = (size_t)(kHiddenRows + kNrcOut) * kPad * 2 + (size_t)kWarps * 16 * kPad * 2 +
                            (size_t)kWarps * 64 * 4;
constexpr size_t kBwdSmem = (size_t)kHiddenRows * kPad * 2 + (size_t)kNrcWidth * kPadT4 * 2 +
                            (size_t)kWarps * 16 * 33 * 4;

template<bool TRAIN, bool LIST>
cudaError_t launch_forward(const NrcState& S, const float4* in, const uint32_t* list, const uint32_t* nDevice,
                           uint32_t nMax, float4* out, int smCount, cudaStream_t st)
{
    static bool configured = false;
    if(!configured)
    {
        cudaError_t e = cudaFuncSetAttribute(k_nrc_forward<TRAIN, LIST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kFwdSmem);
        if(e != cudaSuccess) return e;
        configured = true;
    }
    const uint32_t tiles = (nMax + 16 * kWarps - 1) / (16 * kWarps);
    const uint32_t grid = std::max(1u, std::min(tiles, (uint32_t)smCount * 8u));
    k_nrc_forward<TRAIN, LIST><<<grid, kTPB, kFwdSmem, st>>>(S, in, list, nDevice, nMax, out);
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
    static bool configured = false;
    if(!configured)
    {
        cudaError_t e = cudaFuncSetAttribute(k_nrc_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
        if(e != cudaSuccess) return e;
        configured = true;
    }
    cudaError_t e = cudaMemsetAsync(S.loss, 0, sizeof(float), st);
    // the forward stores the activations and the outputs of the batch
    if(e == cudaSuccess) e = launch_forward<true, false>(S, inputs, nullptr, nDevice, nMax, S.y, smCount, st);
    const uint32_t tiles = (nMax + 16 * kWarps - 1) / (16 * kWarps);
    const uint32_t grid = std::max(1u, std::min(tiles, (uint32_t)smCount * 8u));
    if(e == cudaSuccess)
    {
        k_nrc_backward<<<grid, kTPB, kBwdSmem, st>>>(S, inputs, S.y, targets, nDevice, nMax);
        e = cudaGetLastError();
    }
    const uint32_t chunk = 2048;
    if(e == cudaSuccess)
    {
        k_nrc_wgrad<<<dim3((nMax + chunk - 1) / chunk, kNrcLayers), 256, 0, st>>>(S, nDevice, nMax, chunk);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t nrc_sync_copies(const NrcState& S, cudaStream_t st)
{
    k_copy_params<false><<<64, 256, 0, st>>>(S.w32, S.w16, (size_t)kNrcWeightCount);
    k_copy_params<true><<<1024, 256, 0, st>>>(S.t32, S.t16, nrc_table_entries(S.grid) * 2);
    return cudaGetLastError();
}

} // namespace mrg
