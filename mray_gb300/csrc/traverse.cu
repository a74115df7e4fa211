// traverse.cu -- closest-hit and any-hit traversal of the two-level wide BVH.
//
// One kernel walks TLAS and BLAS (Source/Tracer/AcceleratorLBVH.cu:760-1035
// needs a TLAS kernel, a CUB sort, a host wait and a BLAS kernel per TLAS
// hit; here the instance transform happens in-kernel and the ray never leaves
// the SM).  Node groups / triangle groups on a per-thread stack follow the
// compressed-wide-BVH traversal of Ylitie, Karras and Laine (HPG 2017),
// including its meta-byte hit-mask construction and triangle postponing.
//
// Work distribution is persistent with per-lane refill: a warp keeps up to 32
// rays in flight; whenever enough lanes have finished, the idle lanes claim
// new rays from a global counter together (one atomic per refill), so long
// rays no longer hold a whole warp of finished lanes.
//
// The triangle test, the ray transform and the instance-leaf slab test are
// bit-exact restatements of MRay's host arithmetic (see mrg_device.cuh).
#include "mrg_build.h"
#include "mrg_device.cuh"
#include "mrg_launch.h"

namespace mrg {

namespace {

// Tuning knobs (compile-time; the defaults are the measured best on GB300).
#ifndef MRG_TRACE_MIN_BLOCKS
#define MRG_TRACE_MIN_BLOCKS 7       // resident 128-thread blocks per SM the register budget targets
#endif
#ifndef MRG_TRACE_REFILL
#define MRG_TRACE_REFILL 8           // refill when at least this many lanes are idle
#endif
#ifndef MRG_TRACE_STEP_BUDGET
#define MRG_TRACE_STEP_BUDGET 24     // traversal iterations between refill checks
#endif
#ifndef MRG_TRACE_PREFETCH
#define MRG_TRACE_PREFETCH 0         // L1 prefetch of the next node
#endif
#ifndef MRG_TRACE_SORT_INST
#define MRG_TRACE_SORT_INST 0        // 1: enter the instances of a TLAS leaf group nearest-first
#endif
#ifndef MRG_TRACE_POSTPONE
#define MRG_TRACE_POSTPONE 0         // postpone triangles when fewer lanes want them
#endif
#ifndef MRG_TRACE_SMEM_STACK
#define MRG_TRACE_SMEM_STACK 0       // >0: the first entries of each thread's stack live in shared memory
#endif
#ifndef MRG_NODE_OCTLOAD
#define MRG_NODE_OCTLOAD 0           // 1: near / far plane vectors loaded by the ray's octant, not selected
#endif
#ifndef MRG_NODE_SIGNHIT
#define MRG_NODE_SIGNHIT 0           // 1: child hit from the sign of tf - tn (FMA pipe) instead of a compare
#endif
#ifndef MRG_TRACE_TRI_CHUNK
#define MRG_TRACE_TRI_CHUNK 2        // >0: at most this many triangles per iteration, the rest go on the stack
#endif

constexpr int kTraceTPB = 128;
constexpr int kStackSize = 32;
constexpr uint32_t kStepCap = 1u << 24;
constexpr int kRefillMin = MRG_TRACE_REFILL;
constexpr int kStepBudget = MRG_TRACE_STEP_BUDGET;
constexpr int kPostponeLanes = MRG_TRACE_POSTPONE;

struct LevelRay
{
    float ox, oy, oz;
    float ix, iy, iz;
    uint32_t oct7;      // (octant ^ 7); octant bit i set: direction i negative
    uint32_t octRep;    // oct7 replicated into 4 bytes
};

// Inverse direction for the quantised box tests.  A fast reciprocal is
// enough: its one-ulp error scales each axis' plane distances by 1 +- 2^-23,
// far inside the boxes' inflation (1e-5 of the accelerator extent plus one
// quantum).  Tiny components are clamped so the planes stay finite.
__device__ __forceinline__ float guard_inv(float d)
{
    float a = (fabsf(d) > 1.0e-20f) ? d : copysignf(1.0e-20f, d);
    return __fdividef(1.0f, a);
}

__device__ __forceinline__ void setup_level(LevelRay& r, float ox, float oy, float oz,
                                            float dx, float dy, float dz)
{
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.ix = guard_inv(dx); r.iy = guard_inv(dy); r.iz = guard_inv(dz);
    const uint32_t oct = (signbit(dx) ? 1u : 0u) | (signbit(dy) ? 2u : 0u) | (signbit(dz) ? 4u : 0u);
    r.oct7 = oct ^ 7u;
    r.octRep = r.oct7 * 0x01010101u;
}

__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Byte k of w plus 2^23, as a float (exact): the quantised plane index,
// biased.  The bias is folded into the per-axis offset of the node, or (exact
// decode) subtracted again, which leaves the byte's value exactly.
__device__ __forceinline__ float qbias(uint32_t w, uint32_t k)
{
#if MRG_NODE_EXACT_Q
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k)), 8388608.0f);
#else
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k));
#endif
}

#ifndef MRG_TRACE_RECOMPUTE_WINV
#define MRG_TRACE_RECOMPUTE_WINV 0  // 1: the world ray's 1/dir is recomputed at TLAS leaves, not kept
#endif
#if MRG_NODE_F16
// Tests the ray against the 8 children of node `ni` (fp16 child planes).
// Returns the hit mask: bits 24..31 = internal children keyed by
// (slot ^ oct7) so that the highest key is the nearest corner, bits 0..23 =
// payload slots of leaf children (relative to the node's payload base).  A
// plane at p + h * 2^e is reached at t = h * (2^e / d) + (p - o) / d, one fma
// per plane; the stored planes are rounded outward and every box carries the
// builder's inflation, which covers the rounding of that evaluation.
__device__ __forceinline__ uint32_t intersect_node(const WideNode* __restrict__ nodes, uint32_t ni,
                                                   const LevelRay& r, float tmin, float tmax,
                                                   uint32_t& childBase, uint32_t& triBase,
                                                   uint32_t& imask)
{
    const uint4* np = reinterpret_cast<const uint4*>(nodes + ni);
    const uint4 a = __ldg(np + 0);
    const uint4 b = __ldg(np + 1);
    // near planes: the upper ones on axes the ray runs down
    const uint32_t nxo = (r.oct7 & 1u) ? 0u : 3u, nyo = (r.oct7 & 2u) ? 0u : 3u, nzo = (r.oct7 & 4u) ? 0u : 3u;
    const uint2* pnX = reinterpret_cast<const uint2*>(np + 2 + nxo);
    const uint2* pfX = reinterpret_cast<const uint2*>(np + 5 - nxo);
    const uint2* pnY = reinterpret_cast<const uint2*>(np + 3 + nyo);
    const uint2* pfY = reinterpret_cast<const uint2*>(np + 6 - nyo);
    const uint2* pnZ = reinterpret_cast<const uint2*>(np + 4 + nzo);
    const uint2* pfZ = reinterpret_cast<const uint2*>(np + 7 - nzo);
    const uint32_t packed = a.w;
    const float sx = __uint_as_float((packed & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((packed >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((packed >> 16) & 0xFFu) << 23) * r.iz;
    const float ax = (__uint_as_float(a.x) - r.ox) * r.ix;
    const float ay = (__uint_as_float(a.y) - r.oy) * r.iy;
    const float az = (__uint_as_float(a.z) - r.oz) * r.iz;
    imask = packed >> 24;
    childBase = b.x;
    triBase = b.y;

    uint32_t hm = 0;
#pragma unroll
    for(uint32_t h = 0; h < 2; h++)
    {
        // children 4h .. 4h + 3: 8 bytes of each plane vector
        const uint2 nX = __ldg(pnX + h), fX = __ldg(pfX + h);
        const uint2 nY = __ldg(pnY + h), fY = __ldg(pfY + h);
        const uint2 nZ = __ldg(pnZ + h), fZ = __ldg(pfZ + h);
        const uint32_t nx4[2] = { nX.x, nX.y }, fx4[2] = { fX.x, fX.y };
        const uint32_t ny4[2] = { nY.x, nY.y }, fy4[2] = { fY.x, fY.y };
        const uint32_t nz4[2] = { nZ.x, nZ.y }, fz4[2] = { fZ.x, fZ.y };
        // meta byte: internal = 0b001_11sss (24 + slot), leaf = unary count << 5 | offset,
        // empty = 0.  For internal children xor the slot bits with oct7.
        const uint32_t meta4 = h ? b.w : b.z;
        const uint32_t inner4 = ((meta4 & (meta4 << 1)) & 0x10101010u) >> 4;   // 1 per internal byte
        const uint32_t bitIdx4 = (meta4 ^ (r.octRep & (inner4 * 0xFFu))) & 0x1F1F1F1Fu;
        const uint32_t bits4 = (meta4 >> 5) & 0x07070707u;
#pragma unroll
        for(uint32_t w = 0; w < 2; w++)
        {
            const uint32_t wnx = nx4[w], wfx = fx4[w], wny = ny4[w], wfy = fy4[w], wnz = nz4[w], wfz = fz4[w];
            const float2 tnx2 = __half22float2(*reinterpret_cast<const __half2*>(&wnx));
            const float2 tfx2 = __half22float2(*reinterpret_cast<const __half2*>(&wfx));
            const float2 tny2 = __half22float2(*reinterpret_cast<const __half2*>(&wny));
            const float2 tfy2 = __half22float2(*reinterpret_cast<const __half2*>(&wfy));
            const float2 tnz2 = __half22float2(*reinterpret_cast<const __half2*>(&wnz));
            const float2 tfz2 = __half22float2(*reinterpret_cast<const __half2*>(&wfz));
#pragma unroll
            for(uint32_t c = 0; c < 2; c++)
            {
                const uint32_t k = 2 * w + c;
                const float tnx = fmaf(c ? tnx2.y : tnx2.x, sx, ax);
                const float tny = fmaf(c ? tny2.y : tny2.x, sy, ay);
                const float tnz = fmaf(c ? tnz2.y : tnz2.x, sz, az);
                const float tfx = fmaf(c ? tfx2.y : tfx2.x, sx, ax);
                const float tfy = fmaf(c ? tfy2.y : tfy2.x, sy, ay);
                const float tfz = fmaf(c ? tfz2.y : tfz2.x, sz, az);
                const float tn = fmaxf(max3f(tnx, tny, tnz), tmin);
                const float tf = fminf(min3f(tfx, tfy, tfz), tmax);
                const uint32_t cb = (bits4 >> (8u * k)) & 0xFFu;
                const uint32_t bi = (bitIdx4 >> (8u * k)) & 0xFFu;
                hm |= (tn <= tf) ? (cb << bi) : 0u;
            }
        }
    }
    return hm;
}
#else
#ifndef MRG_NODE_FFMA2
#define MRG_NODE_FFMA2 0            // 1: plane distances of two children per packed fp32x2 fma
#endif

// Two planes at once: (q0, q1) * s + a, both lanes of one fp32x2 fma (and,
// with exact decode, the 2^23 bias removed by one fp32x2 subtract first).
__device__ __forceinline__ float2 plane2(uint32_t w, uint32_t k0, uint32_t k1, float s, float a)
{
    const float b0 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k0));
    const float b1 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k1));
    float r0, r1;
#if MRG_NODE_EXACT_Q
    asm("{\n\t.reg .b64 q, b, s, a, t, d;\n\t"
        "mov.b64 q, {%2, %3};\n\tmov.b64 b, {%4, %4};\n\tmov.b64 s, {%5, %5};\n\tmov.b64 a, {%6, %6};\n\t"
        "sub.rn.f32x2 t, q, b;\n\tfma.rn.f32x2 d, t, s, a;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r0), "=f"(r1) : "f"(b0), "f"(b1), "f"(8388608.0f), "f"(s), "f"(a));
#else
    asm("{\n\t.reg .b64 q, s, a, d;\n\t"
        "mov.b64 q, {%2, %3};\n\tmov.b64 s, {%4, %4};\n\tmov.b64 a, {%5, %5};\n\t"
        "fma.rn.f32x2 d, q, s, a;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r0), "=f"(r1) : "f"(b0), "f"(b1), "f"(s), "f"(a));
#endif
    return make_float2(r0, r1);
}

// The x and y planes of child k: (qx, qy) * (sx, sy) + (ax, ay), one fp32x2 fma.
__device__ __forceinline__ float2 planes_xy(uint32_t wx, uint32_t wy, uint32_t k, float sx, float sy,
                                            float ax, float ay)
{
    const float bx = qbias(wx, k), by = qbias(wy, k);
    float r0, r1;
    asm("{\n\t.reg .b64 q, s, a, d;\n\t"
        "mov.b64 q, {%2, %3};\n\tmov.b64 s, {%4, %5};\n\tmov.b64 a, {%6, %7};\n\t"
        "fma.rn.f32x2 d, q, s, a;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r0), "=f"(r1) : "f"(bx), "f"(by), "f"(sx), "f"(sy), "f"(ax), "f"(ay));
    return make_float2(r0, r1);
}

// Tests the ray against the 8 children of node `ni`.  Returns the hit mask:
// bits 24..31 = internal children keyed by (slot ^ oct7) so that the highest
// key is the nearest corner, bits 0..23 = payload slots of leaf children
// (relative to the node's payload base).  The plane offset
// a' = (p - o) * idir - 2^23 * s is off by at most half a quantum; the
// builder widens every child box by a full quantum to cover it.
__device__ __forceinline__ uint32_t intersect_node(const WideNode* __restrict__ nodes, uint32_t ni,
                                                   const LevelRay& r, float tmin, float tmax,
                                                   uint32_t& childBase, uint32_t& triBase,
                                                   uint32_t& imask)
{
    const uint4* np = reinterpret_cast<const uint4*>(nodes + ni);
    const uint4 a = __ldg(np + 0);
    const uint4 b = __ldg(np + 1);
#if MRG_NODE_OCTLOAD
    // The six 8-byte plane vectors as uint2 [lo_x, lo_y, lo_z, hi_x, hi_y,
    // hi_z]; the near / far vector of each axis is addressed by the ray's
    // octant instead of selected after loading.
    const uint2* qv = reinterpret_cast<const uint2*>(np + 2);
    const uint32_t nxi = (r.oct7 & 1u) ? 0u : 3u, nyi = (r.oct7 & 2u) ? 1u : 4u, nzi = (r.oct7 & 4u) ? 2u : 5u;
    const uint2 vnX = __ldg(qv + nxi), vfX = __ldg(qv + (3u - nxi));
    const uint2 vnY = __ldg(qv + nyi), vfY = __ldg(qv + (5u - nyi));
    const uint2 vnZ = __ldg(qv + nzi), vfZ = __ldg(qv + (7u - nzi));
#else
    const uint4 q0 = __ldg(np + 2);
    const uint4 q1 = __ldg(np + 3);
    const uint4 q2 = __ldg(np + 4);
#endif
    const uint32_t packed = a.w;
    const float sx = __uint_as_float((packed & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((packed >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((packed >> 16) & 0xFFu) << 23) * r.iz;
#if MRG_NODE_EXACT_Q
    const float ax = (__uint_as_float(a.x) - r.ox) * r.ix;
    const float ay = (__uint_as_float(a.y) - r.oy) * r.iy;
    const float az = (__uint_as_float(a.z) - r.oz) * r.iz;
#else
    const float ax = fmaf(-8388608.0f, sx, (__uint_as_float(a.x) - r.ox) * r.ix);
    const float ay = fmaf(-8388608.0f, sy, (__uint_as_float(a.y) - r.oy) * r.iy);
    const float az = fmaf(-8388608.0f, sz, (__uint_as_float(a.z) - r.oz) * r.iz);
#endif
    imask = packed >> 24;
    childBase = b.x;
    triBase = b.y;

    // q0 = lo_x[0..3], lo_x[4..7], lo_y[0..3], lo_y[4..7]
    // q1 = lo_z[0..3], lo_z[4..7], hi_x[0..3], hi_x[4..7]
    // q2 = hi_y[0..3], hi_y[4..7], hi_z[0..3], hi_z[4..7]
    uint32_t hm = 0;
#if !MRG_NODE_OCTLOAD
    const bool nx = !(r.oct7 & 1u), ny = !(r.oct7 & 2u), nz = !(r.oct7 & 4u);
#endif
#pragma unroll
    for(uint32_t h = 0; h < 2; h++)
    {
#if MRG_NODE_OCTLOAD
        const uint32_t nearX = h ? vnX.y : vnX.x, farX = h ? vfX.y : vfX.x;
        const uint32_t nearY = h ? vnY.y : vnY.x, farY = h ? vfY.y : vfY.x;
        const uint32_t nearZ = h ? vnZ.y : vnZ.x, farZ = h ? vfZ.y : vfZ.x;
#else
        const uint32_t loX = h ? q0.y : q0.x, hiX = h ? q1.w : q1.z;
        const uint32_t loY = h ? q0.w : q0.z, hiY = h ? q2.y : q2.x;
        const uint32_t loZ = h ? q1.y : q1.x, hiZ = h ? q2.w : q2.z;
        const uint32_t nearX = nx ? hiX : loX, farX = nx ? loX : hiX;
        const uint32_t nearY = ny ? hiY : loY, farY = ny ? loY : hiY;
        const uint32_t nearZ = nz ? hiZ : loZ, farZ = nz ? loZ : hiZ;
#endif
        // meta byte: internal = 0b001_11sss (24 + slot), leaf = unary count << 5 | offset,
        // empty = 0.  For internal children xor the slot bits with oct7.
        const uint32_t meta4 = h ? b.w : b.z;
        const uint32_t inner4 = ((meta4 & (meta4 << 1)) & 0x10101010u) >> 4;   // 1 per internal byte
        const uint32_t bitIdx4 = (meta4 ^ (r.octRep & (inner4 * 0xFFu))) & 0x1F1F1F1Fu;
        const uint32_t bits4 = (meta4 >> 5) & 0x07070707u;
#if MRG_NODE_FFMA2 == 2
#pragma unroll
        for(uint32_t k = 0; k < 4; k++)
        {
            // x and y planes of one child per fp32x2 fma, z alone
            const float2 nxy = planes_xy(nearX, nearY, k, sx, sy, ax, ay);
            const float2 fxy = planes_xy(farX, farY, k, sx, sy, ax, ay);
            const float tnz = fmaf(qbias(nearZ, k), sz, az);
            const float tfz = fmaf(qbias(farZ, k), sz, az);
            const float tn = fmaxf(max3f(nxy.x, nxy.y, tnz), tmin);
            const float tf = fminf(min3f(fxy.x, fxy.y, tfz), tmax);
            const uint32_t cb = (bits4 >> (8u * k)) & 0xFFu;
            const uint32_t bi = (bitIdx4 >> (8u * k)) & 0xFFu;
            hm |= (tn <= tf) ? (cb << bi) : 0u;
        }
#elif MRG_NODE_FFMA2
#pragma unroll
        for(uint32_t k = 0; k < 4; k += 2)
        {
            const float2 nx2 = plane2(nearX, k, k + 1, sx, ax), fx2 = plane2(farX, k, k + 1, sx, ax);
            const float2 ny2 = plane2(nearY, k, k + 1, sy, ay), fy2 = plane2(farY, k, k + 1, sy, ay);
            const float2 nz2 = plane2(nearZ, k, k + 1, sz, az), fz2 = plane2(farZ, k, k + 1, sz, az);
#pragma unroll
            for(uint32_t c = 0; c < 2; c++)
            {
                const float tn = fmaxf(max3f(c ? nx2.y : nx2.x, c ? ny2.y : ny2.x, c ? nz2.y : nz2.x), tmin);
                const float tf = fminf(min3f(c ? fx2.y : fx2.x, c ? fy2.y : fy2.x, c ? fz2.y : fz2.x), tmax);
                const uint32_t cb = (bits4 >> (8u * (k + c))) & 0xFFu;
                const uint32_t bi = (bitIdx4 >> (8u * (k + c))) & 0xFFu;
                hm |= (tn <= tf) ? (cb << bi) : 0u;
            }
        }
#else
#pragma unroll
        for(uint32_t k = 0; k < 4; k++)
        {
            const float tnx = fmaf(qbias(nearX, k), sx, ax);
            const float tny = fmaf(qbias(nearY, k), sy, ay);
            const float tnz = fmaf(qbias(nearZ, k), sz, az);
            const float tfx = fmaf(qbias(farX, k), sx, ax);
            const float tfy = fmaf(qbias(farY, k), sy, ay);
            const float tfz = fmaf(qbias(farZ, k), sz, az);
            const float tn = fmaxf(max3f(tnx, tny, tnz), tmin);
            const float tf = fminf(min3f(tfx, tfy, tfz), tmax);
            const uint32_t cb = (bits4 >> (8u * k)) & 0xFFu;
            const uint32_t bi = (bitIdx4 >> (8u * k)) & 0xFFu;
#if MRG_NODE_SIGNHIT
            // tn <= tf as the sign of tf - tn (the subtraction runs on the FMA
            // pipe; the all-ones / zero mask from an arithmetic shift then
            // merges into the hit mask in one logic op).  tf - tn is -0 only
            // for tf = -0 <= tn = +0, a box that ends at t = 0 and holds no
            // hit with t > 1e-7.
            const int32_t miss = __float_as_int(__fsub_rn(tf, tn)) >> 31;
            hm |= (cb << bi) & ~(uint32_t)miss;
#else
            hm |= (tn <= tf) ? (cb << bi) : 0u;
#endif
        }
#endif
    }
    return hm;
}

#endif

// LOCAL: listed ray i starts inside instance instIds[i] (its BLAS, in the
// instance's space) and ends when that BLAS is exhausted: CastLocalRays.
// WT: the watertight triangle test on records that hold the three vertices.
template<bool ANY, bool STATS, bool LOCAL = false, bool WT = false>
__global__ void __launch_bounds__(kTraceTPB, MRG_TRACE_MIN_BLOCKS)
k_trace(TraceScene sc, TraceScratch scr, float4* __restrict__ rays,
        const uint32_t* __restrict__ rayIdx, uint32_t nHost, const uint32_t* __restrict__ nDevice,
        uint4* __restrict__ hits, float2* __restrict__ meta, uint32_t* __restrict__ visBits,
        const uint32_t* __restrict__ instIds = nullptr)
{
    // The ray count comes from the host or, for casts inside a device-driven
    // wavefront, from device memory written by the previous kernel.
    const uint32_t n = nDevice ? *nDevice : nHost;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t laneLt = (1u << lane) - 1u;
    constexpr int kSmemStack = MRG_TRACE_SMEM_STACK;
    uint2 stack[kStackSize - kSmemStack];
#if MRG_TRACE_SMEM_STACK > 0
    __shared__ uint2 sStack[kSmemStack][kTraceTPB];
#endif
    // stack entries [0, kSmemStack) in shared memory, the rest in local memory
    auto push = [&](uint2 v, int& p) {
#if MRG_TRACE_SMEM_STACK > 0
        if(p < kSmemStack) sStack[p][threadIdx.x] = v; else
#endif
        stack[p - kSmemStack] = v;
        p++;
    };
    auto pop = [&](int& p) -> uint2 {
        --p;
#if MRG_TRACE_SMEM_STACK > 0
        if(p < kSmemStack) return sStack[p][threadIdx.x];
#endif
        return stack[p - kSmemStack];
    };

    // Per-lane ray state.
    bool live = false;
    uint32_t ri = 0;
    float wox = 0, woy = 0, woz = 0, wdx = 0, wdy = 0, wdz = 0, tmin = 0, tmax = 0;
#if !MRG_TRACE_RECOMPUTE_WINV
    float wix = 0, wiy = 0, wiz = 0;   // IEEE 1/dir of the world ray (exact leaf slab test)
#endif
    LevelRay lr;
    float3 ld = make_float3(0, 0, 0);   // local direction (the local origin is lr.ox/oy/oz)
    uint2 ng = make_uint2(0, 0), tg = make_uint2(0, 0);
    int sp = 0, blasBase = -1;
    uint32_t curInst = kInvalidIndex, hitPrim = 0, hitInst = kInvalidIndex;
    bool cull = false;
    float hitU = 0.0f, hitV = 0.0f;
    uint32_t steps = 0;
    uint32_t statNodes = 0, statTris = 0, statInst = 0, statTlasNodes = 0, statDry = 0;
    uint32_t instHitBefore = kInvalidIndex;
    float instTBefore = 0.0f;
    bool warpDone = false;

    for(;;)
    {
        // ---- refill idle lanes (warp-uniform decision) ------------------------
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !live);
        if(!warpDone && __popc(idle) >= kRefillMin)
        {
            const uint32_t cnt = __popc(idle);
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if((int)lane == leader) base = atomicAdd(scr.workCounter, cnt);
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if(base + cnt >= n) warpDone = true;
            if(!live)
            {
                const uint32_t i = base + __popc(idle & laneLt);
                if(i < n)
                {
                    ri = rayIdx ? __ldg(rayIdx + i) : i;
                    const float4 r0 = rays[2 * (size_t)ri];
                    const float4 r1 = rays[2 * (size_t)ri + 1];
                    wox = r0.x; woy = r0.y; woz = r0.z; tmin = r0.w;
                    wdx = r1.x; wdy = r1.y; wdz = r1.z; tmax = r1.w;
#if !MRG_TRACE_RECOMPUTE_WINV
                    wix = __frcp_rn(wdx); wiy = __frcp_rn(wdy); wiz = __frcp_rn(wdz);
#endif
                    setup_level(lr, wox, woy, woz, wdx, wdy, wdz);
                    ng = make_uint2(sc.tlasRoot, (1u << (24u + lr.oct7)) | 1u);
                    tg = make_uint2(0u, 0u);
                    sp = 0; blasBase = -1;
                    curInst = kInvalidIndex; hitInst = kInvalidIndex;
                    steps = 0;
                    if(STATS) { statNodes = 0; statTris = 0; statInst = 0; statTlasNodes = 0; statDry = 0; }
                    live = true;
                    if(LOCAL)
                    {
                        const uint32_t inst = __ldg(instIds + i);
                        if(inst >= sc.instCount) { atomicOr(scr.errorFlag, kTraceBadIndex); live = false; }
                        else
                        {
                            // enter the instance as at a TLAS leaf, with an empty world stack
                            const float4* ip = reinterpret_cast<const float4*>(sc.insts + inst);
                            const float4 m0 = __ldg(ip), m1 = __ldg(ip + 1), m2 = __ldg(ip + 2);
                            const uint4 keys = __ldg(reinterpret_cast<const uint4*>(ip + 3));
                            float3 lo;
                            transform_ray_exact(m0, m1, m2, make_float3(wox, woy, woz), make_float3(wdx, wdy, wdz),
                                                lo, ld);
                            setup_level(lr, lo.x, lo.y, lo.z, ld.x, ld.y, ld.z);
                            cull = (keys.w & kCullBit) != 0u;
                            curInst = inst;
                            blasBase = 0;
                            ng = make_uint2(keys.w & ~kCullBit, (1u << (24u + lr.oct7)) | 1u);
                        }
                    }
                }
            }
        }
        if(__ballot_sync(0xFFFFFFFFu, live) == 0u) break;
        if(!live) continue;

        // ---- traverse for a bounded number of iterations ----------------------
        bool finished = false;
        for(int it = 0; it < kStepBudget && !finished; it++)
        {
            if(++steps > kStepCap) { atomicOr(scr.errorFlag, kTraceStepCap); finished = true; break; }
            if(ng.y > 0x00FFFFFFu)
            {
                const uint32_t bit = 31u - __clz(ng.y);
                const uint32_t slot = (bit - 24u) ^ lr.oct7;
                ng.y &= ~(1u << bit);
                const uint32_t rank = __popc((ng.y & 0xFFu) & ((1u << slot) - 1u));
                const uint32_t ni = ng.x + rank;
                if(ni >= sc.nodeCount) { atomicOr(scr.errorFlag, kTraceBadIndex); finished = true; break; }
                if(ng.y > 0x00FFFFFFu)
                {
                    if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); finished = true; break; }
                    push(ng, sp);
                }
                uint32_t cb, tb, im;
                const uint32_t hm = intersect_node(sc.nodes, ni, lr, tmin, tmax, cb, tb, im);
                if(STATS) { statNodes++; if(blasBase < 0) statTlasNodes++; }
                ng = make_uint2(cb, (hm & 0xFF000000u) ? ((hm & 0xFF000000u) | im) : 0u);
                tg = make_uint2(tb, hm & 0x00FFFFFFu);
                if(MRG_TRACE_PREFETCH && ng.y)
                {
                    // The nearest hit child is visited next: start its fetch now
                    // so the triangle work below overlaps the L2 latency.
                    const uint32_t nb = 31u - __clz(ng.y);
                    const uint32_t nslot = (nb - 24u) ^ lr.oct7;
                    const uint32_t nni = cb + __popc(im & ((1u << nslot) - 1u));
                    if(nni < sc.nodeCount)
                    {
                        const char* np = reinterpret_cast<const char*>(sc.nodes + nni);
                        asm volatile("prefetch.global.L1 [%0];" :: "l"(np));
                        asm volatile("prefetch.global.L1 [%0];" :: "l"(np + 64));
                    }
                }
            }
            else
            {
                tg = ng;
                ng = make_uint2(0u, 0u);
            }

            if(blasBase >= 0)
            {
                // triangles of a BLAS leaf group
                int triDone = 0;
                while(tg.y != 0u)
                {
                    if(MRG_TRACE_TRI_CHUNK > 0 && triDone == MRG_TRACE_TRI_CHUNK && sp < kStackSize)
                    {
                        // the rest of the group waits on the stack (as postponed triangles do)
                        push(tg, sp);
                        tg.y = 0u;
                        break;
                    }
                    triDone++;
                    // Postpone when few lanes want triangles and this lane has
                    // nodes left: SIMD lanes stay on the wider node work.
                    if(kPostponeLanes > 0 && ng.y > 0x00FFFFFFu && __popc(__activemask()) < kPostponeLanes &&
                       sp < kStackSize)
                    {
                        push(tg, sp);
                        tg.y = 0u;
                        break;
                    }
                    const uint32_t bt = __ffs(tg.y) - 1u;
                    tg.y &= tg.y - 1u;
                    const uint32_t pi = tg.x + bt;
                    if(pi >= sc.triCount) { atomicOr(scr.errorFlag, kTraceBadIndex); finished = true; break; }
                    const float4* tp = reinterpret_cast<const float4*>(sc.tris + pi);
                    const float4 v0 = __ldg(tp), e0 = __ldg(tp + 1), e1 = __ldg(tp + 2);
                    if(STATS) statTris++;
                    float t, u, v;
                    const bool isect = WT ? intersect_tri_watertight(make_float3(lr.ox, lr.oy, lr.oz), ld, v0, e0, e1,
                                                                     cull, t, u, v)
                                          : intersect_tri_exact(make_float3(lr.ox, lr.oy, lr.oz), ld, v0, e0, e1,
                                                                cull, t, u, v);
                    if(isect && t >= tmin && t < tmax)
                    {
                        tmax = t; hitU = u; hitV = v;
                        hitPrim = __float_as_uint(v0.w);
                        hitInst = curInst;
                        if(ANY) { finished = true; break; }
                    }
                }
                if(finished) break;
            }
            else
            {
                // instances of a TLAS leaf group.  MRay's exact slab test on the
                // exact world AABB decides entry (the wide TLAS boxes above are
                // conservative and only cull); among the candidates that pass
                // it, the nearest entry is taken first and the rest go back on
                // the stack, to be re-tested against the shrunken tMax.
                if(tg.y != 0u)
                {
#if MRG_TRACE_RECOMPUTE_WINV
                    // IEEE 1/dir of the world ray, recomputed here to keep registers free
                    const float wix = __frcp_rn(wdx), wiy = __frcp_rn(wdy), wiz = __frcp_rn(wdz);
#endif
                    uint32_t keep = 0u, best = 32u;
                    float bestT = 0.0f;
                    for(uint32_t cand = tg.y; cand != 0u; cand &= cand - 1u)
                    {
                        const uint32_t bt = __ffs(cand) - 1u;
                        const uint32_t pi = tg.x + bt;
                        if(pi >= sc.instCount) { atomicOr(scr.errorFlag, kTraceBadIndex); finished = true; break; }
                        const uint32_t inst = __ldg(sc.tlasLeaf + pi);
                        if(inst >= sc.instCount) { atomicOr(scr.errorFlag, kTraceBadIndex); finished = true; break; }
                        const float4* ip = reinterpret_cast<const float4*>(sc.insts + inst);
                        float tEnter;
                        if(!intersect_aabb_exact(wox, woy, woz, wix, wiy, wiz, __ldg(ip + 4), __ldg(ip + 5),
                                                 tmin, tmax, tEnter))
                            continue;
                        keep |= 1u << bt;
                        if(best == 32u || (MRG_TRACE_SORT_INST && tEnter < bestT)) { best = bt; bestT = tEnter; }
                        if(!MRG_TRACE_SORT_INST) break;
                    }
                    if(finished) break;
                    if(!MRG_TRACE_SORT_INST && best != 32u) keep = tg.y;   // untested ones stay candidates
                    tg.y = 0u;
                    if(best != 32u)
                    {
                        keep &= ~(1u << best);
                        const uint32_t inst = __ldg(sc.tlasLeaf + tg.x + best);
                        const float4* ip = reinterpret_cast<const float4*>(sc.insts + inst);
                        if(ng.y > 0x00FFFFFFu)
                        {
                            if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); finished = true; break; }
                            push(ng, sp);
                        }
                        if(keep != 0u)
                        {
                            if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); finished = true; break; }
                            push(make_uint2(tg.x, keep), sp);
                        }
                        blasBase = sp;
                        const float4 m0 = __ldg(ip), m1 = __ldg(ip + 1), m2 = __ldg(ip + 2);
                        float3 lo;
                        const uint4 keys = __ldg(reinterpret_cast<const uint4*>(ip + 3));
                        transform_ray_exact(m0, m1, m2, make_float3(wox, woy, woz),
                                            make_float3(wdx, wdy, wdz), lo, ld);
                        setup_level(lr, lo.x, lo.y, lo.z, ld.x, ld.y, ld.z);
                        cull = (keys.w & kCullBit) != 0u;
                        curInst = inst;
                        if(STATS) { statInst++; instHitBefore = hitInst; instTBefore = tmax; }
                        ng = make_uint2(keys.w & ~kCullBit, (1u << (24u + lr.oct7)) | 1u);
                    }
                }
            }

            if(ng.y <= 0x00FFFFFFu)
            {
                if(blasBase >= 0 && sp == blasBase)
                {
                    if(STATS && tmax == instTBefore) statDry++;
                    blasBase = -1;
                    setup_level(lr, wox, woy, woz, wdx, wdy, wdz);
                }
                if(sp == 0) { finished = true; break; }
                ng = pop(sp);
            }
        }

        if(finished)
        {
            live = false;
            const bool found = hitInst != kInvalidIndex;
            if(STATS)
            {
                atomicAdd(&scr.stats[0], 1ull);
                atomicAdd(&scr.stats[1], (unsigned long long)statNodes);
                atomicAdd(&scr.stats[2], (unsigned long long)statTris);
                atomicAdd(&scr.stats[3], (unsigned long long)statInst);
                atomicAdd(&scr.stats[4], (unsigned long long)statTlasNodes);
                atomicAdd(&scr.stats[5], (unsigned long long)statDry);
            }
            else if(ANY)
            {
                const uint32_t bitm = 1u << (ri & 31u);
                if(found) atomicAnd(visBits + (ri >> 5), ~bitm);
                else      atomicOr(visBits + (ri >> 5), bitm);
            }
            else if(found)
            {
                const uint4 keys = __ldg(reinterpret_cast<const uint4*>(sc.insts + hitInst) + 3);
                hits[ri] = make_uint4(hitPrim, keys.x, keys.y, keys.z);
                // MT: (1 - u - v, u) as MRay forms it; WT: both weights computed
                const float w = WT ? hitV : __fsub_rn(__fsub_rn(1.0f, hitU), hitV);
                meta[ri] = make_float2(w, hitU);
                reinterpret_cast<float*>(rays)[8 * (size_t)ri + 7] = tmax;
            }
        }
    }
}

template<bool ANY, bool STATS, bool LOCAL = false, bool WT = false>
int blocks_for(int smCount)
{
    static int perSMOf[kMaxDevices] = {};          // 0: not queried on that device yet
    int& perSM = perSMOf[launch_device()];
    if(perSM == 0)
    {
        int b = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<ANY, STATS, LOCAL, WT>, kTraceTPB, 0) != cudaSuccess ||
           b < 1)
            b = 4;
        perSM = b;
    }
    return perSM * smCount;
}

} // namespace

cudaError_t preload_closest()
{
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, k_trace<false, false>);
}

cudaError_t launch_closest(const TraceScene& sc, const TraceScratch& scr, void* rays,
                           const uint32_t* rayIdx, uint32_t n, void* hits, void* meta,
                           int smCount, cudaStream_t st, const uint32_t* nDevice)
{
    if(n == 0 && nDevice == nullptr) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    if(sc.watertight)
        k_trace<false, false, false, true><<<blocks_for<false, false, false, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, static_cast<float4*>(rays), rayIdx, n, nDevice, static_cast<uint4*>(hits),
            static_cast<float2*>(meta), nullptr);
    else
        k_trace<false, false><<<blocks_for<false, false>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, static_cast<float4*>(rays), rayIdx, n, nDevice, static_cast<uint4*>(hits),
            static_cast<float2*>(meta), nullptr);
    return cudaGetLastError();
}

cudaError_t launch_local(const TraceScene& sc, const TraceScratch& scr, void* rays, const uint32_t* rayIdx,
                         const uint32_t* instIds, uint32_t n, void* hits, void* meta, int smCount, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    if(sc.watertight)
        k_trace<false, false, true, true><<<blocks_for<false, false, true, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, static_cast<float4*>(rays), rayIdx, n, nullptr, static_cast<uint4*>(hits),
            static_cast<float2*>(meta), nullptr, instIds);
    else
        k_trace<false, false, true><<<blocks_for<false, false, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, static_cast<float4*>(rays), rayIdx, n, nullptr, static_cast<uint4*>(hits),
            static_cast<float2*>(meta), nullptr, instIds);
    return cudaGetLastError();
}

cudaError_t launch_visibility(const TraceScene& sc, const TraceScratch& scr, uint32_t* visBits,
                              const void* rays, const uint32_t* rayIdx, uint32_t n,
                              int smCount, cudaStream_t st, const uint32_t* nDevice)
{
    if(n == 0 && nDevice == nullptr) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    if(sc.watertight)
        k_trace<true, false, false, true><<<blocks_for<true, false, false, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), rayIdx, n, nDevice, nullptr,
            nullptr, visBits);
    else
        k_trace<true, false><<<blocks_for<true, false>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), rayIdx, n, nDevice, nullptr,
            nullptr, visBits);
    return cudaGetLastError();
}

cudaError_t launch_closest_stats(const TraceScene& sc, const TraceScratch& scr, const void* rays,
                                 uint32_t n, int smCount, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    e = cudaMemsetAsync(scr.stats, 0, 8 * sizeof(unsigned long long), st);
    if(e != cudaSuccess) return e;
    if(sc.watertight)
        k_trace<false, true, false, true><<<blocks_for<false, true, false, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), nullptr, n, nullptr, nullptr,
            nullptr, nullptr);
    else
        k_trace<false, true><<<blocks_for<false, true>(smCount), kTraceTPB, 0, st>>>(
            sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), nullptr, n, nullptr, nullptr,
            nullptr, nullptr);
    return cudaGetLastError();
}

} // namespace mrg
