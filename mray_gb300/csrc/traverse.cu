// traverse.cu -- closest-hit and any-hit traversal of the two-level wide BVH.
//
// One kernel walks TLAS and BLAS (Source/Tracer/AcceleratorLBVH.cu:760-1035
// needs a TLAS kernel, a CUB sort, a host wait and a BLAS kernel per TLAS
// hit; here the instance transform happens in-kernel and the ray never leaves
// the SM).  Node groups / triangle groups on a per-thread stack follow the
// compressed-wide-BVH traversal of Ylitie, Karras and Laine (HPG 2017).
// Work distribution is persistent: each warp claims 32 rays at a time from a
// global counter (work stealing), so the grid is sized to the resident
// capacity of the 152 SMs rather than to the ray count.
// The triangle test and the ray transform are bit-exact restatements of MRay's
// host arithmetic (see mrg_device.cuh).
#include "mrg_build.h"
#include "mrg_device.cuh"

namespace mrg {

namespace {

constexpr int kTraceTPB = 128;
constexpr int kStackSize = 32;
constexpr uint32_t kStepCap = 1u << 24;

struct LevelRay
{
    float ox, oy, oz;
    float ix, iy, iz;
    uint32_t oct;       // bit i set: direction component i is negative
    uint32_t oct7;      // oct ^ 7: slot -> key permutation
};

__device__ __forceinline__ float guard_inv(float d)
{
    float a = (fabsf(d) > 1.0e-20f) ? d : copysignf(1.0e-20f, d);
    return 1.0f / a;
}

__device__ __forceinline__ void setup_level(LevelRay& r, float ox, float oy, float oz,
                                            float dx, float dy, float dz)
{
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.ix = guard_inv(dx); r.iy = guard_inv(dy); r.iz = guard_inv(dz);
    r.oct = (signbit(dx) ? 1u : 0u) | (signbit(dy) ? 2u : 0u) | (signbit(dz) ? 4u : 0u);
    r.oct7 = r.oct ^ 7u;
}

// Integer byte k of w as a float: 2^23 + b reinterpreted, minus 2^23 (exact).
__device__ __forceinline__ float qbyte(uint32_t w, uint32_t k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | k)) - 8388608.0f;
}

// Tests the ray against the (up to) 8 children of node `ni`.  Returns the hit
// mask: bits 24..31 = internal children keyed by (slot ^ oct7), bits 0..23 =
// triangle (or instance) slots relative to the node's payload base.
__device__ __forceinline__ uint32_t intersect_node(const WideNode* __restrict__ nodes, uint32_t ni,
                                                   const LevelRay& r, float tmin, float tmax,
                                                   uint32_t& childBase, uint32_t& triBase,
                                                   uint32_t& imask)
{
    const uint4* np = reinterpret_cast<const uint4*>(nodes + ni);
    const uint4 a = __ldg(np + 0);
    const uint4 b = __ldg(np + 1);
    const uint4 q0 = __ldg(np + 2);
    const uint4 q1 = __ldg(np + 3);
    const uint4 q2 = __ldg(np + 4);
    const float px = __uint_as_float(a.x), py = __uint_as_float(a.y), pz = __uint_as_float(a.z);
    const uint32_t packed = a.w;
    const float sx = __uint_as_float((packed & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((packed >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((packed >> 16) & 0xFFu) << 23) * r.iz;
    const float ax = (px - r.ox) * r.ix;
    const float ay = (py - r.oy) * r.iy;
    const float az = (pz - r.oz) * r.iz;
    imask = packed >> 24;
    childBase = b.x;
    triBase = b.y;

    // q0 = lo_x[0..3], lo_x[4..7], lo_y[0..3], lo_y[4..7]
    // q1 = lo_z[0..3], lo_z[4..7], hi_x[0..3], hi_x[4..7]
    // q2 = hi_y[0..3], hi_y[4..7], hi_z[0..3], hi_z[4..7]
    const bool nx = r.oct & 1u, ny = r.oct & 2u, nz = r.oct & 4u;
    uint32_t hm = 0;
#pragma unroll
    for(uint32_t h = 0; h < 2; h++)
    {
        const uint32_t loX = h ? q0.y : q0.x, hiX = h ? q1.w : q1.z;
        const uint32_t loY = h ? q0.w : q0.z, hiY = h ? q2.y : q2.x;
        const uint32_t loZ = h ? q1.y : q1.x, hiZ = h ? q2.w : q2.z;
        const uint32_t nearX = nx ? hiX : loX, farX = nx ? loX : hiX;
        const uint32_t nearY = ny ? hiY : loY, farY = ny ? loY : hiY;
        const uint32_t nearZ = nz ? hiZ : loZ, farZ = nz ? loZ : hiZ;
        const uint32_t meta4 = h ? b.w : b.z;
#pragma unroll
        for(uint32_t k = 0; k < 4; k++)
        {
            const uint32_t s = 4u * h + k;
            const uint32_t m = (meta4 >> (8u * k)) & 0xFFu;
            const float tnx = fmaf(qbyte(nearX, k), sx, ax);
            const float tny = fmaf(qbyte(nearY, k), sy, ay);
            const float tnz = fmaf(qbyte(nearZ, k), sz, az);
            const float tfx = fmaf(qbyte(farX, k), sx, ax);
            const float tfy = fmaf(qbyte(farY, k), sy, ay);
            const float tfz = fmaf(qbyte(farZ, k), sz, az);
            const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
            const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
            if(m != 0u && tn <= tf)
            {
                if((imask >> s) & 1u) hm |= 1u << (24u + (s ^ r.oct7));
                else hm |= ((m >> 5) & 7u) << (m & 31u);
            }
        }
    }
    return hm;
}

template<bool ANY, bool STATS>
__global__ void __launch_bounds__(kTraceTPB)
k_trace(TraceScene sc, TraceScratch scr, float4* __restrict__ rays,
        const uint32_t* __restrict__ rayIdx, uint32_t n,
        uint4* __restrict__ hits, float2* __restrict__ meta, uint32_t* __restrict__ visBits)
{
    const uint32_t lane = threadIdx.x & 31u;
    uint2 stack[kStackSize];

    for(;;)
    {
        uint32_t base = 0;
        if(lane == 0) base = atomicAdd(scr.workCounter, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if(base >= n) break;
        const uint32_t i = base + lane;
        const bool valid = i < n;
        bool found = false;
        uint32_t ri = 0;
        uint32_t statNodes = 0, statTris = 0, statInst = 0;

        if(valid)
        {
            ri = rayIdx ? __ldg(rayIdx + i) : i;
            const float4 r0 = rays[2 * (size_t)ri];
            const float4 r1 = rays[2 * (size_t)ri + 1];
            const float wox = r0.x, woy = r0.y, woz = r0.z;
            const float wdx = r1.x, wdy = r1.y, wdz = r1.z;
            const float tmin = r0.w;
            float tmax = r1.w;

            LevelRay lr;
            setup_level(lr, wox, woy, woz, wdx, wdy, wdz);
            float3 lo = make_float3(wox, woy, woz);
            float3 ld = make_float3(wdx, wdy, wdz);
            uint2 ng = make_uint2(sc.tlasRoot, (1u << (24u + lr.oct7)) | 1u);
            uint2 tg = make_uint2(0u, 0u);
            int sp = 0;
            int blasBase = -1;
            uint32_t curInst = kInvalidIndex;
            bool cull = false;
            uint32_t hitPrim = 0, hitInst = kInvalidIndex;
            float hitU = 0.0f, hitV = 0.0f;
            uint32_t steps = 0;

            for(;;)
            {
                if(++steps > kStepCap) { atomicOr(scr.errorFlag, kTraceStepCap); break; }
                if(ng.y > 0x00FFFFFFu)
                {
                    const uint32_t bit = 31u - __clz(ng.y);
                    const uint32_t slot = (bit - 24u) ^ lr.oct7;
                    ng.y &= ~(1u << bit);
                    const uint32_t rank = __popc((ng.y & 0xFFu) & ((1u << slot) - 1u));
                    const uint32_t ni = ng.x + rank;
                    if(ni >= sc.nodeCount) { atomicOr(scr.errorFlag, kTraceBadIndex); break; }
                    if(ng.y > 0x00FFFFFFu)
                    {
                        if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); break; }
                        stack[sp++] = ng;
                    }
                    uint32_t cb, tb, im;
                    const uint32_t hm = intersect_node(sc.nodes, ni, lr, tmin, tmax, cb, tb, im);
                    if(STATS) statNodes++;
                    ng = make_uint2(cb, (hm & 0xFF000000u) ? ((hm & 0xFF000000u) | im) : 0u);
                    tg = make_uint2(tb, hm & 0x00FFFFFFu);
                }
                else
                {
                    tg = ng;
                    ng = make_uint2(0u, 0u);
                }

                bool stop = false;
                while(tg.y != 0u)
                {
                    const uint32_t b = __ffs(tg.y) - 1u;
                    tg.y &= tg.y - 1u;
                    const uint32_t pi = tg.x + b;
                    if(blasBase >= 0)
                    {
                        if(pi >= sc.triCount) { atomicOr(scr.errorFlag, kTraceBadIndex); stop = true; break; }
                        const float4* tp = reinterpret_cast<const float4*>(sc.tris + pi);
                        const float4 v0 = __ldg(tp), e0 = __ldg(tp + 1), e1 = __ldg(tp + 2);
                        if(STATS) statTris++;
                        float t, u, v;
                        if(intersect_tri_exact(lo, ld, v0, e0, e1, cull, t, u, v) &&
                           t >= tmin && t < tmax)
                        {
                            tmax = t; hitU = u; hitV = v;
                            hitPrim = __float_as_uint(v0.w);
                            hitInst = curInst;
                            if(ANY) { stop = true; break; }
                        }
                    }
                    else
                    {
                        if(pi >= sc.instCount) { atomicOr(scr.errorFlag, kTraceBadIndex); stop = true; break; }
                        const uint32_t inst = __ldg(sc.tlasLeaf + pi);
                        if(inst >= sc.instCount) { atomicOr(scr.errorFlag, kTraceBadIndex); stop = true; break; }
                        const float4* ip = reinterpret_cast<const float4*>(sc.insts + inst);
                        // MRay's own leaf test decides whether the instance is entered
                        // (the wide TLAS boxes above are conservative and only cull).
                        if(!intersect_aabb_exact(wox, woy, woz, wdx, wdy, wdz, __ldg(ip + 4), __ldg(ip + 5),
                                                 tmin, tmax))
                            continue;
                        if(ng.y > 0x00FFFFFFu)
                        {
                            if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); stop = true; break; }
                            stack[sp++] = ng;
                        }
                        if(tg.y != 0u)
                        {
                            if(sp >= kStackSize) { atomicOr(scr.errorFlag, kTraceStackOverflow); stop = true; break; }
                            stack[sp++] = tg;
                        }
                        blasBase = sp;
                        const float4 m0 = __ldg(ip), m1 = __ldg(ip + 1), m2 = __ldg(ip + 2);
                        const uint4 keys = __ldg(reinterpret_cast<const uint4*>(ip + 3));
                        transform_ray_exact(m0, m1, m2, make_float3(wox, woy, woz),
                                            make_float3(wdx, wdy, wdz), lo, ld);
                        setup_level(lr, lo.x, lo.y, lo.z, ld.x, ld.y, ld.z);
                        cull = (keys.w & kCullBit) != 0u;
                        curInst = inst;
                        if(STATS) statInst++;
                        ng = make_uint2(keys.w & ~kCullBit, (1u << (24u + lr.oct7)) | 1u);
                        tg.y = 0u;
                        break;
                    }
                }
                if(stop) break;
                if(ng.y <= 0x00FFFFFFu)
                {
                    if(blasBase >= 0 && sp == blasBase)
                    {
                        blasBase = -1;
                        setup_level(lr, wox, woy, woz, wdx, wdy, wdz);
                    }
                    if(sp == 0) break;
                    ng = stack[--sp];
                }
            }

            found = hitInst != kInvalidIndex;
            if(!ANY && !STATS && found)
            {
                const uint4 keys = __ldg(reinterpret_cast<const uint4*>(sc.insts + hitInst) + 3);
                hits[ri] = make_uint4(hitPrim, keys.x, keys.y, keys.z);
                const float w = __fsub_rn(__fsub_rn(1.0f, hitU), hitV);
                meta[ri] = make_float2(w, hitU);
                reinterpret_cast<float*>(rays)[8 * (size_t)ri + 7] = tmax;
            }
        }

        if(STATS)
        {
            if(valid)
            {
                atomicAdd(&scr.stats[0], 1ull);
                atomicAdd(&scr.stats[1], (unsigned long long)statNodes);
                atomicAdd(&scr.stats[2], (unsigned long long)statTris);
                atomicAdd(&scr.stats[3], (unsigned long long)statInst);
            }
        }
        if(ANY)
        {
            if(rayIdx == nullptr)
            {
                // Lanes of this warp own word base/32 of the bitspan.
                const uint32_t vis = __ballot_sync(0xFFFFFFFFu, valid && !found);
                const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
                if(lane == 0)
                {
                    uint32_t* w = visBits + (base >> 5);
                    *w = (vmask == 0xFFFFFFFFu) ? vis : ((*w & ~vmask) | vis);
                }
            }
            else if(valid)
            {
                const uint32_t bit = 1u << (ri & 31u);
                if(found) atomicAnd(visBits + (ri >> 5), ~bit);
                else      atomicOr(visBits + (ri >> 5), bit);
            }
        }
    }
}

template<bool ANY, bool STATS>
int blocks_for(int smCount)
{
    static int perSM = 0;
    if(perSM == 0)
    {
        int b = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<ANY, STATS>, kTraceTPB, 0) != cudaSuccess || b < 1)
            b = 4;
        perSM = b;
    }
    return perSM * smCount;
}

} // namespace

cudaError_t launch_closest(const TraceScene& sc, const TraceScratch& scr, void* rays,
                           const uint32_t* rayIdx, uint32_t n, void* hits, void* meta,
                           int smCount, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    k_trace<false, false><<<blocks_for<false, false>(smCount), kTraceTPB, 0, st>>>(
        sc, scr, static_cast<float4*>(rays), rayIdx, n, static_cast<uint4*>(hits),
        static_cast<float2*>(meta), nullptr);
    return cudaGetLastError();
}

cudaError_t launch_visibility(const TraceScene& sc, const TraceScratch& scr, uint32_t* visBits,
                              const void* rays, const uint32_t* rayIdx, uint32_t n,
                              int smCount, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    k_trace<true, false><<<blocks_for<true, false>(smCount), kTraceTPB, 0, st>>>(
        sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), rayIdx, n, nullptr,
        nullptr, visBits);
    return cudaGetLastError();
}

cudaError_t launch_closest_stats(const TraceScene& sc, const TraceScratch& scr, const void* rays,
                                 uint32_t n, int smCount, cudaStream_t st)
{
    if(n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scr.workCounter, 0, sizeof(uint32_t), st);
    if(e != cudaSuccess) return e;
    e = cudaMemsetAsync(scr.stats, 0, 4 * sizeof(unsigned long long), st);
    if(e != cudaSuccess) return e;
    k_trace<false, true><<<blocks_for<false, true>(smCount), kTraceTPB, 0, st>>>(
        sc, scr, const_cast<float4*>(static_cast<const float4*>(rays)), nullptr, n, nullptr,
        nullptr, nullptr);
    return cudaGetLastError();
}

} // namespace mrg
