// mrg_device.cuh -- device-side data layout and exact-arithmetic helpers.
//
// HBM layout of one accelerator (all arrays 16-byte aligned):
//   WideNode  wnodes[]   80 B each: 8-wide node with 8-bit quantised child
//                        boxes (compressed wide BVH, Ylitie/Karras/Laine 2017).
//   TriRecord tris[]     48 B each: v0, e0 = v1 - v0, e1 = v2 - v0, primKey.
//                        e0/e1 are the exact float differences MRay's
//                        Moller-Trumbore forms first (Source/Core/Ray.hpp:131-132),
//                        so storing them keeps the test bit-identical.
//   InstRecord insts[]   96 B each: inverse 3x4 transform rows, keys, exact world AABB.
//   uint32    tlasLeaf[] instance index per TLAS leaf slot.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "mrg_build.h"

namespace mrg {

struct __align__(16) WideNode
{
    // w0: origin p (x,y,z) + packed (ex | ey<<8 | ez<<16 | imask<<24)
    float4 w0;
    // w1: childBase, triBase, meta[0..3], meta[4..7]
    uint4  w1;
#if MRG_NODE_F16
    // h[a]: the 8 children's planes as fp16 offsets (plane - p) * 2^-e, a =
    // 0, 1, 2: lower x, y, z; 3, 4, 5: upper x, y, z (lower rounded down,
    // upper rounded up)
    uint4  h[6];
#else
    // q[0]: qlo_x[0..7] qlo_y[0..7]; q[1]: qlo_z qhi_x; q[2]: qhi_y qhi_z
    uint4  q[3];
#endif
};
static_assert(sizeof(WideNode) == (MRG_NODE_F16 ? 128 : 80), "wide node size");

struct __align__(16) TriRecord
{
    float4 v0;   // w = primKey (bit pattern)
    float4 e0;   // w = 0
    float4 e1;   // w = 0
};
static_assert(sizeof(TriRecord) == 48, "triangle record must be 48 bytes");

struct __align__(16) InstRecord
{
    float4 inv[3];   // rows of the world->local 3x4 matrix
    uint4  keys;     // lightOrMatKey, transKey, accelKey, blasRoot | cull<<31
    float4 wmin;     // exact world AABB (Matrix3x4::TransformAABB of the BLAS box), w unused
    float4 wmax;
};
static_assert(sizeof(InstRecord) == 96, "instance record must be 96 bytes");

constexpr uint32_t kCullBit = 0x80000000u;
constexpr uint32_t kInvalidIndex = 0xFFFFFFFFu;

// -------------------------------------------------------------------------
// Exact arithmetic in MRay's operation order.  Each helper uses
// round-to-nearest intrinsics, which nvcc never contracts or reassociates,
// so results are bit-identical to the reference host build.
// -------------------------------------------------------------------------
// Math::Dot (Source/Core/Math.h:1586-1596): r = 0; r = fma(a_i, b_i, r).
__device__ __forceinline__ float dot3_exact(float ax, float ay, float az,
                                            float bx, float by, float bz)
{
    float r = __fmaf_rn(ax, bx, 0.0f);
    r = __fmaf_rn(ay, by, r);
    r = __fmaf_rn(az, bz, r);
    return r;
}
// 4-term Dot with w = 1 (Matrix3x4 * Vector4(p, 1), Source/Core/Matrix.hpp:777-788).
__device__ __forceinline__ float dot4w1_exact(float4 row, float px, float py, float pz)
{
    float r = __fmaf_rn(row.x, px, 0.0f);
    r = __fmaf_rn(row.y, py, r);
    r = __fmaf_rn(row.z, pz, r);
    r = __fmaf_rn(row.w, 1.0f, r);
    return r;
}
// Math::Cross (Source/Core/Math.h:1627-1633).
__device__ __forceinline__ void cross_exact(float ax, float ay, float az,
                                            float bx, float by, float bz,
                                            float& ox, float& oy, float& oz)
{
    ox = __fmaf_rn(ay, bz, -__fmul_rn(az, by));
    oy = __fmaf_rn(az, bx, -__fmul_rn(ax, bz));
    oz = __fmaf_rn(ax, by, -__fmul_rn(ay, bx));
}

constexpr float kSmallEpsilon = 1.0e-7f;   // MathConstants::SmallEpsilon

// Ray::IntersectsTriangle (Source/Core/Ray.hpp:121-167) on a stored record.
// Returns true on a hit; t, b0 (= u) and b1 (= v) are MRay's values; the
// reported MetaHit is (1 - u - v, u).
__device__ __forceinline__ bool intersect_tri_exact(const float3& o, const float3& d,
                                                    const float4& v0, const float4& e0,
                                                    const float4& e1, bool cull,
                                                    float& tOut, float& uOut, float& vOut)
{
    float px, py, pz;
    cross_exact(d.x, d.y, d.z, e1.x, e1.y, e1.z, px, py, pz);
    float det = dot3_exact(e0.x, e0.y, e0.z, px, py, pz);
    bool backface = det < kSmallEpsilon;
    bool parallel = fabsf(det) < kSmallEpsilon;
    if((cull && backface) || parallel) return false;
    float invDet = __frcp_rn(det);          // IEEE 1/det
    float tx = __fsub_rn(o.x, v0.x);
    float ty = __fsub_rn(o.y, v0.y);
    float tz = __fsub_rn(o.z, v0.z);
    float u = __fmul_rn(dot3_exact(tx, ty, tz, px, py, pz), invDet);
    if(u < 0.0f || u > 1.0f) return false;
    float qx, qy, qz;
    cross_exact(tx, ty, tz, e0.x, e0.y, e0.z, qx, qy, qz);
    float v = __fmul_rn(dot3_exact(d.x, d.y, d.z, qx, qy, qz), invDet);
    if(v < 0.0f || __fadd_rn(v, u) > 1.0f) return false;
    float t = __fmul_rn(dot3_exact(e1.x, e1.y, e1.z, qx, qy, qz), invDet);
    if(t <= kSmallEpsilon) return false;
    tOut = t; uOut = u; vOut = v;
    return true;
}

// Watertight ray/triangle test (S. Woop, C. Benthin, I. Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013), the opt-in alternative to
// MRay's Moller-Trumbore test.  The ray is sheared to run along +z; the
// triangle's scaled barycentrics are 2D edge functions of the sheared
// vertices, so two triangles sharing an edge evaluate it from the same two
// vertices and a ray through the edge hits one of them.  Edge functions that
// round to exactly 0 are recomputed in double.  The record holds the three
// vertices (v0, v1 = e0 slot, v2 = e1 slot).  Same outputs as the MT test:
// t > SmallEpsilon, (u, v) = weights of v1 and v2, back faces where MT's
// determinant is negative; the MetaHit pair is (U, V) / det, both computed.
// IEEE round-to-nearest operations only, in the oracle's order
// (orc_intersect_triangle_wt).
__device__ __forceinline__ bool intersect_tri_watertight(const float3& o, const float3& d,
                                                         const float4& v0, const float4& v1,
                                                         const float4& v2, bool cull,
                                                         float& tOut, float& uOut, float& wOut)
{
    const float dd[3] = { d.x, d.y, d.z };
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = (kz == 2) ? 0 : kz + 1;
    int ky = (kx == 2) ? 0 : kx + 1;
    if(dd[kz] < 0.0f) { const int t = kx; kx = ky; ky = t; }
    const float Sx = __fdiv_rn(dd[kx], dd[kz]), Sy = __fdiv_rn(dd[ky], dd[kz]);
    const float Sz = __frcp_rn(dd[kz]);
    const float A[3] = { __fsub_rn(v0.x, o.x), __fsub_rn(v0.y, o.y), __fsub_rn(v0.z, o.z) };
    const float B[3] = { __fsub_rn(v1.x, o.x), __fsub_rn(v1.y, o.y), __fsub_rn(v1.z, o.z) };
    const float C[3] = { __fsub_rn(v2.x, o.x), __fsub_rn(v2.y, o.y), __fsub_rn(v2.z, o.z) };
    const float Ax = __fsub_rn(A[kx], __fmul_rn(Sx, A[kz])), Ay = __fsub_rn(A[ky], __fmul_rn(Sy, A[kz]));
    const float Bx = __fsub_rn(B[kx], __fmul_rn(Sx, B[kz])), By = __fsub_rn(B[ky], __fmul_rn(Sy, B[kz]));
    const float Cx = __fsub_rn(C[kx], __fmul_rn(Sx, C[kz])), Cy = __fsub_rn(C[ky], __fmul_rn(Sy, C[kz]));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if(U == 0.0f || V == 0.0f || W == 0.0f)
    {
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    const bool allNeg = (U <= 0.0f && V <= 0.0f && W <= 0.0f);
    const bool allPos = (U >= 0.0f && V >= 0.0f && W >= 0.0f);
    if(!allNeg && !allPos) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if(det == 0.0f) return false;
    if(cull && det < 0.0f) return false;
    const float Az = __fmul_rn(Sz, A[kz]), Bz = __fmul_rn(Sz, B[kz]), Cz = __fmul_rn(Sz, C[kz]);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __frcp_rn(det);
    const float t = __fmul_rn(T, rcp);
    if(t <= kSmallEpsilon) return false;
    tOut = t;
    uOut = __fmul_rn(V, rcp);      // weight of v1 (MRay's b0, MetaHit[1])
    wOut = __fmul_rn(U, rcp);      // weight of v0 (MetaHit[0], computed, not 1 - u - v)
    return true;
}

// Matrix3x4::TransformRay (Source/Core/Matrix.hpp:906-913) with the inverse.
__device__ __forceinline__ void transform_ray_exact(const float4 r0, const float4 r1,
                                                    const float4 r2,
                                                    const float3& o, const float3& d,
                                                    float3& lo, float3& ld)
{
    ld.x = dot3_exact(r0.x, r0.y, r0.z, d.x, d.y, d.z);
    ld.y = dot3_exact(r1.x, r1.y, r1.z, d.x, d.y, d.z);
    ld.z = dot3_exact(r2.x, r2.y, r2.z, d.x, d.y, d.z);
    lo.x = dot4w1_exact(r0, o.x, o.y, o.z);
    lo.y = dot4w1_exact(r1, o.x, o.y, o.z);
    lo.z = dot4w1_exact(r2, o.x, o.y, o.z);
}

// std::max / std::min as the reference host build evaluates them
// (Source/Core/Math.h:342-380): the first argument wins unless the compare holds.
__device__ __forceinline__ float std_max(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float std_min(float x, float y) { return (y < x) ? y : x; }

// Ray::IntersectsAABB (Source/Core/Ray.hpp:192-219), bit-exact: the decision
// MRay takes at every TLAS leaf (AcceleratorLBVH.cu:465-473).  ix/iy/iz are
// the IEEE reciprocals of the direction, 1 / dir (__frcp_rn gives exactly the
// correctly rounded quotient), computed once per ray by the caller.
__device__ __forceinline__ bool intersect_aabb_exact(float ox, float oy, float oz,
                                                     float ix, float iy, float iz,
                                                     const float4& bmin, const float4& bmax,
                                                     float tmin, float tmax, float& tEnter)
{
    const float id[3] = { ix, iy, iz };
    const float o[3] = { ox, oy, oz };
    const float lo[3] = { bmin.x, bmin.y, bmin.z };
    const float hi[3] = { bmax.x, bmax.y, bmax.z };
    float o0 = tmin, o1 = tmax;
#pragma unroll
    for(int i = 0; i < 3; i++)
    {
        float t0 = __fmul_rn(__fsub_rn(lo[i], o[i]), id[i]);
        float t1 = __fmul_rn(__fsub_rn(hi[i], o[i]), id[i]);
        if(id[i] < 0.0f) { float s = t0; t0 = t1; t1 = s; }
        o0 = std_max(o0, std_min(t0, t1));
        o1 = std_min(o1, std_max(t0, t1));
    }
    tEnter = o0;
    return o1 >= o0;
}

} // namespace mrg
