// ref_core_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" driver over MRay's OWN core math headers, compiled from
// the reference source tree where it lies (include path = <mray>/Source).
// The resulting library (oracle/_ref/libmray_ref_core.so) is used by the CPU
// tests to pin the oracle restatement (mrg_oracle.c) against the reference's
// compiled code, and to generate the golden fixtures under tests/golden/.
//
// Functions wrapped (reference file:line):
//   RayT<float>::IntersectsTriangle   Source/Core/Ray.hpp:121-167
//   RayT<float>::IntersectsAABB       Source/Core/Ray.hpp:192-219
//   RayT<float>::Nudge                Source/Core/Ray.hpp:258-300
//   Matrix3x4T<float>::Inverse        Source/Core/Matrix.hpp:855-904
//   Matrix3x4T<float>::TransformRay   Source/Core/Matrix.hpp:906-913
//   Matrix3x4T<float>::TransformAABB  Source/Core/Matrix.hpp:915-931
//   MortonCode::Compose3D<uint64_t>   Source/Core/GraphicsFunctions.h:605-625
#include "Core/Ray.h"
#include "Core/Matrix.h"
#include "Core/AABB.h"
#include "Core/GraphicsFunctions.h"

#include <cstdint>
#include <cstring>

extern "C" {

// Batch MT: rays[i] (dir3,pos3) against tris[i] (v0,v1,v2 = 9 floats).
// out_hit[i] = intersected | (backface << 1); bary/t written when hit.
void ref_intersect_triangles(uint32_t n, const float* rays, const float* tris, int cull,
                             uint32_t* out_hit, float* out_bary, float* out_t)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* r = rays + 6 * i;
        const float* t = tris + 9 * i;
        Ray ray(Vector3(r[0], r[1], r[2]), Vector3(r[3], r[4], r[5]));
        Vector3 bary(0);
        Float tt = 0;
        auto res = ray.IntersectsTriangle(bary, tt,
                                          Vector3(t[0], t[1], t[2]),
                                          Vector3(t[3], t[4], t[5]),
                                          Vector3(t[6], t[7], t[8]),
                                          cull != 0);
        out_hit[i] = (res.intersected ? 1u : 0u) | (res.backFace ? 2u : 0u);
        if(res.intersected)
        {
            out_bary[3 * i + 0] = bary[0];
            out_bary[3 * i + 1] = bary[1];
            out_bary[3 * i + 2] = bary[2];
            out_t[i] = tt;
        }
    }
}

// Batch slab test: rays (dir3,pos3), boxes (min3,max3), tmm (2 floats).
void ref_intersect_aabbs(uint32_t n, const float* rays, const float* boxes, const float* tmm,
                         uint32_t* out_hit, float* out_tout)
{
    for(uint32_t i = 0; i < n; i++)
    {
        const float* r = rays + 6 * i;
        const float* b = boxes + 6 * i;
        Ray ray(Vector3(r[0], r[1], r[2]), Vector3(r[3], r[4], r[5]));
        Vector2 tOut;
        auto res = ray.IntersectsAABB(tOut, Vector3(b[0], b[1], b[2]), Vector3(b[3], b[4], b[5]),
                                      Vector2(tmm[2 * i], tmm[2 * i + 1]));
        out_hit[i] = res.intersected ? 1u : 0u;
        out_tout[2 * i] = tOut[0];
        out_tout[2 * i + 1] = tOut[1];
    }
}

void ref_mat34_inverse(const float* m, float* inv)
{
    Matrix3x4 M(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11]);
    Matrix3x4 I = M.Inverse();
    for(int i = 0; i < 12; i++) inv[i] = I[i];
}

void ref_transform_rays(uint32_t n, const float* m, const float* rays, float* out)
{
    Matrix3x4 M(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11]);
    for(uint32_t i = 0; i < n; i++)
    {
        const float* r = rays + 6 * i;
        Ray ray(Vector3(r[0], r[1], r[2]), Vector3(r[3], r[4], r[5]));
        Ray o = M.TransformRay(ray);
        out[6 * i + 0] = o.dir[0]; out[6 * i + 1] = o.dir[1]; out[6 * i + 2] = o.dir[2];
        out[6 * i + 3] = o.pos[0]; out[6 * i + 4] = o.pos[1]; out[6 * i + 5] = o.pos[2];
    }
}

void ref_transform_aabb(const float* m, const float* box, float* out)
{
    Matrix3x4 M(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11]);
    AABB3 a(Vector3(box[0], box[1], box[2]), Vector3(box[3], box[4], box[5]));
    AABB3 r = M.TransformAABB(a);
    for(int k = 0; k < 3; k++) { out[k] = r.Min()[k]; out[3 + k] = r.Max()[k]; }
}

void ref_morton3d_u64(uint32_t n, const uint32_t* xyz, uint64_t* out)
{
    for(uint32_t i = 0; i < n; i++)
        out[i] = Graphics::MortonCode::Compose3D<uint64_t>(Vector3ui(xyz[3 * i], xyz[3 * i + 1],
                                                                     xyz[3 * i + 2]));
}

void ref_nudge(uint32_t n, const float* pos, const float* dirs, float* out)
{
    for(uint32_t i = 0; i < n; i++)
    {
        Ray r(Vector3(0, 0, 1), Vector3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
        Ray o = r.Nudge(Vector3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        out[3 * i] = o.pos[0]; out[3 * i + 1] = o.pos[1]; out[3 * i + 2] = o.pos[2];
    }
}

}
