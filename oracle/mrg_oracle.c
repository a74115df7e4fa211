/*
 * mrg_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see mrg_oracle.h).
 *
 * Plain-C restatement of MRay's host-backend software BVH path:
 *   - Moller-Trumbore triangle test      Source/Core/Ray.hpp:121-167
 *   - slab ray/AABB test                 Source/Core/Ray.hpp:192-219
 *   - Matrix3x4 inverse / ray transform  Source/Core/Matrix.hpp:855-904, 906-931
 *   - 64-bit 3D Morton code              Source/Core/GraphicsFunctions.h:605-625
 *   - LBVH build (Karras 2012)           Source/Tracer/AcceleratorLBVH.cu:69-435,
 *                                        Source/Tracer/AcceleratorLBVH.hpp:584-899
 *   - stack traversal (CPU backend)      Source/Tracer/AcceleratorLBVH.hpp:111-166
 *   - closest / first hit                Source/Tracer/AcceleratorLBVH.hpp:225-410
 *   - instance transform of the ray      Source/Tracer/AcceleratorWork.kt.h:179-244
 *   - two-level cast semantics           Source/Tracer/AcceleratorLBVH.cu:437-495, 760-1035
 * Compile with -ffp-contract=off.
 */
#include "mrg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>

/* ------------------------------------------------------------------------ */
/* Scalar helpers with the reference's host semantics                        */
/* ------------------------------------------------------------------------ */
/* std::max / std::min (Source/Core/Math.h:342-380, host path). */
static inline float smax(float x, float y) { return (x < y) ? y : x; }
static inline float smin(float x, float y) { return (y < x) ? y : x; }

/* Math::Dot: r = 0; r = fma(a_i, b_i, r) for i = 0..2 (Math.h:1586-1596). */
static inline float dot3(const float a[3], const float b[3])
{
    float r = 0.0f;
    r = fmaf(a[0], b[0], r);
    r = fmaf(a[1], b[1], r);
    r = fmaf(a[2], b[2], r);
    return r;
}
static inline float dot4(const float a[4], const float b[4])
{
    float r = 0.0f;
    r = fmaf(a[0], b[0], r);
    r = fmaf(a[1], b[1], r);
    r = fmaf(a[2], b[2], r);
    r = fmaf(a[3], b[3], r);
    return r;
}
/* Math::Cross (Math.h:1627-1633). */
static inline void cross3(const float a[3], const float b[3], float o[3])
{
    float x = fmaf(a[1], b[2], -a[2] * b[1]);
    float y = fmaf(a[2], b[0], -a[0] * b[2]);
    float z = fmaf(a[0], b[1], -a[1] * b[0]);
    o[0] = x; o[1] = y; o[2] = z;
}

#define SMALL_EPS 1.0e-7f   /* MathConstants::SmallEpsilon (MathConstants.h:26) */

/* ------------------------------------------------------------------------ */
/* Ray::IntersectsTriangle (Source/Core/Ray.hpp:121-167)                     */
/* ------------------------------------------------------------------------ */
int orc_intersect_triangle(const float dir[3], const float pos[3],
                           const float v0[3], const float v1[3], const float v2[3],
                           int cull, float bary_out[3], float* t_out, int* backface_out)
{
    float e0[3] = { v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2] };
    float e1[3] = { v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2] };
    float p[3];
    cross3(dir, e1, p);
    float det = dot3(e0, p);

    int backfaceHit = (det < SMALL_EPS);
    int nearlyParallel = (fabsf(det) < SMALL_EPS);
    if((cull && backfaceHit) || nearlyParallel) return 0;

    float invDet = 1.0f / det;
    float tVec[3] = { pos[0] - v0[0], pos[1] - v0[1], pos[2] - v0[2] };
    float b0 = dot3(tVec, p) * invDet;
    if(b0 < 0.0f || b0 > 1.0f) return 0;

    float q[3];
    cross3(tVec, e0, q);
    float b1 = dot3(dir, q) * invDet;
    if((b1 < 0.0f) || (b1 + b0) > 1.0f) return 0;

    float t = dot3(e1, q) * invDet;
    if(t <= SMALL_EPS) return 0;

    float b2 = 1.0f - b0 - b1;
    bary_out[0] = b2; bary_out[1] = b0; bary_out[2] = b1;
    *t_out = t;
    *backface_out = backfaceHit;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Watertight ray/triangle test (S. Woop, C. Benthin, I. Wald, "Watertight   */
/* Ray/Triangle Intersection", JCGT 2(1), 2013): the ray is sheared so that   */
/* it runs along +z through the origin, and the triangle's scaled barycentric */
/* coordinates are 2D edge functions of the sheared vertices.  Two triangles */
/* that share an edge evaluate that edge's function from the same two        */
/* vertices, so a ray through the edge cannot miss both.  Edge functions that */
/* come out exactly 0 in float are recomputed in double.  The project's       */
/* opt-in alternative to MRay's Moller-Trumbore test: same outputs (MRay's   */
/* barycentric order, backface flag, t > SmallEpsilon), no epsilon on the    */
/* determinant.  Plain IEEE operations only (no fma).                        */
/* ------------------------------------------------------------------------ */
int orc_intersect_triangle_wt(const float dir[3], const float pos[3],
                              const float v0[3], const float v1[3], const float v2[3],
                              int cull, float bary_out[3], float* t_out, int* backface_out)
{
    /* largest direction component (first on ties), then the winding-keeping
     * order of the other two */
    float ax = fabsf(dir[0]), ay = fabsf(dir[1]), az = fabsf(dir[2]);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if(dir[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    float Sx = dir[kx] / dir[kz], Sy = dir[ky] / dir[kz], Sz = 1.0f / dir[kz];

    float A[3] = { v0[0] - pos[0], v0[1] - pos[1], v0[2] - pos[2] };
    float B[3] = { v1[0] - pos[0], v1[1] - pos[1], v1[2] - pos[2] };
    float C[3] = { v2[0] - pos[0], v2[1] - pos[1], v2[2] - pos[2] };
    float Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    float Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    float Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if(U == 0.0f || V == 0.0f || W == 0.0f)
    {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    int allNeg = (U <= 0.0f && V <= 0.0f && W <= 0.0f);
    int allPos = (U >= 0.0f && V >= 0.0f && W >= 0.0f);
    if(!allNeg && !allPos) return 0;
    float det = U + V + W;
    if(det == 0.0f) return 0;
    /* front face: the side MRay's Moller-Trumbore calls front (its det > 0) */
    int backfaceHit = (det < 0.0f);
    if(cull && backfaceHit) return 0;
    float Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if(t <= SMALL_EPS) return 0;
    bary_out[0] = U * rcp; bary_out[1] = V * rcp; bary_out[2] = W * rcp;
    *t_out = t;
    *backface_out = backfaceHit;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Ray::IntersectsAABB (Source/Core/Ray.hpp:192-219)                         */
/* ------------------------------------------------------------------------ */
int orc_intersect_aabb(const float dir[3], const float pos[3],
                       const float bmin[3], const float bmax[3],
                       const float tmm[2], float tout[2])
{
    float invD[3] = { 1.0f / dir[0], 1.0f / dir[1], 1.0f / dir[2] };
    float t0[3], t1[3];
    for(int i = 0; i < 3; i++) t0[i] = (bmin[i] - pos[i]) * invD[i];
    for(int i = 0; i < 3; i++) t1[i] = (bmax[i] - pos[i]) * invD[i];
    float o0 = tmm[0], o1 = tmm[1];
    for(int i = 0; i < 3; i++)
    {
        if(invD[i] < 0.0f) { float s = t0[i]; t0[i] = t1[i]; t1[i] = s; }
        o0 = smax(o0, smin(t0[i], t1[i]));
        o1 = smin(o1, smax(t0[i], t1[i]));
    }
    if(tout) { tout[0] = o0; tout[1] = o1; }
    return o1 >= o0;
}

/* ------------------------------------------------------------------------ */
/* Matrix3x4T::Inverse (Source/Core/Matrix.hpp:855-904)                       */
/* ------------------------------------------------------------------------ */
static inline float det2x2(float m00, float m01, float m10, float m11)
{
    return fmaf(m00, m11, -m01 * m10);
}
static void mat34_inverse_impl(const float m[12], float inv[12], int corrected)
{
    float s0 = det2x2(m[0], m[1], m[4], m[5]);
    float s1 = det2x2(m[0], m[2], m[4], m[6]);
    float s2 = det2x2(m[0], m[3], m[4], m[7]);
    float s3 = det2x2(m[1], m[2], m[5], m[6]);
    float s4 = det2x2(m[1], m[3], m[5], m[7]);
    float s5 = det2x2(m[2], m[3], m[6], m[7]);
    float c5 = m[10], c4 = m[9], c2 = m[8];
    float det = ((s0 * c5) - (s1 * c4) + (s3 * c2));
    float detInv = 1.0f / det;
    float r[12];
    r[0]  = (+m[5] * c5 - m[6] * c4);
    r[1]  = (-m[1] * c5 + m[2] * c4);
    r[2]  = s3;
    r[3]  = (-m[9] * s5 + m[10] * s4 - m[11] * s3);
    r[4]  = (-m[4] * c5 + m[6] * c2);
    r[5]  = (+m[0] * c5 - m[2] * c2);
    /* The reference stores +s1 here (Matrix.hpp:888); the cofactor is -s1.
     * corrected != 0 gives the mathematically correct inverse. */
    r[6]  = corrected ? -s1 : s1;
    r[7]  = (+m[8] * s5 - m[10] * s2 + m[11] * s1);
    r[8]  = (+m[4] * c4 - m[5] * c2);
    r[9]  = (-m[0] * c4 + m[1] * c2);
    r[10] = s0;
    r[11] = (-m[8] * s4 + m[9] * s2 - m[11] * s0);
    /* Matrix3x4T::operator*(T) multiplies every element. */
    for(int i = 0; i < 12; i++) inv[i] = r[i] * detInv;
}
void orc_mat34_inverse(const float m[12], float inv[12]) { mat34_inverse_impl(m, inv, 0); }
void orc_mat34_inverse_corrected(const float m[12], float inv[12]) { mat34_inverse_impl(m, inv, 1); }

/* Matrix3x4T::TransformRay (Matrix.hpp:906-913): dir via 3-term Dot,
 * pos via 4-term Dot with w = 1 (Matrix.hpp:763-788). */
void orc_transform_ray(const float m[12], const float dir[3], const float pos[3],
                       float dir_out[3], float pos_out[3])
{
    float d[3], p[3];
    for(int r = 0; r < 3; r++)
    {
        const float row3[3] = { m[4 * r + 0], m[4 * r + 1], m[4 * r + 2] };
        d[r] = dot3(row3, dir);
        const float row4[4] = { m[4 * r + 0], m[4 * r + 1], m[4 * r + 2], m[4 * r + 3] };
        const float v4[4] = { pos[0], pos[1], pos[2], 1.0f };
        p[r] = dot4(row4, v4);
    }
    memcpy(dir_out, d, sizeof(d));
    memcpy(pos_out, p, sizeof(p));
}

/* Matrix3x4T::TransformAABB (Matrix.hpp:915-931). */
void orc_transform_aabb(const float m[12], const float bmin[3], const float bmax[3],
                        float omin[3], float omax[3])
{
    float rmin[3] = { INFINITY, INFINITY, INFINITY };
    float rmax[3] = { -INFINITY, -INFINITY, -INFINITY };
    float vtx[4] = { 1.0f, 1.0f, 1.0f, 1.0f };
    for(unsigned i = 0; i < 8; i++)
    {
        for(unsigned j = 0; j < 3; j++)
            vtx[j] = ((i >> j) & 1u) ? bmax[j] : bmin[j];
        float o[4];
        for(int r = 0; r < 3; r++)
        {
            const float row4[4] = { m[4 * r + 0], m[4 * r + 1], m[4 * r + 2], m[4 * r + 3] };
            o[r] = dot4(row4, vtx);
        }
        /* vertex = M * vertex; the 4th component of a Matrix3x4 * Vector4
         * product keeps the input's w (Matrix.hpp:777-788: out = v, then xyz). */
        o[3] = vtx[3];
        for(int j = 0; j < 3; j++) vtx[j] = o[j];
        vtx[3] = o[3];
        for(int j = 0; j < 3; j++)
        {
            rmax[j] = smax(rmax[j], vtx[j]);
            rmin[j] = smin(rmin[j], vtx[j]);
        }
    }
    memcpy(omin, rmin, sizeof(rmin));
    memcpy(omax, rmax, sizeof(rmax));
}

/* MortonCode::Compose3D<uint64_t> (GraphicsFunctions.h:605-625). */
static inline uint64_t expand3d_u64(uint32_t v)
{
    uint64_t x = v;
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x001f00000000ffffull;
    x = (x | x << 16) & 0x001f0000ff0000ffull;
    x = (x | x << 8)  & 0x100f00f00f00f00full;
    x = (x | x << 4)  & 0x10c30c30c30c30c3ull;
    x = (x | x << 2)  & 0x1249249249249249ull;
    return x;
}
uint64_t orc_morton3d_u64(uint32_t x, uint32_t y, uint32_t z)
{
    return expand3d_u64(x) | (expand3d_u64(y) << 1) | (expand3d_u64(z) << 2);
}

/* Ray::Nudge (Ray.hpp:258-300), Ray Tracing Gems I ch. 6 offsets. */
void orc_nudge(const float pos[3], const float n[3], float out[3])
{
    const float ORIGIN = 1.0f / 32.0f;
    const float FLOAT_SCALE = 1.0f / 65536.0f;
    const float INT_SCALE = 256.0f;
    for(int i = 0; i < 3; i++)
    {
        int32_t ofi = (int32_t)(INT_SCALE * n[i]);
        int32_t pi;
        memcpy(&pi, &pos[i], 4);
        pi += (pos[i] < 0.0f) ? -ofi : ofi;
        float pf;
        memcpy(&pf, &pi, 4);
        out[i] = (fabsf(pos[i]) < ORIGIN) ? (pos[i] + FLOAT_SCALE * n[i]) : pf;
    }
}

/* Triangle::GetCenter (PrimitiveDefaultTriangle.hpp:106-113). */
void orc_tri_center(const float v0[3], const float v1[3], const float v2[3], float c[3])
{
    const float k = 0.333333333f;
    for(int i = 0; i < 3; i++)
        c[i] = (v0[i] * k + v1[i] * k) + v2[i] * k;
}

/* ------------------------------------------------------------------------ */
/* LBVH                                                                      */
/* ------------------------------------------------------------------------ */
#define IS_LEAF_BIT 0x80000000u          /* ChildIndex = KeyT<uint32_t,1,31> */
#define INVALID_CHILD 0xFFFFFFFFu
#define NO_PARENT 0xFFFFFFFFu

typedef struct { uint32_t left, right, parent; } lbvh_node;     /* AcceleratorLBVH.h:64-69 */
typedef struct { float mn[3], mx[3]; } aabb3;                   /* AcceleratorLBVH.h:73-77 */

typedef struct
{
    uint32_t    leafCount;
    uint32_t    nodeCount;
    lbvh_node*  nodes;
    aabb3*      boxes;
    uint32_t*   leafs;       /* leaf index -> primitive (local index) */
    aabb3       root;
} lbvh;

typedef struct
{
    float*      pos;         /* 3 * nv */
    uint32_t    nv;
    uint32_t*   idx;         /* 3 * nt */
    uint32_t    nt;
    uint32_t    primKeyBase;
    int         watertight;  /* triangle test: 0 Moller-Trumbore (MRay), 1 watertight */
    lbvh        bvh;
} orc_mesh;

typedef struct
{
    uint32_t    mesh;
    float       m[12];
    float       inv[12];
    int         cull;
    uint32_t    lmKey, transKey, accelKey;
    aabb3       world;
} orc_inst;

struct orc_scene
{
    orc_mesh*   meshes;  uint32_t meshCount, meshCap;
    orc_inst*   insts;   uint32_t instCount, instCap;
    lbvh        tlas;
    int         built;
    int         watertight;
};

typedef struct { uint64_t code; uint32_t idx; } code_idx;

/* Stable sort by code: CUB's (segmented) radix sort is stable, so equal codes
 * keep increasing original index order. */
static int cmp_code_idx(const void* a, const void* b)
{
    const code_idx* x = (const code_idx*)a;
    const code_idx* y = (const code_idx*)b;
    if(x->code < y->code) return -1;
    if(x->code > y->code) return 1;
    return (x->idx < y->idx) ? -1 : (x->idx > y->idx);
}

/* Delta (AcceleratorLBVH.cu:69-94). */
static inline int32_t lbvh_delta(const code_idx* c, int32_t n, int32_t i, int32_t j)
{
    if(j < 0 || j >= n) return -1;
    uint64_t l = c[i].code, r = c[j].code;
    if(l == r) { l = (uint64_t)i; r = (uint64_t)j; }
    uint64_t d = l ^ r;
    return d ? (int32_t)__builtin_clzll(d) : 64;
}

static int32_t div_up(int32_t a, int32_t b) { return (a + b - 1) / b; }

/* Builds an LBVH over n boxes with the given centers.  The quantisation
 * follows KCGenMortonCode (AcceleratorLBVH.cu:96-168): double-precision
 * scale by 2^21 / maxSide, lround of the float result, clamp to 21 bits. */
static int lbvh_build(lbvh* b, const aabb3* leafBoxes, const float* centers, uint32_t n)
{
    memset(b, 0, sizeof(*b));
    if(n == 0) return 0;
    b->leafCount = n;
    b->nodeCount = (n == 1) ? 1 : (n - 1);
    b->nodes = (lbvh_node*)malloc(sizeof(lbvh_node) * b->nodeCount);
    b->boxes = (aabb3*)malloc(sizeof(aabb3) * b->nodeCount);
    b->leafs = (uint32_t*)malloc(sizeof(uint32_t) * n);
    code_idx* ci = (code_idx*)malloc(sizeof(code_idx) * n);
    uint32_t* leafParent = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if(!b->nodes || !b->boxes || !b->leafs || !ci || !leafParent) return -1;

    /* Accelerator AABB = union of leaf AABBs (SegmentedTransformReduce). */
    aabb3 all = { { INFINITY, INFINITY, INFINITY }, { -INFINITY, -INFINITY, -INFINITY } };
    for(uint32_t i = 0; i < n; i++)
        for(int k = 0; k < 3; k++)
        {
            all.mn[k] = smin(all.mn[k], leafBoxes[i].mn[k]);
            all.mx[k] = smax(all.mx[k], leafBoxes[i].mx[k]);
        }
    b->root = all;
    float span[3] = { all.mx[0] - all.mn[0], all.mx[1] - all.mn[1], all.mx[2] - all.mn[2] };
    /* Vector::Maximum returns the index of the largest component (first on ties). */
    int mi = 0;
    if(span[1] > span[mi]) mi = 1;
    if(span[2] > span[mi]) mi = 2;
    float maxSide = span[mi];
    const double sliceCount = (double)(1ull << 21);
    double deltaRecip = sliceCount / (double)maxSide;
    const uint32_t lastValue = (1u << 21) - 1u;
    for(uint32_t i = 0; i < n; i++)
    {
        uint32_t q[3];
        for(int k = 0; k < 3; k++)
        {
            float diff = centers[3 * i + k] - all.mn[k];
            diff = smax(diff, 0.0f);
            float scaled = (float)((double)diff * deltaRecip);
            int32_t r = (int32_t)lroundf(scaled);
            uint32_t u = (uint32_t)r;
            /* Math::Clamp(v, 0u, last) = Min(Max(0, v), last) on unsigned. */
            u = (u < lastValue) ? u : lastValue;
            q[k] = u;
        }
        ci[i].code = orc_morton3d_u64(q[0], q[1], q[2]);
        ci[i].idx = i;
    }
    qsort(ci, n, sizeof(code_idx), cmp_code_idx);

    int32_t totalLeafs = (int32_t)n;
    int32_t totalNodes = (int32_t)b->nodeCount;
    if(totalLeafs == 1)
    {
        b->nodes[0].left = IS_LEAF_BIT | 0u;
        b->nodes[0].right = INVALID_CHILD;
        b->nodes[0].parent = NO_PARENT;
        leafParent[0] = 0;
        b->leafs[0] = ci[0].idx;
    }
    else
    {
        /* KCConstructLBVHInternalNodes (AcceleratorLBVH.cu:170-299). */
        for(int32_t i = 0; i < totalNodes; i++)
        {
            int32_t diff = lbvh_delta(ci, totalLeafs, i, i + 1) - lbvh_delta(ci, totalLeafs, i, i - 1);
            int32_t d = (diff < 0) ? -1 : 1;
            int32_t deltaMin = lbvh_delta(ci, totalLeafs, i, i - d);
            int32_t lMax = 2;
            while(lbvh_delta(ci, totalLeafs, i, i + lMax * d) > deltaMin) lMax <<= 1;
            int32_t l = 0;
            for(int32_t t = lMax >> 1; t != 0; t >>= 1)
                if(lbvh_delta(ci, totalLeafs, i, i + (l + t) * d) > deltaMin) l += t;
            int32_t j = i + l * d;
            int32_t s = 0;
            int32_t deltaNode = lbvh_delta(ci, totalLeafs, i, j);
            for(int32_t t = div_up(l, 2); t != 0; t = (t == 1) ? 0 : div_up(t, 2))
                if(lbvh_delta(ci, totalLeafs, i, i + (s + t) * d) > deltaNode) s += t;
            int32_t gamma = i + s * d + ((d < 0) ? d : 0);
            lbvh_node* me = &b->nodes[i];
            int32_t mn = (i < j) ? i : j, mx = (i > j) ? i : j;
            if(mn == gamma)
            {
                /* Leaf ids are positions in sorted order; the primitive is
                 * looked up through the sorted index list. */
                me->left = IS_LEAF_BIT | (uint32_t)gamma;
                leafParent[gamma] = (uint32_t)i;
            }
            else
            {
                me->left = (uint32_t)gamma;
                b->nodes[gamma].parent = (uint32_t)i;
            }
            if(mx == gamma + 1)
            {
                me->right = IS_LEAF_BIT | (uint32_t)(gamma + 1);
                leafParent[gamma + 1] = (uint32_t)i;
            }
            else
            {
                me->right = (uint32_t)(gamma + 1);
                b->nodes[gamma + 1].parent = (uint32_t)i;
            }
            if(i == 0) me->parent = NO_PARENT;
        }
        for(int32_t i = 0; i < totalLeafs; i++) b->leafs[i] = ci[i].idx;
    }

    /* KCUnionLBVHBoundingBoxes (AcceleratorLBVH.cu:301-435), sequentially:
     * a post-order walk gives the same unions. */
    if(totalLeafs == 1)
    {
        b->boxes[0] = leafBoxes[b->leafs[0]];
    }
    else
    {
        uint32_t* cnt = (uint32_t*)calloc(b->nodeCount, sizeof(uint32_t));
        for(int32_t li = 0; li < totalLeafs; li++)
        {
            uint32_t node = leafParent[li];
            while(node != NO_PARENT)
            {
                if(cnt[node]++ == 0) break;
                const lbvh_node* nd = &b->nodes[node];
                aabb3 lb, rb;
                lb = (nd->left & IS_LEAF_BIT) ? leafBoxes[b->leafs[nd->left & ~IS_LEAF_BIT]]
                                              : b->boxes[nd->left];
                rb = (nd->right & IS_LEAF_BIT) ? leafBoxes[b->leafs[nd->right & ~IS_LEAF_BIT]]
                                               : b->boxes[nd->right];
                for(int k = 0; k < 3; k++)
                {
                    b->boxes[node].mn[k] = smin(lb.mn[k], rb.mn[k]);
                    b->boxes[node].mx[k] = smax(lb.mx[k], rb.mx[k]);
                }
                node = nd->parent;
            }
        }
        free(cnt);
    }
    free(ci);
    free(leafParent);
    return 0;
}

static void lbvh_free(lbvh* b)
{
    free(b->nodes); free(b->boxes); free(b->leafs);
    memset(b, 0, sizeof(*b));
}

/* ------------------------------------------------------------------------ */
/* Scene                                                                     */
/* ------------------------------------------------------------------------ */
orc_scene* orc_scene_create(void)
{
    return (orc_scene*)calloc(1, sizeof(orc_scene));
}

void orc_scene_destroy(orc_scene* s)
{
    if(!s) return;
    for(uint32_t i = 0; i < s->meshCount; i++)
    {
        free(s->meshes[i].pos); free(s->meshes[i].idx);
        lbvh_free(&s->meshes[i].bvh);
    }
    free(s->meshes); free(s->insts);
    lbvh_free(&s->tlas);
    free(s);
}

int orc_scene_add_mesh(orc_scene* s, const float* pos, uint32_t nv,
                       const uint32_t* idx, uint32_t nt, uint32_t primKeyBase)
{
    if(!s || nt == 0 || nv == 0) return -1;
    for(uint64_t i = 0; i < 3ull * nt; i++) if(idx[i] >= nv) return -1;
    if(s->meshCount == s->meshCap)
    {
        uint32_t c = s->meshCap ? 2 * s->meshCap : 4;
        orc_mesh* m = (orc_mesh*)realloc(s->meshes, c * sizeof(orc_mesh));
        if(!m) return -1;
        s->meshes = m; s->meshCap = c;
    }
    orc_mesh* m = &s->meshes[s->meshCount];
    memset(m, 0, sizeof(*m));
    m->pos = (float*)malloc(sizeof(float) * 3 * nv);
    m->idx = (uint32_t*)malloc(sizeof(uint32_t) * 3 * nt);
    if(!m->pos || !m->idx) return -1;
    memcpy(m->pos, pos, sizeof(float) * 3 * nv);
    memcpy(m->idx, idx, sizeof(uint32_t) * 3 * nt);
    m->nv = nv; m->nt = nt; m->primKeyBase = primKeyBase; m->watertight = s->watertight;
    s->built = 0;
    return (int)s->meshCount++;
}

int orc_scene_add_instance(orc_scene* s, uint32_t mesh, const float mtx[12], uint32_t flags,
                           uint32_t lmKey, uint32_t transKey, uint32_t accelKey)
{
    if(!s || mesh >= s->meshCount) return -1;
    if(s->instCount == s->instCap)
    {
        uint32_t c = s->instCap ? 2 * s->instCap : 8;
        orc_inst* p = (orc_inst*)realloc(s->insts, c * sizeof(orc_inst));
        if(!p) return -1;
        s->insts = p; s->instCap = c;
    }
    orc_inst* in = &s->insts[s->instCount];
    memset(in, 0, sizeof(*in));
    in->mesh = mesh;
    memcpy(in->m, mtx, sizeof(float) * 12);
    mat34_inverse_impl(mtx, in->inv, (flags & ORC_INSTANCE_CORRECTED_INVERSE) ? 1 : 0);
    in->cull = (flags & ORC_INSTANCE_CULL_BACKFACE) ? 1 : 0;
    in->lmKey = lmKey; in->transKey = transKey; in->accelKey = accelKey;
    s->built = 0;
    return (int)s->instCount++;
}

static inline void tri_verts(const orc_mesh* m, uint32_t t, float v[3][3])
{
    for(int c = 0; c < 3; c++)
    {
        uint32_t vi = m->idx[3 * t + c];
        v[c][0] = m->pos[3 * vi + 0];
        v[c][1] = m->pos[3 * vi + 1];
        v[c][2] = m->pos[3 * vi + 2];
    }
}

int orc_scene_build(orc_scene* s)
{
    if(!s) return -1;
    for(uint32_t mi = 0; mi < s->meshCount; mi++)
    {
        orc_mesh* m = &s->meshes[mi];
        lbvh_free(&m->bvh);
        aabb3* boxes = (aabb3*)malloc(sizeof(aabb3) * m->nt);
        float* centers = (float*)malloc(sizeof(float) * 3 * m->nt);
        if(!boxes || !centers) return -1;
        for(uint32_t t = 0; t < m->nt; t++)
        {
            float v[3][3];
            tri_verts(m, t, v);
            /* Shape::Triangle::BoundingBox (ShapeFunctions.h:49-57). */
            for(int k = 0; k < 3; k++)
            {
                float mn = v[0][k], mx = v[0][k];
                mn = smin(mn, v[1][k]); mn = smin(mn, v[2][k]);
                mx = smax(mx, v[1][k]); mx = smax(mx, v[2][k]);
                boxes[t].mn[k] = mn; boxes[t].mx[k] = mx;
            }
            orc_tri_center(v[0], v[1], v[2], &centers[3 * t]);
        }
        int rc = lbvh_build(&m->bvh, boxes, centers, m->nt);
        free(boxes); free(centers);
        if(rc) return rc;
    }
    /* TLAS over instance world AABBs (AcceleratorLBVH.cu:537-740); leaf
     * centres are AABB centroids (KCGenAABBCenters, .cu:497-510). */
    lbvh_free(&s->tlas);
    if(s->instCount)
    {
        aabb3* boxes = (aabb3*)malloc(sizeof(aabb3) * s->instCount);
        float* centers = (float*)malloc(sizeof(float) * 3 * s->instCount);
        for(uint32_t i = 0; i < s->instCount; i++)
        {
            orc_inst* in = &s->insts[i];
            const aabb3* lb = &s->meshes[in->mesh].bvh.root;
            orc_transform_aabb(in->m, lb->mn, lb->mx, in->world.mn, in->world.mx);
            boxes[i] = in->world;
            for(int k = 0; k < 3; k++)
                centers[3 * i + k] = in->world.mn[k] + (in->world.mx[k] - in->world.mn[k]) * 0.5f;
        }
        int rc = lbvh_build(&s->tlas, boxes, centers, s->instCount);
        free(boxes); free(centers);
        if(rc) return rc;
    }
    s->built = 1;
    return 0;
}

void orc_scene_instance_inverse(const orc_scene* s, uint32_t inst, float inv[12])
{
    memcpy(inv, s->insts[inst].inv, sizeof(float) * 12);
}

void orc_scene_aabb(const orc_scene* s, float out[6])
{
    for(int k = 0; k < 3; k++) { out[k] = 3.0e38f; out[3 + k] = -3.0e38f; }
    for(uint32_t i = 0; i < s->instCount; i++)
        for(int k = 0; k < 3; k++)
        {
            const aabb3* w = &s->insts[i].world;
            out[k] = (w->mn[k] < out[k]) ? w->mn[k] : out[k];
            out[3 + k] = (out[3 + k] < w->mx[k]) ? w->mx[k] : out[3 + k];
        }
}

float orc_scene_diameter(const orc_scene* s)
{
    float b[6];
    orc_scene_aabb(s, b);
    float sx = b[3] - b[0], sz = b[5] - b[2];
    /* Math::Length of a Vector2: sqrt of the fused dot product */
    return sqrtf(fmaf(sz, sz, sx * sx));
}

void orc_scene_stats(const orc_scene* s, uint64_t out[4])
{
    uint64_t nodes = 0, leaves = 0;
    for(uint32_t i = 0; i < s->meshCount; i++)
    {
        nodes += s->meshes[i].bvh.nodeCount;
        leaves += s->meshes[i].bvh.leafCount;
    }
    out[0] = nodes; out[1] = leaves;
    out[2] = s->tlas.nodeCount; out[3] = s->tlas.leafCount;
}

/* ------------------------------------------------------------------------ */
/* Traversal                                                                 */
/* ------------------------------------------------------------------------ */
typedef struct
{
    int      hit;
    float    t;
    float    bary[3];
    uint32_t prim;       /* local primitive index */
} blas_hit;

/* IntersectionCheck (AcceleratorLBVH.hpp:225-299) for a triangle without
 * alpha map or media: MT with the instance's cull flag, then t in [tMin,tMax). */
static inline int isect_check(const orc_mesh* m, uint32_t prim, int cull,
                              const float dir[3], const float pos[3],
                              const float tmm[2], blas_hit* out)
{
    float v[3][3];
    tri_verts(m, prim, v);
    float bary[3], t; int bf;
    const int hit = m->watertight ? orc_intersect_triangle_wt(dir, pos, v[0], v[1], v[2], cull, bary, &t, &bf)
                                  : orc_intersect_triangle(dir, pos, v[0], v[1], v[2], cull, bary, &t, &bf);
    if(!hit) return 0;
    if(!((t >= tmm[0]) && (t < tmm[1]))) return 0;
    out->hit = 1; out->t = t;
    out->bary[0] = bary[0]; out->bary[1] = bary[1]; out->bary[2] = bary[2];
    out->prim = prim;
    return 1;
}

#define STACK_MAX (64 * 2 + 1)

/* TraverseLBVHStack (AcceleratorLBVH.hpp:111-166) with the ClosestHit /
 * FirstHit leaf functors (.hpp:327-410). */
static int blas_traverse(const orc_mesh* m, int cull, const float dir[3], const float pos[3],
                         float tmm[2], int anyHit, blas_hit* result)
{
    const lbvh* b = &m->bvh;
    uint32_t stack[STACK_MAX];
    int sp = 0;
    int found = 0;
    stack[sp++] = 0u;
    while(sp > 0)
    {
        uint32_t ni = stack[--sp];
        if(ni == INVALID_CHILD) continue;
        if(ni & IS_LEAF_BIT)
        {
            uint32_t prim = b->leafs[ni & ~IS_LEAF_BIT];
            blas_hit h;
            if(isect_check(m, prim, cull, dir, pos, tmm, &h))
            {
                if(anyHit) { *result = h; return 1; }
                if(h.t < tmm[1]) { *result = h; tmm[1] = h.t; found = 1; }
            }
        }
        else
        {
            const aabb3* bb = &b->boxes[ni];
            if(orc_intersect_aabb(dir, pos, bb->mn, bb->mx, tmm, NULL))
            {
                stack[sp++] = b->nodes[ni].right;
                stack[sp++] = b->nodes[ni].left;
            }
        }
    }
    return found;
}

/* Two-level cast.  The TLAS is walked left-first (the order of the GPU
 * bit-stack and of the CPU stack walk); at each instance leaf whose world
 * AABB the world ray enters within the current [tMin, tMax], the ray is moved
 * to local space with the inverse transform (AcceleratorWork.kt.h:213-224)
 * and the BLAS is traversed with the same [tMin, tMax]. */
typedef struct { int hit; float t; float bary[3]; uint32_t prim; uint32_t inst; } scene_hit;

static int scene_cast(const orc_scene* s, const orc_ray_gmem* r, int anyHit, scene_hit* out)
{
    if(s->instCount == 0) return 0;
    float tmm[2] = { r->tMin, r->tMax };
    const lbvh* T = &s->tlas;
    uint32_t stack[STACK_MAX];
    int sp = 0, found = 0;
    stack[sp++] = 0u;
    while(sp > 0)
    {
        uint32_t ni = stack[--sp];
        if(ni == INVALID_CHILD) continue;
        if(ni & IS_LEAF_BIT)
        {
            uint32_t ii = T->leafs[ni & ~IS_LEAF_BIT];
            const orc_inst* in = &s->insts[ii];
            if(!orc_intersect_aabb(r->dir, r->pos, in->world.mn, in->world.mx, tmm, NULL))
                continue;
            float ld[3], lp[3];
            orc_transform_ray(in->inv, r->dir, r->pos, ld, lp);
            blas_hit h; memset(&h, 0, sizeof(h));
            if(blas_traverse(&s->meshes[in->mesh], in->cull, ld, lp, tmm, anyHit, &h))
            {
                out->hit = 1; out->t = h.t; out->prim = h.prim; out->inst = ii;
                out->bary[0] = h.bary[0]; out->bary[1] = h.bary[1]; out->bary[2] = h.bary[2];
                found = 1;
                if(anyHit) return 1;
            }
        }
        else
        {
            const aabb3* bb = &T->boxes[ni];
            if(orc_intersect_aabb(r->dir, r->pos, bb->mn, bb->mx, tmm, NULL))
            {
                stack[sp++] = T->nodes[ni].right;
                stack[sp++] = T->nodes[ni].left;
            }
        }
    }
    return found;
}

/* Brute force over every instance and triangle (AcceleratorLinear semantics,
 * Source/Tracer/AcceleratorLinear.hpp:109-127) in instance order. */
static int scene_cast_linear(const orc_scene* s, const orc_ray_gmem* r, scene_hit* out)
{
    float tmm[2] = { r->tMin, r->tMax };
    int found = 0;
    for(uint32_t ii = 0; ii < s->instCount; ii++)
    {
        const orc_inst* in = &s->insts[ii];
        const orc_mesh* m = &s->meshes[in->mesh];
        float ld[3], lp[3];
        orc_transform_ray(in->inv, r->dir, r->pos, ld, lp);
        for(uint32_t p = 0; p < m->nt; p++)
        {
            blas_hit h;
            if(isect_check(m, p, in->cull, ld, lp, tmm, &h) && h.t < tmm[1])
            {
                tmm[1] = h.t;
                out->hit = 1; out->t = h.t; out->prim = p; out->inst = ii;
                out->bary[0] = h.bary[0]; out->bary[1] = h.bary[1]; out->bary[2] = h.bary[2];
                found = 1;
            }
        }
    }
    return found;
}

/* ------------------------------------------------------------------------ */
/* Threaded drivers                                                          */
/* ------------------------------------------------------------------------ */
typedef struct
{
    const orc_scene*    s;
    orc_ray_gmem*       rays;
    const orc_ray_gmem* crays;
    const uint32_t*     ridx;
    uint32_t            n;
    orc_hit_keys*       hits;
    orc_meta_hit*       meta;
    uint32_t*           hitInst;
    uint32_t*           vis;
    const uint32_t*     instIds;  /* mode 3: instance of each listed ray */
    int                 mode;     /* 0 closest, 1 linear, 2 visibility, 3 local */
    atomic_uint         next;
} cast_job;

#define CHUNK 256u

static void* cast_worker(void* arg)
{
    cast_job* j = (cast_job*)arg;
    for(;;)
    {
        uint32_t start = atomic_fetch_add(&j->next, CHUNK);
        if(start >= j->n) break;
        uint32_t end = (start + CHUNK < j->n) ? start + CHUNK : j->n;
        for(uint32_t i = start; i < end; i++)
        {
            uint32_t ri = j->ridx ? j->ridx[i] : i;
            if(j->mode == 2)
            {
                scene_hit h; memset(&h, 0, sizeof(h));
                if(scene_cast(j->s, &j->crays[ri], 1, &h))
                    atomic_fetch_and((atomic_uint*)&j->vis[ri >> 5], ~(1u << (ri & 31u)));
                continue;
            }
            scene_hit h; memset(&h, 0, sizeof(h));
            int got;
            if(j->mode == 3)
            {
                /* KCLocalRayCast (AcceleratorWork.kt.h:179-244): the listed
                 * instance only, the ray moved to its local space, ClosestHit
                 * of its BLAS in [tMin, tMax); no instance-box test. */
                const uint32_t ii = j->instIds[i];
                if(ii >= j->s->instCount) continue;
                const orc_inst* in = &j->s->insts[ii];
                float ld[3], lp[3];
                orc_transform_ray(in->inv, j->rays[ri].dir, j->rays[ri].pos, ld, lp);
                float tmm[2] = { j->rays[ri].tMin, j->rays[ri].tMax };
                blas_hit bh; memset(&bh, 0, sizeof(bh));
                got = blas_traverse(&j->s->meshes[in->mesh], in->cull, ld, lp, tmm, 0, &bh);
                if(got)
                {
                    h.hit = 1; h.t = bh.t; h.prim = bh.prim; h.inst = ii;
                    h.bary[0] = bh.bary[0]; h.bary[1] = bh.bary[1]; h.bary[2] = bh.bary[2];
                }
            }
            else
                got = (j->mode == 0) ? scene_cast(j->s, &j->rays[ri], 0, &h)
                                     : scene_cast_linear(j->s, &j->rays[ri], &h);
            if(!got)
            {
                if(j->hitInst) j->hitInst[ri] = 0xFFFFFFFFu;
                continue;
            }
            const orc_inst* in = &j->s->insts[h.inst];
            const orc_mesh* m = &j->s->meshes[in->mesh];
            j->hits[ri].primKey = m->primKeyBase + h.prim;
            j->hits[ri].lmKey = in->lmKey;
            j->hits[ri].transKey = in->transKey;
            j->hits[ri].accelKey = in->accelKey;
            j->rays[ri].tMax = h.t;
            j->meta[ri].bary[0] = h.bary[0];
            j->meta[ri].bary[1] = h.bary[1];
            if(j->hitInst) j->hitInst[ri] = h.inst;
        }
    }
    return NULL;
}

static void run_job(cast_job* j, int nthreads)
{
    if(nthreads < 1) nthreads = 1;
    if(nthreads > 256) nthreads = 256;
    atomic_init(&j->next, 0u);
    pthread_t th[256];
    int started = 0;
    for(int t = 1; t < nthreads; t++)
        if(pthread_create(&th[started], NULL, cast_worker, j) == 0) started++;
    cast_worker(j);
    for(int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

void orc_cast_closest(const orc_scene* s, orc_ray_gmem* rays, const uint32_t* ridx,
                      uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta,
                      uint32_t* hitInst, int nthreads)
{
    cast_job j; memset(&j, 0, sizeof(j));
    j.s = s; j.rays = rays; j.ridx = ridx; j.n = n; j.hits = hits; j.meta = meta;
    j.hitInst = hitInst; j.mode = 0;
    run_job(&j, nthreads);
}

void orc_cast_closest_linear(const orc_scene* s, orc_ray_gmem* rays, const uint32_t* ridx,
                             uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta,
                             uint32_t* hitInst, int nthreads)
{
    cast_job j; memset(&j, 0, sizeof(j));
    j.s = s; j.rays = rays; j.ridx = ridx; j.n = n; j.hits = hits; j.meta = meta;
    j.hitInst = hitInst; j.mode = 1;
    run_job(&j, nthreads);
}

void orc_cast_local(const orc_scene* s, orc_ray_gmem* rays, const uint32_t* ridx, const uint32_t* inst_ids,
                    uint32_t n, orc_hit_keys* hits, orc_meta_hit* meta, int nthreads)
{
    cast_job j; memset(&j, 0, sizeof(j));
    j.s = s; j.rays = rays; j.ridx = ridx; j.instIds = inst_ids; j.n = n; j.hits = hits; j.meta = meta;
    j.mode = 3;
    run_job(&j, nthreads);
}

void orc_cast_visibility(const orc_scene* s, const orc_ray_gmem* rays, const uint32_t* ridx,
                         uint32_t n, uint32_t* vis, int nthreads)
{
    /* KCSetIsVisibleIndirect: every listed ray starts visible. */
    for(uint32_t i = 0; i < n; i++)
    {
        uint32_t ri = ridx ? ridx[i] : i;
        vis[ri >> 5] |= (1u << (ri & 31u));
    }
    cast_job j; memset(&j, 0, sizeof(j));
    j.s = s; j.crays = rays; j.ridx = ridx; j.n = n; j.vis = vis; j.mode = 2;
    run_job(&j, nthreads);
}

/* Selects the triangle test of every mesh of the scene (0 Moller-Trumbore,
 * MRay's; 1 the watertight test above). */
void orc_scene_set_watertight(orc_scene* s, int on)
{
    s->watertight = on;
    for(uint32_t i = 0; i < s->meshCount; i++) s->meshes[i].watertight = on;
}
