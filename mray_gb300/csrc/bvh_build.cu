// bvh_build.cu -- GPU builder of the 8-wide compressed BVH.
//
// Replaces MRay's LBVH construction (Source/Tracer/AcceleratorLBVH.hpp:584-899,
// Source/Tracer/AcceleratorLBVH.cu:96-435, .cu:537-740) with:
//   1. leaf boxes + centroid bounds          (k_leaf_boxes_*)
//   2. 63-bit Morton codes in fp32/int       (k_morton; the reference quantises
//      in double, which is slow on this part and changes only the tree shape)
//   3. radix sort of (code, leaf)            (CUB DeviceRadixSort, build only)
//   4. Karras 2012 binary radix tree         (k_karras)
//   5. bottom-up boxes + leaf counts         (k_bottom_up; fence + atomic)
//   6. top-down collapse to 8-wide nodes     (k_collapse, one launch per level)
//      with 8-bit quantised child boxes, up to `maxLeaf` primitives per leaf
//      child, children placed in slots by direction so that traversal visits
//      them near-to-far (Ylitie, Karras, Laine 2017).
// Closest-hit results do not depend on the tree shape: every box is inflated
// outward (see `inflate`) so no box can cull a hit the triangle test accepts.
#include "mrg_build.h"
#include "mrg_device.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <vector>
#include <cstring>

namespace mrg {

namespace {

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kNoParent = 0xFFFFFFFFu;
constexpr int kTPB = 256;

struct BinNode
{
    uint32_t left, right, parent, leafCount;
};

struct BoxF
{
    float mn[3];
    float mx[3];
};

// One mesh of a batched BLAS build: its triangles are leaves
// [first, first + count) of the concatenated leaf arrays.
struct MeshSeg
{
    const float*    pos;
    const uint32_t* idx;
    uint32_t        first;
    uint32_t        count;
    uint32_t        primKeyBase;
    uint32_t        maxLeaf;
    float           inflate;
    uint32_t        rawVerts;   // 1: triangle records hold v0, v1, v2 (watertight test)
};

// Mesh of sorted leaf position p in a batched build (firsts: nMesh + 1 offsets).
__device__ __forceinline__ uint32_t mesh_of(const uint32_t* __restrict__ firsts, uint32_t nMesh, uint32_t p)
{
    uint32_t lo = 0, hi = nMesh;      // firsts[lo] <= p < firsts[hi]
    while(hi - lo > 1u)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if(firsts[mid] <= p) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t f2ord(float f)
{
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Triangle leaves: box of the three vertices, centroid bounds (ordered ints).
__global__ void k_leaf_boxes_tri(const float* __restrict__ pos, const uint32_t* __restrict__ idx,
                                 uint32_t n, BoxF* __restrict__ boxes, float* __restrict__ cent,
                                 uint32_t* __restrict__ cbounds)
{
    __shared__ uint32_t sb[6];
    if(threadIdx.x < 6) sb[threadIdx.x] = (threadIdx.x < 3) ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n)
    {
        uint32_t a = idx[3 * i], b = idx[3 * i + 1], c = idx[3 * i + 2];
        BoxF bx;
        for(int k = 0; k < 3; k++)
        {
            float va = pos[3 * a + k], vb = pos[3 * b + k], vc = pos[3 * c + k];
            bx.mn[k] = fminf(va, fminf(vb, vc));
            bx.mx[k] = fmaxf(va, fmaxf(vb, vc));
            float cc = 0.5f * (bx.mn[k] + bx.mx[k]);
            cent[3 * i + k] = cc;
            atomicMin(&sb[k], f2ord(cc));
            atomicMax(&sb[3 + k], f2ord(cc));
        }
        boxes[i] = bx;
    }
    __syncthreads();
    if(threadIdx.x < 3) atomicMin(&cbounds[threadIdx.x], sb[threadIdx.x]);
    else if(threadIdx.x < 6) atomicMax(&cbounds[threadIdx.x], sb[threadIdx.x]);
}

// Box leaves (TLAS over instance boxes).
__global__ void k_leaf_boxes_given(const BoxF* __restrict__ in, uint32_t n,
                                   BoxF* __restrict__ boxes, float* __restrict__ cent,
                                   uint32_t* __restrict__ cbounds)
{
    __shared__ uint32_t sb[6];
    if(threadIdx.x < 6) sb[threadIdx.x] = (threadIdx.x < 3) ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n)
    {
        BoxF bx = in[i];
        boxes[i] = bx;
        for(int k = 0; k < 3; k++)
        {
            float cc = 0.5f * (bx.mn[k] + bx.mx[k]);
            cent[3 * i + k] = cc;
            atomicMin(&sb[k], f2ord(cc));
            atomicMax(&sb[3 + k], f2ord(cc));
        }
    }
    __syncthreads();
    if(threadIdx.x < 3) atomicMin(&cbounds[threadIdx.x], sb[threadIdx.x]);
    else if(threadIdx.x < 6) atomicMax(&cbounds[threadIdx.x], sb[threadIdx.x]);
}

__device__ __forceinline__ uint64_t expand21(uint32_t v)
{
    uint64_t x = v & 0x1FFFFFu;
    x = (x | x << 32) & 0x001F00000000FFFFull;
    x = (x | x << 16) & 0x001F0000FF0000FFull;
    x = (x | x << 8)  & 0x100F00F00F00F00Full;
    x = (x | x << 4)  & 0x10C30C30C30C30C3ull;
    x = (x | x << 2)  & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float* __restrict__ cent, const uint32_t* __restrict__ cbounds,
                         uint32_t n, uint64_t* __restrict__ codes, uint32_t* __restrict__ ids)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    uint32_t q[3];
    for(int k = 0; k < 3; k++)
    {
        float lo = ord2f(cbounds[k]), hi = ord2f(cbounds[3 + k]);
        float ext = hi - lo;
        float s = (ext > 0.0f) ? (2097151.0f / ext) : 0.0f;
        float v = (cent[3 * i + k] - lo) * s;
        v = fminf(fmaxf(v, 0.0f), 2097151.0f);
        q[k] = (uint32_t)v;
    }
    codes[i] = expand21(q[0]) | (expand21(q[1]) << 1) | (expand21(q[2]) << 2);
    ids[i] = i;
}

// Batched BLAS build, leaves of every mesh: box, centroid, per-mesh centroid
// bounds.  A block whose leaves all belong to one mesh reduces in shared
// memory first; a block that straddles meshes uses per-leaf atomics.
__global__ void k_leaf_boxes_multi(const MeshSeg* __restrict__ segs, const uint32_t* __restrict__ firsts,
                                   uint32_t nMesh, uint32_t n, BoxF* __restrict__ boxes, float* __restrict__ cent,
                                   uint32_t* __restrict__ cbounds, uint32_t* __restrict__ leafMesh)
{
    __shared__ uint32_t sb[6];
    __shared__ uint32_t blockMesh;
    const uint32_t b0 = blockIdx.x * blockDim.x;
    const uint32_t b1 = min(n, b0 + blockDim.x) - 1u;
    if(threadIdx.x < 6) sb[threadIdx.x] = (threadIdx.x < 3) ? 0xFFFFFFFFu : 0u;
    if(threadIdx.x == 0)
    {
        const uint32_t m0 = mesh_of(firsts, nMesh, b0), m1 = mesh_of(firsts, nMesh, b1);
        blockMesh = (m0 == m1) ? m0 : 0xFFFFFFFFu;
    }
    __syncthreads();
    const uint32_t i = b0 + threadIdx.x;
    if(i < n)
    {
        const uint32_t m = mesh_of(firsts, nMesh, i);
        const MeshSeg& sg = segs[m];
        const uint32_t t = i - sg.first;
        const uint32_t a = sg.idx[3 * t], b = sg.idx[3 * t + 1], c = sg.idx[3 * t + 2];
        BoxF bx;
        for(int k = 0; k < 3; k++)
        {
            const float va = sg.pos[3 * a + k], vb = sg.pos[3 * b + k], vc = sg.pos[3 * c + k];
            bx.mn[k] = fminf(va, fminf(vb, vc));
            bx.mx[k] = fmaxf(va, fmaxf(vb, vc));
            const float cc = 0.5f * (bx.mn[k] + bx.mx[k]);
            cent[3 * i + k] = cc;
            if(blockMesh != 0xFFFFFFFFu)
            {
                atomicMin(&sb[k], f2ord(cc));
                atomicMax(&sb[3 + k], f2ord(cc));
            }
            else
            {
                atomicMin(&cbounds[6 * m + k], f2ord(cc));
                atomicMax(&cbounds[6 * m + 3 + k], f2ord(cc));
            }
        }
        boxes[i] = bx;
        leafMesh[i] = m;
    }
    __syncthreads();
    if(blockMesh != 0xFFFFFFFFu)
    {
        if(threadIdx.x < 3) atomicMin(&cbounds[6 * blockMesh + threadIdx.x], sb[threadIdx.x]);
        else if(threadIdx.x < 6) atomicMax(&cbounds[6 * blockMesh + threadIdx.x], sb[threadIdx.x]);
    }
}

// Keys of a batched build: mesh id above a Morton code of `bits` bits per
// axis, quantised in the mesh's own centroid bounds.  With one mesh (no id
// bits, 21 bits per axis) the keys equal k_morton's.
__global__ void k_morton_multi(const float* __restrict__ cent, const uint32_t* __restrict__ cbounds,
                               const uint32_t* __restrict__ leafMesh, uint32_t n, uint32_t bits,
                               uint64_t* __restrict__ codes, uint32_t* __restrict__ ids)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t m = leafMesh[i];
    const float qmax = (float)((1u << bits) - 1u);
    uint32_t q[3];
    for(int k = 0; k < 3; k++)
    {
        const float lo = ord2f(cbounds[6 * m + k]), hi = ord2f(cbounds[6 * m + 3 + k]);
        const float ext = hi - lo;
        const float sc = (ext > 0.0f) ? (qmax / ext) : 0.0f;
        float v = (cent[3 * i + k] - lo) * sc;
        v = fminf(fmaxf(v, 0.0f), qmax);
        q[k] = (uint32_t)v;
    }
    const uint64_t morton = expand21(q[0]) | (expand21(q[1]) << 1) | (expand21(q[2]) << 2);
    codes[i] = ((uint64_t)m << (3u * bits)) | morton;
    ids[i] = i;
}

// Root box of every mesh of a batched build (a leaf root for one-triangle meshes).
__global__ void k_mesh_boxes(const uint32_t* __restrict__ meshRoot, uint32_t nMesh, const BoxF* __restrict__ nodeBoxes,
                             const BoxF* __restrict__ leafBoxes, const uint32_t* __restrict__ sortedIds, uint32_t n,
                             BoxF* __restrict__ out, uint32_t* errorFlag)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if(m >= nMesh) return;
    const uint32_t r = meshRoot[m];
    const uint32_t ix = r & ~kLeafBit;
    if(r == kNoParent || ((r & kLeafBit) ? ix >= n : ix + 1u >= n)) { atomicOr(errorFlag, 1u); return; }
    out[m] = (r & kLeafBit) ? leafBoxes[sortedIds[ix]] : nodeBoxes[ix];
}

__device__ __forceinline__ int k_delta(const uint64_t* __restrict__ c, int n, int i, int j)
{
    if(j < 0 || j >= n) return -1;
    uint64_t a = c[i], b = c[j];
    if(a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll(a ^ b);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs".  In a
// batched build (firsts != null) the mesh id heads every key, so each mesh's
// leaves form one subtree; the node whose range is exactly a mesh's leaves
// is recorded as that mesh's root.
__global__ void k_karras(const uint64_t* __restrict__ codes, int n, BinNode* __restrict__ nodes,
                         uint32_t* __restrict__ leafParent, const uint32_t* __restrict__ firsts,
                         uint32_t nMesh, uint32_t* __restrict__ meshRoot)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n - 1) return;
    int d = (k_delta(codes, n, i, i + 1) - k_delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = k_delta(codes, n, i, i - d);
    int lmax = 2;
    while(k_delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for(int t = lmax >> 1; t >= 1; t >>= 1)
        if(k_delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = k_delta(codes, n, i, j);
    int s = 0;
    int t = l;
    do
    {
        t = (t + 1) >> 1;
        if(k_delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while(t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    BinNode& me = nodes[i];
    if(lo == gamma) { me.left = kLeafBit | (uint32_t)gamma; leafParent[gamma] = (uint32_t)i; }
    else            { me.left = (uint32_t)gamma; nodes[gamma].parent = (uint32_t)i; }
    if(hi == gamma + 1) { me.right = kLeafBit | (uint32_t)(gamma + 1); leafParent[gamma + 1] = (uint32_t)i; }
    else                { me.right = (uint32_t)(gamma + 1); nodes[gamma + 1].parent = (uint32_t)i; }
    if(i == 0) me.parent = kNoParent;
    if(firsts)
    {
        const uint32_t m = mesh_of(firsts, nMesh, (uint32_t)lo);
        if((uint32_t)lo == firsts[m] && (uint32_t)hi + 1u == firsts[m + 1]) meshRoot[m] = (uint32_t)i;
    }
}

// Bottom-up boxes and leaf counts.  The second thread to reach a node merges
// its children.  Writers fence before the counter atomic; readers of another
// thread's node box load through L2 (__ldcg) since L1 is not coherent.
__global__ void k_bottom_up(const uint32_t* __restrict__ leafParent, const uint32_t* __restrict__ sortedIds,
                            const BoxF* __restrict__ leafBoxes, BinNode* nodes, BoxF* nodeBoxes,
                            uint32_t* counters, int n, uint32_t* errorFlag)
{
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if(li >= n) return;
    const uint32_t nInt = (uint32_t)(n - 1);
    uint32_t p = leafParent[li];
    for(int guard = 0; p != kNoParent; guard++)
    {
        if(p >= nInt || guard > n) { atomicOr(errorFlag, 1u); return; }
        uint32_t old = atomicAdd(&counters[p], 1u);
        if(old == 0) return;
        __threadfence();
        uint32_t ch[2] = { __ldcg(&nodes[p].left), __ldcg(&nodes[p].right) };
        for(int c = 0; c < 2; c++)
        {
            const bool leaf = (ch[c] & kLeafBit) != 0u;
            const uint32_t ix = ch[c] & ~kLeafBit;
            if((leaf && ix >= (uint32_t)n) || (!leaf && ix >= nInt)) { atomicOr(errorFlag, 1u); return; }
        }
        BoxF b;
        uint32_t cnt = 0;
        for(int k = 0; k < 3; k++) { b.mn[k] = FLT_MAX; b.mx[k] = -FLT_MAX; }
        for(int c = 0; c < 2; c++)
        {
            BoxF cb;
            if(ch[c] & kLeafBit)
            {
                cb = leafBoxes[sortedIds[ch[c] & ~kLeafBit]];
                cnt += 1;
            }
            else
            {
                const float* src = reinterpret_cast<const float*>(&nodeBoxes[ch[c]]);
                for(int k = 0; k < 3; k++) { cb.mn[k] = __ldcg(src + k); cb.mx[k] = __ldcg(src + 3 + k); }
                cnt += __ldcg(&nodes[ch[c]].leafCount);
            }
            for(int k = 0; k < 3; k++) { b.mn[k] = fminf(b.mn[k], cb.mn[k]); b.mx[k] = fmaxf(b.mx[k], cb.mx[k]); }
        }
        nodeBoxes[p] = b;
        nodes[p].leafCount = cnt;
        __threadfence();
        p = __ldcg(&nodes[p].parent);
    }
}

// ---------------------------------------------------------------------------
// SAH-optimal collapse to 8-wide nodes (Ylitie, Karras and Laine 2017,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs",
// section 3.1).  Bottom up over the binary tree, C(n, i) is the least SAH
// cost of the subtree at n written as a forest of at most i roots (i = 1..8):
//   C(n, 1) = min(leaf cost cPrim * P(n) * A(n) where the subtree fits a
//             leaf child (P(n) <= maxLeaf), cNode * A(n) + D(n, 8): n as a
//             wide node of its own);
//   C(n, i) = min(C(n, i - 1), D(n, i)),
//   D(n, i) = min over k of C(left, k) + C(right, i - k);
// a binary leaf costs cPrim * A for every i.  The collapse then expands each
// wide node's root by its recorded choices instead of greedily opening the
// largest child.
// ---------------------------------------------------------------------------
struct WideCost
{
    float   c[8];          // C(n, i), i = 1..8
    uint8_t split[8];      // for i >= 2: 0 = C(n, i - 1), else k of D(n, i)
    uint32_t fullSplit;    // k of D(n, 8): the split of n opened as a wide node
    uint32_t asLeaf;       // 1: n is a leaf child (it fits one and that is cheaper)
};

__device__ __forceinline__ float ref_cost(const WideCost* costs, const BoxF* __restrict__ leafBoxes,
                                          const uint32_t* __restrict__ sortedIds, uint32_t ref, int i, float cPrim)
{
    if(ref & kLeafBit)
    {
        const BoxF b = leafBoxes[sortedIds[ref & ~kLeafBit]];
        const float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
        return cPrim * (dx * dy + dy * dz + dz * dx);
    }
    return __ldcg(&costs[ref].c[i - 1]);
}

__global__ void k_wide_cost(const uint32_t* __restrict__ leafParent, const uint32_t* __restrict__ sortedIds,
                            const BoxF* __restrict__ leafBoxes, const BinNode* __restrict__ nodes,
                            const BoxF* __restrict__ nodeBoxes, WideCost* costs, uint32_t* counters, int n,
                            const uint32_t* __restrict__ firsts, const MeshSeg* __restrict__ segs, uint32_t nMesh,
                            uint32_t maxLeaf, float cNode, float cPrim, uint32_t* errorFlag)
{
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if(li >= n) return;
    const uint32_t nInt = (uint32_t)(n - 1);
    const uint32_t ml = segs ? segs[mesh_of(firsts, nMesh, (uint32_t)li)].maxLeaf : maxLeaf;
    uint32_t p = leafParent[li];
    for(int guard = 0; p != kNoParent; guard++)
    {
        if(p >= nInt || guard > n) { atomicOr(errorFlag, 1u); return; }
        if(atomicAdd(&counters[p], 1u) == 0u) return;
        __threadfence();
        const uint32_t ch[2] = { nodes[p].left, nodes[p].right };
        for(int c = 0; c < 2; c++)
        {
            const bool leaf = (ch[c] & kLeafBit) != 0u;
            const uint32_t ix = ch[c] & ~kLeafBit;
            if((leaf && ix >= (uint32_t)n) || (!leaf && ix >= nInt)) { atomicOr(errorFlag, 1u); return; }
        }
        float cl[8], cr[8];
        for(int i = 0; i < 8; i++)
        {
            cl[i] = ref_cost(costs, leafBoxes, sortedIds, ch[0], i + 1, cPrim);
            cr[i] = ref_cost(costs, leafBoxes, sortedIds, ch[1], i + 1, cPrim);
        }
        WideCost w;
        float d[8];
        uint8_t kd[8];
        d[0] = __int_as_float(0x7f800000);
        kd[0] = 0;
        for(int i = 2; i <= 8; i++)
        {
            float best = __int_as_float(0x7f800000);
            int bk = 1;
            for(int k = 1; k < i; k++)
            {
                const float v = cl[k - 1] + cr[i - k - 1];
                if(v < best) { best = v; bk = k; }
            }
            d[i - 1] = best;
            kd[i - 1] = (uint8_t)bk;
        }
        const BoxF b = nodeBoxes[p];
        const float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
        const float area = dx * dy + dy * dz + dz * dx;
        const uint32_t cnt = nodes[p].leafCount;
        const float cInt = cNode * area + d[7];
        const float cLeaf = cPrim * (float)cnt * area;
        w.asLeaf = (cnt <= ml && cLeaf <= cInt) ? 1u : 0u;
        w.c[0] = w.asLeaf ? cLeaf : cInt;
        w.split[0] = 0;
        for(int i = 2; i <= 8; i++)
        {
            if(d[i - 1] < w.c[i - 2]) { w.c[i - 1] = d[i - 1]; w.split[i - 1] = kd[i - 1]; }
            else { w.c[i - 1] = w.c[i - 2]; w.split[i - 1] = 0; }
        }
        w.fullSplit = kd[7];
        costs[p] = w;
        __threadfence();
        p = nodes[p].parent;
    }
}

// ---------------------------------------------------------------------------
// PLOC (Meister & Bittner 2018, "Parallel Locally-Ordered Clustering for
// Bounding Volume Hierarchy Construction"): clusters in Morton order merge
// with their mutual nearest neighbour (smallest union surface area) inside a
// window of +-kPlocRadius, until one cluster remains.  Higher quality than
// the Karras radix tree, so traversal visits fewer nodes.
// ---------------------------------------------------------------------------
constexpr int kPlocRadius = 16;

__device__ __forceinline__ float union_area(const BoxF& a, const BoxF& b)
{
    const float dx = fmaxf(a.mx[0], b.mx[0]) - fminf(a.mn[0], b.mn[0]);
    const float dy = fmaxf(a.mx[1], b.mx[1]) - fminf(a.mn[1], b.mn[1]);
    const float dz = fmaxf(a.mx[2], b.mx[2]) - fminf(a.mn[2], b.mn[2]);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_init(const uint32_t* __restrict__ sortedIds, const BoxF* __restrict__ leafBoxes, uint32_t n,
                            uint32_t* __restrict__ C, BoxF* __restrict__ CB, uint32_t* __restrict__ CC)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    C[i] = kLeafBit | i;
    CB[i] = leafBoxes[sortedIds[i]];
    CC[i] = 1u;
}

__global__ void k_ploc_nearest(const BoxF* __restrict__ CB, uint32_t n, uint32_t* __restrict__ nn)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const BoxF me = CB[i];
    const uint32_t lo = (i > (uint32_t)kPlocRadius) ? i - kPlocRadius : 0u;
    const uint32_t hi = min(n - 1u, i + (uint32_t)kPlocRadius);
    uint32_t best = 0xFFFFFFFFu;
    float bestA = FLT_MAX;
    for(uint32_t j = lo; j <= hi; j++)
    {
        if(j == i) continue;
        const float a = union_area(me, CB[j]);
        if(a < bestA || (a == bestA && j < best)) { bestA = a; best = j; }
    }
    nn[i] = best;
}

// Mutual nearest neighbours merge into a new node at the lower position;
// the higher one is dropped (keep = 0).
__global__ void k_ploc_merge(const uint32_t* __restrict__ C, const BoxF* __restrict__ CB,
                             const uint32_t* __restrict__ CC, const uint32_t* __restrict__ nn, uint32_t n,
                             BinNode* __restrict__ nodes, BoxF* __restrict__ nodeBoxes, uint32_t* nextNode,
                             uint32_t capNodes, uint32_t* __restrict__ outC, BoxF* __restrict__ outCB,
                             uint32_t* __restrict__ outCC, uint32_t* __restrict__ keep, uint32_t* errorFlag)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const uint32_t j = nn[i];
    const bool mutual = (j < n) && nn[j] == i;
    if(mutual && j < i) { keep[i] = 0u; return; }
    keep[i] = 1u;
    if(!mutual) { outC[i] = C[i]; outCB[i] = CB[i]; outCC[i] = CC[i]; return; }
    const uint32_t m = atomicAdd(nextNode, 1u);
    if(m >= capNodes) { atomicOr(errorFlag, 1u); outC[i] = C[i]; outCB[i] = CB[i]; outCC[i] = CC[i]; return; }
    const BoxF a = CB[i], b = CB[j];
    BoxF u;
    for(int k = 0; k < 3; k++) { u.mn[k] = fminf(a.mn[k], b.mn[k]); u.mx[k] = fmaxf(a.mx[k], b.mx[k]); }
    BinNode nd;
    nd.left = C[i]; nd.right = C[j]; nd.parent = kNoParent; nd.leafCount = CC[i] + CC[j];
    nodes[m] = nd;
    nodeBoxes[m] = u;
    outC[i] = m; outCB[i] = u; outCC[i] = nd.leafCount;
}

__global__ void k_ploc_compact(const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, uint32_t n,
                               const uint32_t* __restrict__ inC, const BoxF* __restrict__ inCB,
                               const uint32_t* __restrict__ inCC, uint32_t* __restrict__ C, BoxF* __restrict__ CB,
                               uint32_t* __restrict__ CC)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n || !keep[i]) return;
    const uint32_t o = pos[i];
    C[o] = inC[i]; CB[o] = inCB[i]; CC[o] = inCC[i];
}

struct CollapseArgs
{
    const MeshSeg*  segs;       // batched builds: per-mesh payload, leaf size, inflation (else null)
    const BinNode*  nodes;
    const BoxF*     nodeBoxes;
    const BoxF*     leafBoxes;
    const uint32_t* sortedIds;
    // triangle payload (kind 0) or leaf ids (kind 1)
    const float*    pos;
    const uint32_t* idx;
    uint32_t        primKeyBase;
    int             kind;
    uint32_t        maxLeaf;
    float           inflate;
    uint32_t        rawVerts;   // single builds: 1 = records hold v0, v1, v2
    // outputs
    WideNode*       wnodes;
    TriRecord*      tris;
    uint32_t*       leafIds;
    uint32_t*       counters;   // [0] nodes, [1] leaf payloads, [2] next-queue size, [3] error
    uint32_t        leafCount;  // leaves (payload capacity)
    uint32_t        wideCap;    // wide node / queue capacity
    const WideCost* costs;      // SAH-optimal collapse choices (k_wide_cost), or null: greedy
    uint32_t        sahMaxLeaf; // the choices apply to wide nodes whose leaf size is at most this
};

// Child references are validated before every dereference: a malformed tree
// sets counters[3] and yields an empty box instead of an out-of-range read.
__device__ __forceinline__ bool ref_ok(const CollapseArgs& a, uint32_t ref)
{
    const bool ok = (ref & kLeafBit) ? ((ref & ~kLeafBit) < a.leafCount)
                                     : (ref < (a.leafCount > 1 ? a.leafCount - 1 : 1));
    if(!ok) atomicOr(&a.counters[3], 1u);
    return ok;
}

__device__ __forceinline__ void ref_box(const CollapseArgs& a, uint32_t ref, BoxF& b, uint32_t& cnt)
{
    if(!ref_ok(a, ref))
    {
        for(int k = 0; k < 3; k++) { b.mn[k] = 0.0f; b.mx[k] = 0.0f; }
        cnt = 1;
        return;
    }
    if(ref & kLeafBit) { b = a.leafBoxes[a.sortedIds[ref & ~kLeafBit]]; cnt = 1; }
    else { b = a.nodeBoxes[ref]; cnt = a.nodes[ref].leafCount; }
    if(cnt == 0u || cnt > a.leafCount) { atomicOr(&a.counters[3], 1u); cnt = 1; }
}

__device__ __forceinline__ float half_area(const BoxF& b)
{
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void emit_payload(const CollapseArgs& a, uint32_t leafPos, uint32_t dst, uint32_t mesh)
{
    uint32_t prim = a.sortedIds[leafPos];
    if(a.kind == 1) { a.leafIds[dst] = prim; return; }
    const float* pos = a.pos;
    const uint32_t* idx = a.idx;
    uint32_t keyBase = a.primKeyBase;
    uint32_t raw = a.rawVerts;
    if(a.segs)
    {
        const MeshSeg& m = a.segs[mesh];
        prim -= m.first;
        pos = m.pos; idx = m.idx; keyBase = m.primKeyBase; raw = m.rawVerts;
    }
    uint32_t i0 = idx[3 * prim], i1 = idx[3 * prim + 1], i2 = idx[3 * prim + 2];
    float v0x = pos[3 * i0], v0y = pos[3 * i0 + 1], v0z = pos[3 * i0 + 2];
    float v1x = pos[3 * i1], v1y = pos[3 * i1 + 1], v1z = pos[3 * i1 + 2];
    float v2x = pos[3 * i2], v2y = pos[3 * i2 + 1], v2z = pos[3 * i2 + 2];
    TriRecord r;
    r.v0 = make_float4(v0x, v0y, v0z, __uint_as_float(keyBase + prim));
    if(raw)
    {
        // the watertight test reads the shared vertices themselves
        r.e0 = make_float4(v1x, v1y, v1z, 0.0f);
        r.e1 = make_float4(v2x, v2y, v2z, 0.0f);
    }
    else
    {
        r.e0 = make_float4(__fsub_rn(v1x, v0x), __fsub_rn(v1y, v0y), __fsub_rn(v1z, v0z), 0.0f);
        r.e1 = make_float4(__fsub_rn(v2x, v0x), __fsub_rn(v2y, v0y), __fsub_rn(v2z, v0z), 0.0f);
    }
    a.tris[dst] = r;
}

// One thread per wide node of the current level.  Queue items: binary node
// (or leaf) reference, wide node index, mesh of a batched build.
__global__ void k_collapse(CollapseArgs a, const uint4* __restrict__ queue, uint32_t qn,
                           uint4* __restrict__ nextQueue)
{
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if(w >= qn) return;
    uint4 item = queue[w];
    uint32_t root = item.x;
    uint32_t wideIdx = item.y;
    const uint32_t mesh = item.z;
    const uint32_t maxLeaf = a.segs ? a.segs[mesh].maxLeaf : a.maxLeaf;
    const float inflate = a.segs ? a.segs[mesh].inflate : a.inflate;

    uint32_t cand[8];
    BoxF cbox[8];
    uint32_t ccnt[8];
    int nc = 0;
    BoxF nbox; uint32_t ncnt;
    ref_box(a, root, nbox, ncnt);
    const bool sah = a.costs && maxLeaf <= a.sahMaxLeaf;
    // a child that fits a leaf is one, unless the SAH chose to open it
    auto as_leaf = [&](uint32_t ref, uint32_t cnt) -> bool
    {
        if(ref & kLeafBit) return true;
        if(cnt > maxLeaf) return false;
        if(!sah || !ref_ok(a, ref)) return true;
        return a.costs[ref].asLeaf != 0u;
    };
    if(as_leaf(root, ncnt))
    {
        cand[0] = root; cbox[0] = nbox; ccnt[0] = ncnt; nc = 1;
    }
    else
    {
        const BinNode& bn = a.nodes[root];
        if(sah)
        {
            // expand by the recorded choices; the slots of the stack's
            // entries sum to at most 8, so it never holds more than 8
            uint32_t stR[8];
            int stI[8];
            int sp = 0;
            const int k0 = (int)a.costs[root].fullSplit;
            stR[sp] = bn.right; stI[sp++] = (k0 >= 1 && k0 <= 7) ? 8 - k0 : 4;
            stR[sp] = bn.left;  stI[sp++] = (k0 >= 1 && k0 <= 7) ? k0 : 4;
            while(sp > 0 && nc < 8)
            {
                const uint32_t r = stR[--sp];
                int i = stI[sp];
                if(!ref_ok(a, r)) break;
                if(!(r & kLeafBit))
                    while(i > 1 && a.costs[r].split[i - 1] == 0) i--;
                if((r & kLeafBit) || i == 1)
                {
                    cand[nc] = r; ref_box(a, r, cbox[nc], ccnt[nc]); nc++;
                    continue;
                }
                const int k = (int)a.costs[r].split[i - 1];
                if(k < 1 || k >= i || sp + 2 > 8) { atomicOr(&a.counters[3], 1u); break; }
                const BinNode& on = a.nodes[r];
                stR[sp] = on.right; stI[sp++] = i - k;
                stR[sp] = on.left;  stI[sp++] = k;
            }
            if(sp > 0) atomicOr(&a.counters[3], 1u);     // more than 8 children: a malformed table
        }
        else
        {
        cand[0] = bn.left;  ref_box(a, bn.left, cbox[0], ccnt[0]);
        cand[1] = bn.right; ref_box(a, bn.right, cbox[1], ccnt[1]);
        nc = 2;
        while(nc < 8)
        {
            int best = -1; float bestA = -1.0f;
            for(int c = 0; c < nc; c++)
            {
                if((cand[c] & kLeafBit) || ccnt[c] <= maxLeaf) continue;
                float ar = half_area(cbox[c]);
                if(ar > bestA) { bestA = ar; best = c; }
            }
            if(best < 0 || !ref_ok(a, cand[best])) break;
            const BinNode& on = a.nodes[cand[best]];
            cand[best] = on.left;  ref_box(a, on.left, cbox[best], ccnt[best]);
            cand[nc] = on.right;   ref_box(a, on.right, cbox[nc], ccnt[nc]);
            nc++;
        }
        }
    }

    // Quantisation frame.  Children are stored one quantum wider on each side
    // than their outward-rounded box (the traversal evaluates planes with a
    // 2^23-biased byte, whose offset term can be off by half a quantum), so
    // the frame reserves a quantum below and above: 2^e * 252 >= extent and
    // p = inflated min - 2^e.  Every stored child then lies in [0, 255].
    float px[3];
    uint32_t eb[3];
    float invS[3];
    for(int k = 0; k < 3; k++)
    {
        float lo = __fsub_rd(nbox.mn[k], inflate);
        float hi = __fadd_ru(nbox.mx[k], inflate);
        float ext = __fsub_ru(hi, lo);
#if MRG_NODE_F16
        // fp16 frame: p = inflated min, 2^e the smallest power of two with
        // ext * 2^-e <= 2^15 (every offset fits fp16 exactly scaled)
        uint32_t bits = __float_as_uint(ext);
        int ex = (int)((bits >> 23) & 0xFF);
        int e = (ex == 0) ? -126 : ex - 127 + (((bits & 0x7FFFFFu) != 0u) ? 1 : 0) - 15;
        e = max(-126, min(e, 126));
        eb[k] = (uint32_t)(e + 127);
        px[k] = lo;
        invS[k] = __uint_as_float((uint32_t)(127 - e) << 23);
#else
        float x = __fdiv_ru(ext, MRG_NODE_EXACT_Q ? 255.0f : 252.0f);
        uint32_t bits = __float_as_uint(x);
        int ex = (int)((bits >> 23) & 0xFF);
        int e;
        if(ex == 0) e = -126;
        else e = ex - 127 + (((bits & 0x7FFFFFu) != 0u) ? 1 : 0);
        e = max(-126, min(e, 126));
        eb[k] = (uint32_t)(e + 127);
        px[k] = MRG_NODE_EXACT_Q ? lo : __fsub_rd(lo, __uint_as_float((uint32_t)(e + 127) << 23));
        invS[k] = __uint_as_float((uint32_t)(127 - e) << 23);
#endif
    }

    // Slot assignment by direction: slot s holds the child whose centre lies
    // farthest towards corner s (bit i of s set = +axis i).
    float ncx = 0.5f * (nbox.mn[0] + nbox.mx[0]);
    float ncy = 0.5f * (nbox.mn[1] + nbox.mx[1]);
    float ncz = 0.5f * (nbox.mn[2] + nbox.mx[2]);
    int slotOf[8];
    int childInSlot[8];
    for(int s = 0; s < 8; s++) childInSlot[s] = -1;
    for(int c = 0; c < 8; c++) slotOf[c] = -1;
    for(int it = 0; it < nc; it++)
    {
        float bestV = -FLT_MAX; int bc = -1, bs = -1;
        for(int c = 0; c < nc; c++)
        {
            if(slotOf[c] >= 0) continue;
            float vx = 0.5f * (cbox[c].mn[0] + cbox[c].mx[0]) - ncx;
            float vy = 0.5f * (cbox[c].mn[1] + cbox[c].mx[1]) - ncy;
            float vz = 0.5f * (cbox[c].mn[2] + cbox[c].mx[2]) - ncz;
            for(int s = 0; s < 8; s++)
            {
                if(childInSlot[s] >= 0) continue;
                float v = ((s & 1) ? vx : -vx) + ((s & 2) ? vy : -vy) + ((s & 4) ? vz : -vz);
                if(v > bestV) { bestV = v; bc = c; bs = s; }
            }
        }
        slotOf[bc] = bs;
        childInSlot[bs] = bc;
    }

    // Allocate children and payloads.
    uint32_t numInternal = 0, numPayload = 0;
    for(int c = 0; c < nc; c++)
    {
        bool leaf = as_leaf(cand[c], ccnt[c]);
        if(leaf) numPayload += ccnt[c]; else numInternal++;
    }
    uint32_t childBase = numInternal ? atomicAdd(&a.counters[0], numInternal) : 0u;
    uint32_t triBase = numPayload ? atomicAdd(&a.counters[1], numPayload) : 0u;
    uint32_t qBase = numInternal ? atomicAdd(&a.counters[2], numInternal) : 0u;
    if(childBase + numInternal > a.wideCap || qBase + numInternal > a.wideCap ||
       triBase + numPayload > a.leafCount || wideIdx >= a.wideCap)
    {
        atomicOr(&a.counters[3], 2u);
        return;
    }

    uint8_t meta[8];
#if MRG_NODE_F16
    __half hlo[3][8], hhi[3][8];
#else
    uint8_t qlo[3][8], qhi[3][8];
#endif
    uint32_t imask = 0;
    uint32_t rank = 0, triOff = 0;
    for(int s = 0; s < 8; s++)
    {
        int c = childInSlot[s];
        if(c < 0)
        {
            meta[s] = 0;
#if MRG_NODE_F16
            for(int k = 0; k < 3; k++) { hlo[k][s] = __float2half(0.0f); hhi[k][s] = __float2half(0.0f); }
#else
            for(int k = 0; k < 3; k++) { qlo[k][s] = 0; qhi[k][s] = 0; }
#endif
            continue;
        }
        for(int k = 0; k < 3; k++)
        {
            float lo = __fsub_rd(cbox[c].mn[k], inflate);
            float hi = __fadd_ru(cbox[c].mx[k], inflate);
#if MRG_NODE_F16
            // offsets rounded outward at every step (the scale is a power of two)
            const float vl = fmaxf(__fmul_rd(__fsub_rd(lo, px[k]), invS[k]), 0.0f);
            const float vh = __fmul_ru(__fsub_ru(hi, px[k]), invS[k]);
            hlo[k][s] = __float2half_rd(vl);
            hhi[k][s] = __float2half_ru(vh);
#else
            const float pad = MRG_NODE_EXACT_Q ? 0.0f : 1.0f;
            float ql = floorf(__fmul_rd(__fsub_rd(lo, px[k]), invS[k])) - pad;
            float qh = ceilf(__fmul_ru(__fsub_ru(hi, px[k]), invS[k])) + pad;
            qlo[k][s] = (uint8_t)fminf(fmaxf(ql, 0.0f), 255.0f);
            qhi[k][s] = (uint8_t)fminf(fmaxf(qh, 0.0f), 255.0f);
#endif
        }
        bool leaf = as_leaf(cand[c], ccnt[c]);
        if(!leaf)
        {
            imask |= 1u << s;
            meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
            nextQueue[qBase + rank] = make_uint4(cand[c], childBase + rank, mesh, 0u);
            rank++;
        }
        else
        {
            uint32_t k = ccnt[c];
            meta[s] = (uint8_t)((((1u << k) - 1u) << 5) | triOff);
            // gather the subtree's leaves (at most maxLeaf <= 3)
            uint32_t stack[8]; int sp = 0; stack[sp++] = cand[c];
            uint32_t m = 0;
            while(sp > 0)
            {
                uint32_t r = stack[--sp];
                if(!ref_ok(a, r)) continue;
                if(r & kLeafBit)
                {
                    if(m < k) emit_payload(a, r & ~kLeafBit, triBase + triOff + m, mesh);
                    else atomicOr(&a.counters[3], 4u);
                    m++;
                }
                else if(sp + 2 <= 8) { stack[sp++] = a.nodes[r].right; stack[sp++] = a.nodes[r].left; }
                else atomicOr(&a.counters[3], 4u);
            }
            triOff += k;
        }
    }

    WideNode out;
    out.w0 = make_float4(px[0], px[1], px[2],
                         __uint_as_float(eb[0] | (eb[1] << 8) | (eb[2] << 16) | (imask << 24)));
    uint32_t m0 = meta[0] | (meta[1] << 8) | (meta[2] << 16) | ((uint32_t)meta[3] << 24);
    uint32_t m1 = meta[4] | (meta[5] << 8) | (meta[6] << 16) | ((uint32_t)meta[7] << 24);
    out.w1 = make_uint4(childBase, triBase, m0, m1);
#if MRG_NODE_F16
    auto pack2 = [](__half a, __half b) -> uint32_t {
        return (uint32_t)__half_as_ushort(a) | ((uint32_t)__half_as_ushort(b) << 16);
    };
    for(int k = 0; k < 3; k++)
    {
        out.h[k] = make_uint4(pack2(hlo[k][0], hlo[k][1]), pack2(hlo[k][2], hlo[k][3]),
                              pack2(hlo[k][4], hlo[k][5]), pack2(hlo[k][6], hlo[k][7]));
        out.h[3 + k] = make_uint4(pack2(hhi[k][0], hhi[k][1]), pack2(hhi[k][2], hhi[k][3]),
                                  pack2(hhi[k][4], hhi[k][5]), pack2(hhi[k][6], hhi[k][7]));
    }
#else
    uint32_t qw[12];
    for(int k = 0; k < 3; k++)
    {
        qw[2 * k + 0] = qlo[k][0] | (qlo[k][1] << 8) | (qlo[k][2] << 16) | ((uint32_t)qlo[k][3] << 24);
        qw[2 * k + 1] = qlo[k][4] | (qlo[k][5] << 8) | (qlo[k][6] << 16) | ((uint32_t)qlo[k][7] << 24);
        qw[6 + 2 * k + 0] = qhi[k][0] | (qhi[k][1] << 8) | (qhi[k][2] << 16) | ((uint32_t)qhi[k][3] << 24);
        qw[6 + 2 * k + 1] = qhi[k][4] | (qhi[k][5] << 8) | (qhi[k][6] << 16) | ((uint32_t)qhi[k][7] << 24);
    }
    out.q[0] = make_uint4(qw[0], qw[1], qw[2], qw[3]);
    out.q[1] = make_uint4(qw[4], qw[5], qw[6], qw[7]);
    out.q[2] = make_uint4(qw[8], qw[9], qw[10], qw[11]);
#endif
    a.wnodes[wideIdx] = out;
}

// Adds fixed offsets to child / payload bases when a build is placed into the
// shared node and triangle arrays.
__global__ void k_relocate(const WideNode* __restrict__ in, WideNode* __restrict__ out, uint32_t n,
                           uint32_t nodeOff, uint32_t triOff)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    WideNode w = in[i];
    uint32_t imask = __float_as_uint(w.w0.w) >> 24;
    if(imask) w.w1.x += nodeOff;
    w.w1.y += triOff;
    out[i] = w;
}

inline unsigned gridFor(uint32_t n, int tpb = kTPB) { return (unsigned)((n + tpb - 1) / tpb); }

#define MRG_CK(x) do { cudaError_t e_ = (x); if(e_ != cudaSuccess) { err = std::string(#x) + ": " + cudaGetErrorString(e_); goto fail; } } while(0)

} // namespace

namespace {
// Collapse of the binary tree to 8-wide nodes, MRG_BVH_COLLAPSE: "sah" the
// SAH-optimal one (k_wide_cost) everywhere, "sah-blas" for BLASes only,
// "sah-large" only for BLASes with one triangle per leaf child, "greedy" the
// largest-child-first expansion everywhere; the default is "sah-blas".
// MRG_BVH_SAH_CPRIM / MRG_BVH_SAH_CINST are the costs of a triangle test and
// of an instance entry relative to a wide node test in the SAH.
enum { kCollapseGreedy = 0, kCollapseSah = 1, kCollapseSahBlas = 2, kCollapseSahLarge = 3 };
int collapse_mode()
{
    const char* v = std::getenv("MRG_BVH_COLLAPSE");
    if(!v) return kCollapseSahBlas;
    if(std::strcmp(v, "greedy") == 0) return kCollapseGreedy;
    if(std::strcmp(v, "sah-blas") == 0) return kCollapseSahBlas;
    if(std::strcmp(v, "sah-large") == 0) return kCollapseSahLarge;
    return kCollapseSah;
}
// the SAH collapse applies to wide nodes whose leaf size is at most this
uint32_t sah_max_leaf(bool tlas)
{
    switch(collapse_mode())
    {
        case kCollapseSah: return 3u;
        case kCollapseSahBlas: return tlas ? 0u : 3u;
        case kCollapseSahLarge: return tlas ? 0u : 1u;
        default: return 0u;
    }
}
float env_cost(const char* name, float dflt)
{
    const char* v = std::getenv(name);
    const float c = v ? (float)std::atof(v) : dflt;
    return (c > 0.0f && c < 1000.0f) ? c : dflt;
}
float sah_cprim() { return env_cost("MRG_BVH_SAH_CPRIM", 1.0f); }
// an instance entry (transform and a BLAS root) against a node test, for the TLAS
float sah_cinst() { return env_cost("MRG_BVH_SAH_CINST", 8.0f); }
} // namespace

bool build_wide_bvh(const BuildInput& in, BuildResult& out, cudaStream_t st, std::string& err)
{
    const uint32_t n = in.count;
    out = BuildResult{};
    if(n == 0) { err = "empty build"; return false; }

    BoxF* dLeafBoxes = nullptr; float* dCent = nullptr; uint32_t* dCB = nullptr;
    uint64_t* dCodes[2] = { nullptr, nullptr }; uint32_t* dIds[2] = { nullptr, nullptr };
    void* dTemp = nullptr; size_t tempBytes = 0;
    BinNode* dNodes = nullptr; BoxF* dNodeBoxes = nullptr; uint32_t* dLeafParent = nullptr; WideCost* dCosts = nullptr;
    uint32_t* dCnt = nullptr; uint4* dQ[2] = { nullptr, nullptr };
    uint32_t* dCounters = nullptr;
    WideNode* dW = nullptr;
    const uint32_t nInt = (n > 1) ? (n - 1) : 1;
    const uint32_t wideCap = n;      // each wide node consumes >= 1 binary node
    uint32_t cbInit[6] = { 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u };
    uint32_t hostCounters[4];
    BoxF rootBox;
    cub::DoubleBuffer<uint64_t> kb;
    cub::DoubleBuffer<uint32_t> vb;
    uint32_t qn = 1;
    int cur = 0;
    uint4 rootItem;
    CollapseArgs ca;
    float ext;

    MRG_CK(cudaMallocAsync(&dLeafBoxes, sizeof(BoxF) * n, st));
    MRG_CK(cudaMallocAsync(&dCent, sizeof(float) * 3 * n, st));
    MRG_CK(cudaMallocAsync(&dCB, sizeof(uint32_t) * 6, st));
    MRG_CK(cudaMallocAsync(&dCodes[0], sizeof(uint64_t) * n, st));
    MRG_CK(cudaMallocAsync(&dCodes[1], sizeof(uint64_t) * n, st));
    MRG_CK(cudaMallocAsync(&dIds[0], sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dIds[1], sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dNodes, sizeof(BinNode) * nInt, st));
    MRG_CK(cudaMallocAsync(&dNodeBoxes, sizeof(BoxF) * nInt, st));
    MRG_CK(cudaMallocAsync(&dLeafParent, sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dCnt, sizeof(uint32_t) * nInt, st));
    MRG_CK(cudaMallocAsync(&dQ[0], sizeof(uint4) * wideCap, st));
    MRG_CK(cudaMallocAsync(&dQ[1], sizeof(uint4) * wideCap, st));
    MRG_CK(cudaMallocAsync(&dCounters, sizeof(uint32_t) * 4, st));
    MRG_CK(cudaMallocAsync(&dW, sizeof(WideNode) * wideCap, st));
    if(in.kind == 0) MRG_CK(cudaMallocAsync(&out.tris, sizeof(TriRecord) * n, st));
    else             MRG_CK(cudaMallocAsync(&out.leafIds, sizeof(uint32_t) * n, st));

    MRG_CK(cudaMemcpyAsync(dCB, cbInit, sizeof(cbInit), cudaMemcpyHostToDevice, st));
    if(in.kind == 0)
        k_leaf_boxes_tri<<<gridFor(n), kTPB, 0, st>>>(in.pos, in.idx, n, dLeafBoxes, dCent, dCB);
    else
        k_leaf_boxes_given<<<gridFor(n), kTPB, 0, st>>>(reinterpret_cast<const BoxF*>(in.boxes), n,
                                                        dLeafBoxes, dCent, dCB);
    MRG_CK(cudaGetLastError());
    k_morton<<<gridFor(n), kTPB, 0, st>>>(dCent, dCB, n, dCodes[0], dIds[0]);
    MRG_CK(cudaGetLastError());

    kb = cub::DoubleBuffer<uint64_t>(dCodes[0], dCodes[1]);
    vb = cub::DoubleBuffer<uint32_t>(dIds[0], dIds[1]);
    MRG_CK(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, kb, vb, (int)n, 0, 63, st));
    MRG_CK(cudaMallocAsync(&dTemp, tempBytes, st));
    MRG_CK(cub::DeviceRadixSort::SortPairs(dTemp, tempBytes, kb, vb, (int)n, 0, 63, st));

    if(n > 1 && in.ploc)
    {
        // PLOC clustering in Morton order
        uint32_t *dC[2] = { nullptr, nullptr }, *dCC[2] = { nullptr, nullptr }, *dNN = nullptr, *dKeep = nullptr;
        uint32_t* dPos = nullptr;
        BoxF* dCB[2] = { nullptr, nullptr };
        void* dScanTemp = nullptr;
        size_t scanBytes = 0;
        bool okP = true;
        for(int k = 0; k < 2 && okP; k++)
        {
            okP = cudaMallocAsync(&dC[k], sizeof(uint32_t) * n, st) == cudaSuccess &&
                  cudaMallocAsync(&dCC[k], sizeof(uint32_t) * n, st) == cudaSuccess &&
                  cudaMallocAsync(&dCB[k], sizeof(BoxF) * n, st) == cudaSuccess;
        }
        okP = okP && cudaMallocAsync(&dNN, sizeof(uint32_t) * n, st) == cudaSuccess &&
              cudaMallocAsync(&dKeep, sizeof(uint32_t) * n, st) == cudaSuccess &&
              cudaMallocAsync(&dPos, sizeof(uint32_t) * n, st) == cudaSuccess &&
              cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, dKeep, dPos, (int)n, st) == cudaSuccess &&
              cudaMallocAsync(&dScanTemp, scanBytes, st) == cudaSuccess;
        okP = okP && cudaMemsetAsync(dCounters, 0, sizeof(uint32_t) * 4, st) == cudaSuccess;
        if(okP) k_ploc_init<<<gridFor(n), kTPB, 0, st>>>(vb.Current(), dLeafBoxes, n, dC[0], dCB[0], dCC[0]);
        uint32_t cn = n;
        int pc = 0;
        for(int iter = 0; okP && cn > 1; iter++)
        {
            if(iter > 4096) { okP = false; break; }
            k_ploc_nearest<<<gridFor(cn), kTPB, 0, st>>>(dCB[pc], cn, dNN);
            k_ploc_merge<<<gridFor(cn), kTPB, 0, st>>>(dC[pc], dCB[pc], dCC[pc], dNN, cn, dNodes, dNodeBoxes,
                                                       dCounters + 0, nInt, dC[pc ^ 1], dCB[pc ^ 1], dCC[pc ^ 1],
                                                       dKeep, dCounters + 3);
            okP = cub::DeviceScan::ExclusiveSum(dScanTemp, scanBytes, dKeep, dPos, (int)cn, st) == cudaSuccess;
            uint32_t lastKeep = 0, lastPos = 0;
            okP = okP && cudaMemcpyAsync(&lastKeep, dKeep + cn - 1, 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                  cudaMemcpyAsync(&lastPos, dPos + cn - 1, 4, cudaMemcpyDeviceToHost, st) == cudaSuccess;
            k_ploc_compact<<<gridFor(cn), kTPB, 0, st>>>(dKeep, dPos, cn, dC[pc ^ 1], dCB[pc ^ 1], dCC[pc ^ 1],
                                                         dC[pc], dCB[pc], dCC[pc]);
            okP = okP && cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(st) == cudaSuccess;
            const uint32_t next = lastPos + lastKeep;
            if(next >= cn) { okP = false; break; }     // no merge: cannot happen with a total order
            cn = next;
        }
        uint32_t rootRef = 0;
        if(okP) okP = cudaMemcpyAsync(&rootRef, dC[pc], 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                      cudaStreamSynchronize(st) == cudaSuccess;
        for(int k = 0; k < 2; k++) { cudaFreeAsync(dC[k], st); cudaFreeAsync(dCC[k], st); cudaFreeAsync(dCB[k], st); }
        cudaFreeAsync(dNN, st); cudaFreeAsync(dKeep, st); cudaFreeAsync(dPos, st); cudaFreeAsync(dScanTemp, st);
        if(!okP) { err = "PLOC clustering failed"; goto fail; }
        MRG_CK(cudaMemcpyAsync(&rootBox, dNodeBoxes + rootRef, sizeof(BoxF), cudaMemcpyDeviceToHost, st));
        rootItem = make_uint4(rootRef, 0u, 0u, 0u);
    }
    else if(n > 1)
    {
        MRG_CK(cudaMemsetAsync(dNodes, 0xFF, sizeof(BinNode) * nInt, st));
        MRG_CK(cudaMemsetAsync(dLeafParent, 0xFF, sizeof(uint32_t) * n, st));
        k_karras<<<gridFor(n - 1), kTPB, 0, st>>>(kb.Current(), (int)n, dNodes, dLeafParent, nullptr, 0u, nullptr);
        MRG_CK(cudaGetLastError());
        MRG_CK(cudaMemsetAsync(dCnt, 0, sizeof(uint32_t) * nInt, st));
        MRG_CK(cudaMemsetAsync(dCounters, 0, sizeof(uint32_t) * 4, st));
        k_bottom_up<<<gridFor(n), kTPB, 0, st>>>(dLeafParent, vb.Current(), dLeafBoxes, dNodes,
                                                 dNodeBoxes, dCnt, (int)n, dCounters + 3);
        MRG_CK(cudaGetLastError());
        if(in.maxLeaf <= sah_max_leaf(in.kind == 1))
        {
            MRG_CK(cudaMallocAsync(&dCosts, sizeof(WideCost) * nInt, st));
            MRG_CK(cudaMemsetAsync(dCnt, 0, sizeof(uint32_t) * nInt, st));
            k_wide_cost<<<gridFor(n), kTPB, 0, st>>>(dLeafParent, vb.Current(), dLeafBoxes, dNodes, dNodeBoxes,
                                                     dCosts, dCnt, (int)n, nullptr, nullptr, 0u, in.maxLeaf, 1.0f,
                                                     in.kind == 1 ? sah_cinst() : sah_cprim(), dCounters + 3);
            MRG_CK(cudaGetLastError());
        }
        MRG_CK(cudaMemcpyAsync(&rootBox, dNodeBoxes, sizeof(BoxF), cudaMemcpyDeviceToHost, st));
        rootItem = make_uint4(0u, 0u, 0u, 0u);
    }
    else
    {
        MRG_CK(cudaMemcpyAsync(&rootBox, dLeafBoxes, sizeof(BoxF), cudaMemcpyDeviceToHost, st));
        rootItem = make_uint4(kLeafBit | 0u, 0u, 0u, 0u);
    }
    MRG_CK(cudaMemcpyAsync(hostCounters, dCounters, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost, st));
    MRG_CK(cudaStreamSynchronize(st));
    if(n > 1 && hostCounters[3] != 0) { err = "binary tree construction produced an invalid node"; goto fail; }
    for(int k = 0; k < 3; k++) { out.box[k] = rootBox.mn[k]; out.box[3 + k] = rootBox.mx[k]; }

    ext = 0.0f;
    for(int k = 0; k < 3; k++)
    {
        float e = fabsf(rootBox.mx[k]) > fabsf(rootBox.mn[k]) ? fabsf(rootBox.mx[k]) : fabsf(rootBox.mn[k]);
        ext = (ext > e) ? ext : e;
        float sp = rootBox.mx[k] - rootBox.mn[k];
        ext = (ext > sp) ? ext : sp;
    }

    ca.segs = nullptr;
    ca.nodes = dNodes; ca.nodeBoxes = dNodeBoxes; ca.leafBoxes = dLeafBoxes;
    ca.sortedIds = vb.Current(); ca.pos = in.pos; ca.idx = in.idx;
    ca.primKeyBase = in.primKeyBase; ca.kind = in.kind; ca.maxLeaf = in.maxLeaf;
    ca.rawVerts = in.rawVerts ? 1u : 0u;
    ca.inflate = ext * 1.0e-5f + 1.0e-30f;
    ca.wnodes = dW; ca.tris = out.tris; ca.leafIds = out.leafIds; ca.counters = dCounters;
    ca.leafCount = n; ca.wideCap = wideCap;
    ca.costs = dCosts; ca.sahMaxLeaf = dCosts ? 3u : 0u;

    hostCounters[0] = 1; hostCounters[1] = 0; hostCounters[2] = 0; hostCounters[3] = 0;
    MRG_CK(cudaMemcpyAsync(dCounters, hostCounters, sizeof(hostCounters), cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemcpyAsync(dQ[0], &rootItem, sizeof(uint4), cudaMemcpyHostToDevice, st));
    for(int level = 0; qn > 0; level++)
    {
        if(level > 64) { err = "wide BVH deeper than 64 levels"; goto fail; }
        MRG_CK(cudaMemsetAsync(dCounters + 2, 0, sizeof(uint32_t), st));
        k_collapse<<<gridFor(qn, 128), 128, 0, st>>>(ca, dQ[cur], qn, dQ[cur ^ 1]);
        MRG_CK(cudaGetLastError());
        MRG_CK(cudaMemcpyAsync(hostCounters, dCounters, sizeof(hostCounters), cudaMemcpyDeviceToHost, st));
        MRG_CK(cudaStreamSynchronize(st));
        if(hostCounters[3] != 0) { err = "wide BVH collapse reported an invalid tree"; goto fail; }
        if(hostCounters[0] > wideCap) { err = "wide node capacity exceeded"; goto fail; }
        qn = hostCounters[2];
        cur ^= 1;
    }
    if(hostCounters[1] != n) { err = "payload count mismatch"; goto fail; }
    out.nodeCount = hostCounters[0];
    MRG_CK(cudaMallocAsync(&out.nodes, sizeof(WideNode) * out.nodeCount, st));
    MRG_CK(cudaMemcpyAsync(out.nodes, dW, sizeof(WideNode) * out.nodeCount, cudaMemcpyDeviceToDevice, st));
    out.payloadCount = n;

    cudaFreeAsync(dLeafBoxes, st); cudaFreeAsync(dCent, st); cudaFreeAsync(dCB, st);
    cudaFreeAsync(dCodes[0], st); cudaFreeAsync(dCodes[1], st);
    cudaFreeAsync(dIds[0], st); cudaFreeAsync(dIds[1], st); cudaFreeAsync(dTemp, st);
    cudaFreeAsync(dNodes, st); cudaFreeAsync(dNodeBoxes, st); cudaFreeAsync(dLeafParent, st);
    cudaFreeAsync(dCnt, st); cudaFreeAsync(dQ[0], st); cudaFreeAsync(dQ[1], st);
    cudaFreeAsync(dCounters, st); cudaFreeAsync(dW, st); cudaFreeAsync(dCosts, st);
    if(cudaStreamSynchronize(st) != cudaSuccess) { err = "stream sync failed"; return false; }
    return true;

fail:
    cudaStreamSynchronize(st);
    cudaFree(dLeafBoxes); cudaFree(dCent); cudaFree(dCB); cudaFree(dCodes[0]); cudaFree(dCodes[1]);
    cudaFree(dIds[0]); cudaFree(dIds[1]); cudaFree(dTemp); cudaFree(dNodes); cudaFree(dNodeBoxes);
    cudaFree(dLeafParent); cudaFree(dCnt); cudaFree(dQ[0]); cudaFree(dQ[1]); cudaFree(dCounters);
    cudaFree(dW); cudaFree(dCosts); cudaFree(out.nodes); cudaFree(out.tris); cudaFree(out.leafIds);
    out = BuildResult{};
    return false;
}

bool build_wide_bvh_batch(const std::vector<BatchMeshInput>& meshes, BatchResult& out, cudaStream_t st,
                          std::string& err)
{
    out = BatchResult{};
    const uint32_t M = (uint32_t)meshes.size();
    if(M == 0) { err = "empty batch"; return false; }
    std::vector<uint32_t> firsts(M + 1);
    std::vector<MeshSeg> segs(M);
    uint64_t total = 0;
    for(uint32_t m = 0; m < M; m++)
    {
        const BatchMeshInput& in = meshes[m];
        if(in.count == 0 || !in.pos || !in.idx) { err = "empty mesh in batch"; return false; }
        firsts[m] = (uint32_t)total;
        segs[m] = MeshSeg{ in.pos, in.idx, (uint32_t)total, in.count, in.primKeyBase,
                           std::min(3u, std::max(1u, in.maxLeaf)), 0.0f, in.rawVerts ? 1u : 0u };
        total += in.count;
        if(total >= (1ull << 31)) { err = "batch larger than 2^31 triangles"; return false; }
    }
    firsts[M] = (uint32_t)total;
    const uint32_t n = (uint32_t)total;
    const uint32_t nInt = (n > 1) ? (n - 1) : 1;
    const uint32_t wideCap = n;
    // key layout: mesh id bits above 3 x `bits` Morton bits
    uint32_t mbits = 0;
    while(mbits < 32 && (1ull << mbits) < M) mbits++;
    const uint32_t bits = std::min(21u, (64u - mbits) / 3u);
    const int endBit = (int)(mbits + 3u * bits);

    MeshSeg* dSegs = nullptr; uint32_t* dFirsts = nullptr; uint32_t* dCB = nullptr; uint32_t* dLeafMesh = nullptr;
    BoxF* dLeafBoxes = nullptr; float* dCent = nullptr;
    uint64_t* dCodes[2] = { nullptr, nullptr }; uint32_t* dIds[2] = { nullptr, nullptr };
    void* dTemp = nullptr; size_t tempBytes = 0;
    BinNode* dNodes = nullptr; BoxF* dNodeBoxes = nullptr; uint32_t* dLeafParent = nullptr; WideCost* dCosts = nullptr;
    uint32_t* dCnt = nullptr; uint4* dQ[2] = { nullptr, nullptr };
    uint32_t* dCounters = nullptr; uint32_t* dMeshRoot = nullptr; BoxF* dMeshBoxes = nullptr;
    WideNode* dW = nullptr;
    std::vector<uint32_t> cbInit(6ull * M), meshRoot(M);
    std::vector<BoxF> meshBoxes(M);
    std::vector<uint4> seeds(M);
    uint32_t hostCounters[4] = { 0, 0, 0, 0 };
    cub::DoubleBuffer<uint64_t> kb;
    cub::DoubleBuffer<uint32_t> vb;
    CollapseArgs ca;
    uint32_t qn = M;
    int cur = 0;

    for(uint32_t m = 0; m < M; m++)
    {
        for(int k = 0; k < 3; k++) { cbInit[6 * m + k] = 0xFFFFFFFFu; cbInit[6 * m + 3 + k] = 0u; }
        meshRoot[m] = (segs[m].count == 1u) ? (kLeafBit | segs[m].first) : kNoParent;
    }
    MRG_CK(cudaMallocAsync(&dSegs, sizeof(MeshSeg) * M, st));
    MRG_CK(cudaMallocAsync(&dFirsts, sizeof(uint32_t) * (M + 1), st));
    MRG_CK(cudaMallocAsync(&dCB, sizeof(uint32_t) * 6 * M, st));
    MRG_CK(cudaMallocAsync(&dLeafMesh, sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dLeafBoxes, sizeof(BoxF) * n, st));
    MRG_CK(cudaMallocAsync(&dCent, sizeof(float) * 3 * n, st));
    MRG_CK(cudaMallocAsync(&dCodes[0], sizeof(uint64_t) * n, st));
    MRG_CK(cudaMallocAsync(&dCodes[1], sizeof(uint64_t) * n, st));
    MRG_CK(cudaMallocAsync(&dIds[0], sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dIds[1], sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dNodes, sizeof(BinNode) * nInt, st));
    MRG_CK(cudaMallocAsync(&dNodeBoxes, sizeof(BoxF) * nInt, st));
    MRG_CK(cudaMallocAsync(&dLeafParent, sizeof(uint32_t) * n, st));
    MRG_CK(cudaMallocAsync(&dCnt, sizeof(uint32_t) * nInt, st));
    MRG_CK(cudaMallocAsync(&dQ[0], sizeof(uint4) * wideCap, st));
    MRG_CK(cudaMallocAsync(&dQ[1], sizeof(uint4) * wideCap, st));
    MRG_CK(cudaMallocAsync(&dCounters, sizeof(uint32_t) * 4, st));
    MRG_CK(cudaMallocAsync(&dMeshRoot, sizeof(uint32_t) * M, st));
    MRG_CK(cudaMallocAsync(&dMeshBoxes, sizeof(BoxF) * M, st));
    MRG_CK(cudaMallocAsync(&dW, sizeof(WideNode) * wideCap, st));
    MRG_CK(cudaMallocAsync(&out.tris, sizeof(TriRecord) * n, st));

    MRG_CK(cudaMemcpyAsync(dSegs, segs.data(), sizeof(MeshSeg) * M, cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemcpyAsync(dFirsts, firsts.data(), sizeof(uint32_t) * (M + 1), cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemcpyAsync(dCB, cbInit.data(), sizeof(uint32_t) * 6 * M, cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemcpyAsync(dMeshRoot, meshRoot.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemsetAsync(dCounters, 0, sizeof(uint32_t) * 4, st));
    k_leaf_boxes_multi<<<gridFor(n), kTPB, 0, st>>>(dSegs, dFirsts, M, n, dLeafBoxes, dCent, dCB, dLeafMesh);
    MRG_CK(cudaGetLastError());
    k_morton_multi<<<gridFor(n), kTPB, 0, st>>>(dCent, dCB, dLeafMesh, n, bits, dCodes[0], dIds[0]);
    MRG_CK(cudaGetLastError());
    kb = cub::DoubleBuffer<uint64_t>(dCodes[0], dCodes[1]);
    vb = cub::DoubleBuffer<uint32_t>(dIds[0], dIds[1]);
    MRG_CK(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, kb, vb, (int)n, 0, endBit, st));
    MRG_CK(cudaMallocAsync(&dTemp, tempBytes, st));
    MRG_CK(cub::DeviceRadixSort::SortPairs(dTemp, tempBytes, kb, vb, (int)n, 0, endBit, st));
    if(n > 1)
    {
        MRG_CK(cudaMemsetAsync(dNodes, 0xFF, sizeof(BinNode) * nInt, st));
        MRG_CK(cudaMemsetAsync(dLeafParent, 0xFF, sizeof(uint32_t) * n, st));
        k_karras<<<gridFor(n - 1), kTPB, 0, st>>>(kb.Current(), (int)n, dNodes, dLeafParent, dFirsts, M, dMeshRoot);
        MRG_CK(cudaGetLastError());
        MRG_CK(cudaMemsetAsync(dCnt, 0, sizeof(uint32_t) * nInt, st));
        k_bottom_up<<<gridFor(n), kTPB, 0, st>>>(dLeafParent, vb.Current(), dLeafBoxes, dNodes,
                                                 dNodeBoxes, dCnt, (int)n, dCounters + 3);
        MRG_CK(cudaGetLastError());
        if(sah_max_leaf(false) > 0u)
        {
            MRG_CK(cudaMallocAsync(&dCosts, sizeof(WideCost) * nInt, st));
            MRG_CK(cudaMemsetAsync(dCnt, 0, sizeof(uint32_t) * nInt, st));
            k_wide_cost<<<gridFor(n), kTPB, 0, st>>>(dLeafParent, vb.Current(), dLeafBoxes, dNodes, dNodeBoxes,
                                                     dCosts, dCnt, (int)n, dFirsts, dSegs, M, 3u, 1.0f,
                                                     sah_cprim(), dCounters + 3);
            MRG_CK(cudaGetLastError());
        }
    }
    k_mesh_boxes<<<gridFor(M), kTPB, 0, st>>>(dMeshRoot, M, dNodeBoxes, dLeafBoxes, vb.Current(), n, dMeshBoxes,
                                              dCounters + 3);
    MRG_CK(cudaGetLastError());
    MRG_CK(cudaMemcpyAsync(meshRoot.data(), dMeshRoot, sizeof(uint32_t) * M, cudaMemcpyDeviceToHost, st));
    MRG_CK(cudaMemcpyAsync(meshBoxes.data(), dMeshBoxes, sizeof(BoxF) * M, cudaMemcpyDeviceToHost, st));
    MRG_CK(cudaMemcpyAsync(hostCounters, dCounters, sizeof(hostCounters), cudaMemcpyDeviceToHost, st));
    MRG_CK(cudaStreamSynchronize(st));
    if(hostCounters[3] != 0) { err = "batched binary tree construction produced an invalid node"; goto fail; }

    // per-mesh box, inflation (1e-5 of the mesh's extent, as a single build) and collapse seed
    out.boxes.resize(6ull * M);
    for(uint32_t m = 0; m < M; m++)
    {
        const BoxF& b = meshBoxes[m];
        float ext = 0.0f;
        for(int k = 0; k < 3; k++)
        {
            out.boxes[6ull * m + k] = b.mn[k];
            out.boxes[6ull * m + 3 + k] = b.mx[k];
            const float e = fabsf(b.mx[k]) > fabsf(b.mn[k]) ? fabsf(b.mx[k]) : fabsf(b.mn[k]);
            ext = (ext > e) ? ext : e;
            const float sp = b.mx[k] - b.mn[k];
            ext = (ext > sp) ? ext : sp;
        }
        segs[m].inflate = ext * 1.0e-5f + 1.0e-30f;
        seeds[m] = make_uint4(meshRoot[m], m, m, 0u);
    }
    MRG_CK(cudaMemcpyAsync(dSegs, segs.data(), sizeof(MeshSeg) * M, cudaMemcpyHostToDevice, st));
    MRG_CK(cudaMemcpyAsync(dQ[0], seeds.data(), sizeof(uint4) * M, cudaMemcpyHostToDevice, st));

    ca.segs = dSegs;
    ca.nodes = dNodes; ca.nodeBoxes = dNodeBoxes; ca.leafBoxes = dLeafBoxes;
    ca.sortedIds = vb.Current(); ca.pos = nullptr; ca.idx = nullptr;
    ca.primKeyBase = 0; ca.kind = 0; ca.maxLeaf = 3; ca.inflate = 0.0f; ca.rawVerts = 0u;
    ca.wnodes = dW; ca.tris = out.tris; ca.leafIds = nullptr; ca.counters = dCounters;
    ca.leafCount = n; ca.wideCap = wideCap;
    ca.costs = dCosts; ca.sahMaxLeaf = sah_max_leaf(false);
    hostCounters[0] = M; hostCounters[1] = 0; hostCounters[2] = 0; hostCounters[3] = 0;
    MRG_CK(cudaMemcpyAsync(dCounters, hostCounters, sizeof(hostCounters), cudaMemcpyHostToDevice, st));
    for(int level = 0; qn > 0; level++)
    {
        if(level > 64) { err = "wide BVH deeper than 64 levels"; goto fail; }
        MRG_CK(cudaMemsetAsync(dCounters + 2, 0, sizeof(uint32_t), st));
        k_collapse<<<gridFor(qn, 128), 128, 0, st>>>(ca, dQ[cur], qn, dQ[cur ^ 1]);
        MRG_CK(cudaGetLastError());
        MRG_CK(cudaMemcpyAsync(hostCounters, dCounters, sizeof(hostCounters), cudaMemcpyDeviceToHost, st));
        MRG_CK(cudaStreamSynchronize(st));
        if(hostCounters[3] != 0) { err = "wide BVH collapse reported an invalid tree"; goto fail; }
        if(hostCounters[0] > wideCap) { err = "wide node capacity exceeded"; goto fail; }
        qn = hostCounters[2];
        cur ^= 1;
    }
    if(hostCounters[1] != n) { err = "payload count mismatch"; goto fail; }
    out.nodeCount = hostCounters[0];
    MRG_CK(cudaMallocAsync(&out.nodes, sizeof(WideNode) * out.nodeCount, st));
    MRG_CK(cudaMemcpyAsync(out.nodes, dW, sizeof(WideNode) * out.nodeCount, cudaMemcpyDeviceToDevice, st));
    out.payloadCount = n;

    cudaFreeAsync(dSegs, st); cudaFreeAsync(dFirsts, st); cudaFreeAsync(dCB, st); cudaFreeAsync(dLeafMesh, st);
    cudaFreeAsync(dLeafBoxes, st); cudaFreeAsync(dCent, st);
    cudaFreeAsync(dCodes[0], st); cudaFreeAsync(dCodes[1], st);
    cudaFreeAsync(dIds[0], st); cudaFreeAsync(dIds[1], st); cudaFreeAsync(dTemp, st);
    cudaFreeAsync(dNodes, st); cudaFreeAsync(dNodeBoxes, st); cudaFreeAsync(dLeafParent, st);
    cudaFreeAsync(dCnt, st); cudaFreeAsync(dQ[0], st); cudaFreeAsync(dQ[1], st);
    cudaFreeAsync(dCounters, st); cudaFreeAsync(dMeshRoot, st); cudaFreeAsync(dMeshBoxes, st); cudaFreeAsync(dW, st);
    cudaFreeAsync(dCosts, st);
    if(cudaStreamSynchronize(st) != cudaSuccess) { err = "stream sync failed"; return false; }
    return true;

fail:
    cudaStreamSynchronize(st);
    cudaFree(dSegs); cudaFree(dFirsts); cudaFree(dCB); cudaFree(dLeafMesh);
    cudaFree(dLeafBoxes); cudaFree(dCent); cudaFree(dCodes[0]); cudaFree(dCodes[1]);
    cudaFree(dIds[0]); cudaFree(dIds[1]); cudaFree(dTemp); cudaFree(dNodes); cudaFree(dNodeBoxes);
    cudaFree(dLeafParent); cudaFree(dCnt); cudaFree(dQ[0]); cudaFree(dQ[1]); cudaFree(dCounters);
    cudaFree(dMeshRoot); cudaFree(dMeshBoxes); cudaFree(dW); cudaFree(dCosts); cudaFree(out.nodes); cudaFree(out.tris);
    out = BatchResult{};
    return false;
}

bool relocate_nodes(const WideNode* src, WideNode* dst, uint32_t n, uint32_t nodeOff,
                    uint32_t triOff, cudaStream_t st)
{
    if(n == 0) return true;
    k_relocate<<<gridFor(n), kTPB, 0, st>>>(src, dst, n, nodeOff, triOff);
    return cudaGetLastError() == cudaSuccess;
}

} // namespace mrg
