// mrg_build.h -- host interface of the GPU wide-BVH builder and the kernels.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

namespace mrg {

// Child-plane encoding of the 8-wide node: 0 = 8-bit quantised offsets
// (80-byte nodes), 1 = fp16 offsets (128-byte nodes).
#ifndef MRG_NODE_F16
#define MRG_NODE_F16 0
#endif
// 8-bit planes decoded exactly (byte - 2^23 after the biased conversion, one
// add on the FMA pipe per plane), so child boxes need no padding quantum.
#ifndef MRG_NODE_EXACT_Q
#define MRG_NODE_EXACT_Q 0
#endif

struct WideNode;
struct TriRecord;
struct InstRecord;

struct BuildInput
{
    int             kind = 0;          // 0: triangles (pos/idx), 1: boxes (TLAS)
    const float*    pos = nullptr;     // device, 3 floats per vertex
    const uint32_t* idx = nullptr;     // device, 3 per triangle
    const float*    boxes = nullptr;   // device, 6 floats per leaf (min xyz, max xyz)
    uint32_t        count = 0;         // triangles or boxes
    uint32_t        primKeyBase = 0;
    uint32_t        maxLeaf = 3;       // primitives per leaf child (<= 3)
    bool            ploc = false;      // PLOC clustering instead of the Karras radix tree
    bool            rawVerts = false;  // triangle records hold v0, v1, v2 (watertight test)
};

struct BuildResult
{
    WideNode*   nodes = nullptr;       // device, nodeCount (child bases local to this build)
    uint32_t    nodeCount = 0;
    TriRecord*  tris = nullptr;        // kind 0: device, payloadCount records
    uint32_t*   leafIds = nullptr;     // kind 1: device, payloadCount leaf ids
    uint32_t    payloadCount = 0;
    float       box[6] = { 0, 0, 0, 0, 0, 0 };
};

bool build_wide_bvh(const BuildInput& in, BuildResult& out, cudaStream_t st, std::string& err);

// Batched BLAS build (the counterpart of MRay's segmented multi-build,
// Source/Tracer/AcceleratorLBVH.hpp:585-899): every mesh in one pass of
// leaf boxes, keys, sort, radix tree, bottom-up boxes and level-by-level
// collapse.  Wide node m is the root of mesh m.
struct BatchMeshInput
{
    const float*    pos = nullptr;     // device, 3 floats per vertex
    const uint32_t* idx = nullptr;     // device, 3 per triangle (local to the mesh)
    uint32_t        count = 0;         // triangles (>= 1)
    uint32_t        primKeyBase = 0;
    uint32_t        maxLeaf = 3;       // triangles per leaf child (<= 3)
    bool            rawVerts = false;  // triangle records hold v0, v1, v2 (watertight test)
};

struct BatchResult
{
    WideNode*          nodes = nullptr;     // device, nodeCount (child bases local to the batch)
    uint32_t           nodeCount = 0;
    TriRecord*         tris = nullptr;      // device, payloadCount records
    uint32_t           payloadCount = 0;
    std::vector<float> boxes;               // 6 per mesh: exact root box
};

bool build_wide_bvh_batch(const std::vector<BatchMeshInput>& meshes, BatchResult& out, cudaStream_t st,
                          std::string& err);
bool relocate_nodes(const WideNode* src, WideNode* dst, uint32_t n, uint32_t nodeOff,
                    uint32_t triOff, cudaStream_t st);

// Traversal launch parameters (device pointers).
struct TraceScene
{
    const WideNode*   nodes = nullptr;     // all BLAS nodes then TLAS nodes
    const TriRecord*  tris = nullptr;
    const InstRecord* insts = nullptr;
    const uint32_t*   tlasLeaf = nullptr;  // instance id per TLAS payload slot
    uint32_t          tlasRoot = 0;
    uint32_t          instCount = 0;
    uint32_t          nodeCount = 0;       // bounds for every index read from the tree
    uint32_t          triCount = 0;
    uint32_t          watertight = 0;      // 1: records hold v0, v1, v2; the watertight test runs
};

struct TraceScratch
{
    uint32_t*           workCounter = nullptr;   // 1 word, zeroed before each launch
    uint32_t*           errorFlag = nullptr;     // 1 word, sticky error bits
    unsigned long long* stats = nullptr;         // 8 words (stats kernel only)
};

enum TraceErrorBits : uint32_t
{
    kTraceStackOverflow = 1u,
    kTraceStepCap       = 2u,
    kTraceBadIndex      = 4u
};

// nDevice (optional): device word holding the ray count, read by the kernel
// (device-driven wavefronts); when given, n is ignored.
// Listed ray i against instance instIds[i] only (CastLocalRays).
cudaError_t launch_local(const TraceScene& sc, const TraceScratch& scr, void* rays, const uint32_t* rayIdx,
                         const uint32_t* instIds, uint32_t n, void* hits, void* meta, int smCount, cudaStream_t st);
cudaError_t launch_closest(const TraceScene& sc, const TraceScratch& scr, void* rays,
                           const uint32_t* rayIdx, uint32_t n, void* hits, void* meta,
                           int smCount, cudaStream_t st, const uint32_t* nDevice = nullptr);
cudaError_t launch_visibility(const TraceScene& sc, const TraceScratch& scr, uint32_t* visBits,
                              const void* rays, const uint32_t* rayIdx, uint32_t n,
                              int smCount, cudaStream_t st, const uint32_t* nDevice = nullptr);
// Loads the closest-hit traversal kernel on the current device (a function
// attribute query forces a lazily loaded module in).
cudaError_t preload_closest();
cudaError_t launch_closest_stats(const TraceScene& sc, const TraceScratch& scr, const void* rays,
                                 uint32_t n, int smCount, cudaStream_t st);

} // namespace mrg
