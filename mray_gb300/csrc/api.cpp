// api.cpp -- the C ABI (include/mray_gb300.h): context, scene upload, build,
// casts.  Host C++ over the CUDA runtime; no exceptions cross the boundary.
#include "mrg_ctx.h"
#include "host_math.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace {

// Binary-tree builder of the BVHs: the Karras radix tree by default (on the
// stress workload it gives 23.1 node visits per ray against PLOC's 30.2);
// the environment variable MRG_BVH_BUILDER=ploc selects PLOC clustering.
bool use_ploc()
{
    const char* v = std::getenv("MRG_BVH_BUILDER");
    return v && std::strcmp(v, "ploc") == 0;
}

// Triangles per BLAS leaf child (1..3).  One for large meshes (the stress
// workload's 1.31M-triangle BLAS: 1,317 against 1,243 Mrays/s for three, the
// tree growing from 73.8 to 93.1 MB), three for small ones, where one wide
// node then holds the whole mesh (the box scene renders 14% faster);
// MRG_BVH_LEAF overrides it.
uint32_t leaf_size(uint32_t triangles)
{
    const char* v = std::getenv("MRG_BVH_LEAF");
    const int k = v ? std::atoi(v) : (triangles > 1024u ? 1 : 3);
    return (k >= 1 && k <= 3) ? (uint32_t)k : 1u;
}

// Optional coherence sort of large closest-hit batches (by direction octant,
// then origin) before the cast, MRG_CAST_SORT=1.  Off by default: on the
// stress workload the sort plus the sorted cast took 4.63 ms against 3.13 ms
// for the cast in the caller's order.
constexpr uint32_t kCoherenceSortMin = 1u << 18;
bool cast_sort_enabled()
{
    const char* v = std::getenv("MRG_CAST_SORT");
    return v && std::strcmp(v, "1") == 0;
}


thread_local std::string g_lastError;

mrg_status fail(mrg_status s, const std::string& msg)
{
    g_lastError = msg;
    return s;
}

} // namespace

mrg_status mrg::set_error(mrg_status s, const std::string& msg)
{
    return fail(s, msg);
}

namespace {

mrg_status cuda_fail(cudaError_t e, const char* what)
{
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? MRG_ERR_OUT_OF_MEMORY : MRG_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define MRG_TRY(call, what) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) return cuda_fail(e_, what); } while(0)

void free_accel(mrg_ctx* c)
{
    cudaFree(c->dNodes); c->dNodes = nullptr;
    cudaFree(c->dTris); c->dTris = nullptr;
    cudaFree(c->dInsts); c->dInsts = nullptr;
    cudaFree(c->dTlasLeaf); c->dTlasLeaf = nullptr;
    c->blasNodes = c->blasTris = c->tlasNodes = 0;
    c->scene = mrg::TraceScene{};
    c->built = false;
}

struct DeviceGuard
{
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if(cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if(prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() { if(prev >= 0) cudaSetDevice(prev); }
};

mrg::TraceScratch scratch_of(mrg_ctx* c)
{
    mrg::TraceScratch s;
    s.workCounter = c->dScratch;
    s.errorFlag = c->dScratch + 1;
    s.stats = c->dStats;
    return s;
}

// Chunks of the host-buffer cast pipeline: about 512k rays each, at most
// kHostMaxChunks (MRG_HOST_CHUNKS overrides).
uint32_t host_chunks(uint32_t n)
{
    const char* v = std::getenv("MRG_HOST_CHUNKS");
    const int want = v ? std::atoi(v) : (int)(n >> 19);
    return (uint32_t)std::min(std::max(want, 1), mrg_ctx::kHostMaxChunks);
}

} // namespace

extern "C" {

const char* mrg_last_error(void) { return g_lastError.c_str(); }

const char* mrg_status_string(mrg_status s)
{
    switch(s)
    {
        case MRG_OK: return "ok";
        case MRG_ERR_INVALID_ARG: return "invalid argument";
        case MRG_ERR_CUDA: return "CUDA error";
        case MRG_ERR_OUT_OF_MEMORY: return "out of memory";
        case MRG_ERR_NOT_BUILT: return "accelerator not built";
        case MRG_ERR_LIMIT: return "capacity limit exceeded";
        case MRG_ERR_TRAVERSAL: return "traversal error";
    }
    return "unknown status";
}

mrg_status mrg_create(const mrg_params* params, mrg_ctx** out)
{
    if(!out) return fail(MRG_ERR_INVALID_ARG, "mrg_create: out_ctx is null");
    *out = nullptr;
    int dev = params ? params->device : 0;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if(e != cudaSuccess) return cuda_fail(e, "mrg_create: cudaGetDeviceCount");
    if(dev < 0 || dev >= count) return fail(MRG_ERR_INVALID_ARG, "mrg_create: bad device ordinal");
    mrg_ctx* c = new(std::nothrow) mrg_ctx();
    if(!c) return fail(MRG_ERR_OUT_OF_MEMORY, "mrg_create: host allocation");
    c->device = dev;
    const uint32_t test = params ? params->triangle_test : MRG_TRI_MOLLER_TRUMBORE;
    if(test != MRG_TRI_MOLLER_TRUMBORE && test != MRG_TRI_WATERTIGHT)
    {
        delete c;
        return fail(MRG_ERR_INVALID_ARG, "mrg_create: unknown triangle_test");
    }
    c->watertight = (test == MRG_TRI_WATERTIGHT);
    DeviceGuard g(dev);
    if((e = cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
       (e = cudaStreamCreateWithFlags(&c->buildStream, cudaStreamNonBlocking)) != cudaSuccess ||
       (e = cudaMalloc(&c->dScratch, 8 * sizeof(uint32_t))) != cudaSuccess ||
       (e = cudaMalloc(&c->dStats, 8 * sizeof(unsigned long long))) != cudaSuccess ||
       (e = cudaMemset(c->dScratch, 0, 8 * sizeof(uint32_t))) != cudaSuccess)
    {
        mrg_status s = cuda_fail(e, "mrg_create");
        mrg_destroy(c);
        return s;
    }
    // the allocation-free cast's static array and kernel are loaded here,
    // where allocating is allowed, not in its first call
    if(mrg_status s = mrg::noalloc_prepare(dev); s != MRG_OK)
    {
        mrg_destroy(c);
        return s;
    }
    *out = c;
    return MRG_OK;
}

mrg_status mrg_destroy(mrg_ctx* c)
{
    if(!c) return MRG_OK;
    DeviceGuard g(c->device);
    free_accel(c);
    cudaFree(c->dScratch);
    cudaFree(c->dStats);
    cudaFree(c->dPtSurfaces); cudaFree(c->dPtLights); cudaFree(c->dPtTris); cudaFree(c->ptPathMem);
    cudaFree(c->dPtEnv);
    cudaFree(c->dPtTexTable); cudaFree(c->dPtTexData); cudaFree(c->dPtUvs); cudaFree(c->dPtRadTotal);
    cudaFree(c->dPtMipData);
    cudaFree(c->dPtSpec);
    cudaFree(c->dPartScratch);
    cudaFree(c->dPtCacheBuf);
    cudaFree(c->dGuideGrid);
    cudaFree(c->dGuidePaths);
    for(void* q : c->cacheAllocs) cudaFree(q);
    cudaFree(c->dStageRays); cudaFree(c->dStageHits); cudaFree(c->dStageMeta);
    for(cudaStream_t& q : c->hostStreams) if(q) cudaStreamDestroy(q);
    for(cudaStream_t q : { c->ptSideStream, c->ptStream2, c->ptSideStream2 }) if(q) cudaStreamDestroy(q);
    for(cudaEvent_t q : { c->ptEvShaded, c->ptEvResolved, c->ptEvShaded2, c->ptEvResolved2, c->ptEvFilm,
                          c->ptEvStart, c->ptEvDone2 })
        if(q) cudaEventDestroy(q);
    cudaFree(c->ptPathMem2);
    cudaFree(c->dPtRadTotal2);
    cudaFree(c->dPtGradEmission);
    cudaFree(c->dZsTables);
    cudaFree(c->dZsSeeds);
    cudaFree(c->dHostCounters);
    for(cudaEvent_t& q : c->hostEvents) if(q) cudaEventDestroy(q);
    if(c->buildStream) cudaStreamDestroy(c->buildStream);
    delete c;
    return MRG_OK;
}

mrg_status mrg_upload_mesh(mrg_ctx* c, const float* pos, uint32_t nv, const uint32_t* idx,
                           uint32_t nt, uint32_t primKeyBase, uint32_t* outId)
{
    if(!c || !pos || !idx || nv == 0 || nt == 0)
        return fail(MRG_ERR_INVALID_ARG, "mrg_upload_mesh: null pointer or empty mesh");
    if(nt > (1u << 28) || (uint64_t)primKeyBase + nt > 0xFFFFFFFFull)
        return fail(MRG_ERR_LIMIT, "mrg_upload_mesh: more than 2^28 triangles or key overflow");
    for(uint64_t i = 0; i < 3ull * nt; i++)
        if(idx[i] >= nv) return fail(MRG_ERR_INVALID_ARG, "mrg_upload_mesh: index out of range");
    mrg_ctx::Mesh m;
    try
    {
        m.pos.assign(pos, pos + 3ull * nv);
        m.idx.assign(idx, idx + 3ull * nt);
    }
    catch(...) { return fail(MRG_ERR_OUT_OF_MEMORY, "mrg_upload_mesh: host allocation"); }
    m.primKeyBase = primKeyBase;
    c->meshes.push_back(std::move(m));
    c->built = false;
    if(outId) *outId = (uint32_t)(c->meshes.size() - 1);
    return MRG_OK;
}

mrg_status mrg_upload_mesh_uv(mrg_ctx* c, uint32_t mesh, const float* uv, uint32_t nv)
{
    if(!c || !uv) return fail(MRG_ERR_INVALID_ARG, "mrg_upload_mesh_uv: null pointer");
    if(mesh >= c->meshes.size()) return fail(MRG_ERR_INVALID_ARG, "mrg_upload_mesh_uv: bad mesh id");
    if(3ull * nv != c->meshes[mesh].pos.size())
        return fail(MRG_ERR_INVALID_ARG, "mrg_upload_mesh_uv: uv count differs from the vertex count");
    try { c->meshes[mesh].uv.assign(uv, uv + 2ull * nv); }
    catch(...) { return fail(MRG_ERR_OUT_OF_MEMORY, "mrg_upload_mesh_uv: host allocation"); }
    c->ptDirty = true;
    return MRG_OK;
}

mrg_status mrg_add_instance(mrg_ctx* c, uint32_t mesh, const float m[12], uint32_t flags,
                            uint32_t lm, uint32_t trans, uint32_t accel, uint32_t* outId)
{
    if(!c || !m) return fail(MRG_ERR_INVALID_ARG, "mrg_add_instance: null pointer");
    if(mesh >= c->meshes.size()) return fail(MRG_ERR_INVALID_ARG, "mrg_add_instance: bad mesh id");
    if(c->insts.size() >= (1u << 24)) return fail(MRG_ERR_LIMIT, "mrg_add_instance: more than 2^24 instances");
    mrg_ctx::Inst in;
    in.mesh = mesh;
    std::memcpy(in.m, m, sizeof(in.m));
    mrg::mat34_inverse(in.m, in.inv, (flags & MRG_INSTANCE_CORRECTED_INVERSE) != 0);
    in.flags = flags; in.lm = lm; in.trans = trans; in.accel = accel;
    c->insts.push_back(in);
    c->built = false;
    if(outId) *outId = (uint32_t)(c->insts.size() - 1);
    return MRG_OK;
}

mrg_status mrg_build(mrg_ctx* c)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_build: null context");
    if(c->insts.empty()) return fail(MRG_ERR_INVALID_ARG, "mrg_build: no instances");
    DeviceGuard g(c->device);
    auto t0 = std::chrono::steady_clock::now();
    free_accel(c);
    c->ptDirty = true;
    cudaStream_t st = c->buildStream;
    std::string err;

    // 1. BLASes: every mesh in one batched build (PLOC: one build per mesh).
    //    A piece is a node / triangle block placed into the shared arrays;
    //    meshRoot[m] is mesh m's root within its piece.
    struct Piece { mrg::WideNode* nodes; uint32_t nodeCount; mrg::TriRecord* tris; uint32_t payloadCount; };
    std::vector<Piece> pieces;
    std::vector<uint32_t> pieceOf(c->meshes.size()), meshRoot(c->meshes.size());
    auto free_pieces = [&]() { for(auto& p : pieces) { cudaFree(p.nodes); cudaFree(p.tris); } };
    {
        const size_t M = c->meshes.size();
        std::vector<float*> dPos(M, nullptr);
        std::vector<uint32_t*> dIdx(M, nullptr);
        auto free_uploads = [&]() { for(size_t i = 0; i < M; i++) { cudaFreeAsync(dPos[i], st); cudaFreeAsync(dIdx[i], st); } };
        cudaError_t e = cudaSuccess;
        for(size_t mi = 0; mi < M && e == cudaSuccess; mi++)
        {
            auto& m = c->meshes[mi];
            e = cudaMallocAsync(&dPos[mi], sizeof(float) * m.pos.size(), st);
            if(e == cudaSuccess) e = cudaMallocAsync(&dIdx[mi], sizeof(uint32_t) * m.idx.size(), st);
            if(e == cudaSuccess) e = cudaMemcpyAsync(dPos[mi], m.pos.data(), sizeof(float) * m.pos.size(), cudaMemcpyHostToDevice, st);
            if(e == cudaSuccess) e = cudaMemcpyAsync(dIdx[mi], m.idx.data(), sizeof(uint32_t) * m.idx.size(), cudaMemcpyHostToDevice, st);
        }
        if(e != cudaSuccess) { free_uploads(); cudaStreamSynchronize(st); return cuda_fail(e, "mrg_build: mesh upload"); }
        if(!use_ploc())
        {
            std::vector<mrg::BatchMeshInput> in(M);
            for(size_t mi = 0; mi < M; mi++)
            {
                const auto& m = c->meshes[mi];
                in[mi].pos = dPos[mi]; in[mi].idx = dIdx[mi];
                in[mi].count = (uint32_t)(m.idx.size() / 3);
                in[mi].primKeyBase = m.primKeyBase;
                in[mi].maxLeaf = leaf_size(in[mi].count);
                in[mi].rawVerts = c->watertight;
            }
            mrg::BatchResult br;
            const bool ok = mrg::build_wide_bvh_batch(in, br, st, err);
            free_uploads();
            if(!ok) { cudaStreamSynchronize(st); return fail(MRG_ERR_CUDA, "mrg_build: BLAS build: " + err); }
            pieces.push_back(Piece{ br.nodes, br.nodeCount, br.tris, br.payloadCount });
            for(size_t mi = 0; mi < M; mi++)
            {
                pieceOf[mi] = 0; meshRoot[mi] = (uint32_t)mi;
                std::memcpy(c->meshes[mi].box, &br.boxes[6 * mi], sizeof(c->meshes[mi].box));
            }
        }
        else
        {
            for(size_t mi = 0; mi < M; mi++)
            {
                auto& m = c->meshes[mi];
                mrg::BuildInput bi;
                bi.kind = 0; bi.pos = dPos[mi]; bi.idx = dIdx[mi];
                bi.count = (uint32_t)(m.idx.size() / 3);
                bi.primKeyBase = m.primKeyBase;
                bi.maxLeaf = leaf_size(bi.count);
                bi.ploc = true;
                bi.rawVerts = c->watertight;
                mrg::BuildResult b;
                if(!mrg::build_wide_bvh(bi, b, st, err))
                {
                    free_uploads(); free_pieces(); cudaStreamSynchronize(st);
                    return fail(MRG_ERR_CUDA, "mrg_build: BLAS build: " + err);
                }
                pieceOf[mi] = (uint32_t)pieces.size(); meshRoot[mi] = 0;
                pieces.push_back(Piece{ b.nodes, b.nodeCount, b.tris, b.payloadCount });
                std::memcpy(m.box, b.box, sizeof(m.box));
            }
            free_uploads();
        }
    }

    // 2. instance world boxes + TLAS
    const uint32_t ni = (uint32_t)c->insts.size();
    std::vector<float> instBoxes(6ull * ni);
    for(uint32_t i = 0; i < ni; i++)
        mrg::transform_box_conservative(c->insts[i].m, c->meshes[c->insts[i].mesh].box, &instBoxes[6ull * i]);
    for(int k = 0; k < 3; k++) { c->sceneBox[k] = 3.0e38f; c->sceneBox[3 + k] = -3.0e38f; }
    for(uint32_t i = 0; i < ni; i++)
        for(int k = 0; k < 3; k++)
        {
            c->sceneBox[k] = std::min(c->sceneBox[k], instBoxes[6ull * i + k]);
            c->sceneBox[3 + k] = std::max(c->sceneBox[3 + k], instBoxes[6ull * i + 3 + k]);
        }
    float* dBoxes = nullptr;
    mrg::BuildResult tlas;
    {
        cudaError_t e = cudaMalloc(&dBoxes, sizeof(float) * instBoxes.size());
        if(e == cudaSuccess) e = cudaMemcpyAsync(dBoxes, instBoxes.data(), sizeof(float) * instBoxes.size(), cudaMemcpyHostToDevice, st);
        if(e != cudaSuccess)
        {
            cudaFree(dBoxes);
            free_pieces();
            return cuda_fail(e, "mrg_build: instance boxes");
        }
        mrg::BuildInput bi;
        bi.kind = 1; bi.boxes = dBoxes; bi.count = ni; bi.maxLeaf = 1;
        bi.ploc = use_ploc();
        bool ok = mrg::build_wide_bvh(bi, tlas, st, err);
        cudaFree(dBoxes);
        if(!ok)
        {
            free_pieces();
            return fail(MRG_ERR_CUDA, "mrg_build: TLAS build: " + err);
        }
    }

    // 3. place everything in shared arrays
    uint64_t totalNodes = 0, totalTris = 0;
    for(auto& b : pieces) { totalNodes += b.nodeCount; totalTris += b.payloadCount; }
    const uint64_t tlasOff = totalNodes;
    totalNodes += tlas.nodeCount;
    cudaError_t e = cudaMalloc(&c->dNodes, mrg::kWideNodeBytes * totalNodes);
    if(e == cudaSuccess) e = cudaMalloc(&c->dTris, mrg::kTriRecordBytes * totalTris);
    if(e == cudaSuccess) e = cudaMalloc(&c->dInsts, sizeof(mrg::HostInstRecord) * ni);
    if(e == cudaSuccess) e = cudaMalloc(&c->dTlasLeaf, sizeof(uint32_t) * ni);
    uint64_t nodeOff = 0, triOff = 0;
    std::vector<uint64_t> pieceNodeOff(pieces.size());
    for(size_t pi = 0; pi < pieces.size() && e == cudaSuccess; pi++)
    {
        auto& b = pieces[pi];
        pieceNodeOff[pi] = nodeOff;
        if(!mrg::relocate_nodes(b.nodes, reinterpret_cast<mrg::WideNode*>(
                                    static_cast<char*>(c->dNodes) + mrg::kWideNodeBytes * nodeOff),
                                b.nodeCount, (uint32_t)nodeOff, (uint32_t)triOff, st))
            e = cudaErrorLaunchFailure;
        if(e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<char*>(c->dTris) + mrg::kTriRecordBytes * triOff, b.tris,
                                mrg::kTriRecordBytes * b.payloadCount, cudaMemcpyDeviceToDevice, st);
        nodeOff += b.nodeCount; triOff += b.payloadCount;
    }
    for(size_t mi = 0; mi < c->meshes.size(); mi++)
        c->meshes[mi].rootNode = (uint32_t)(pieceNodeOff[pieceOf[mi]] + meshRoot[mi]);
    if(e == cudaSuccess &&
       !mrg::relocate_nodes(tlas.nodes, reinterpret_cast<mrg::WideNode*>(
                                static_cast<char*>(c->dNodes) + mrg::kWideNodeBytes * tlasOff),
                            tlas.nodeCount, (uint32_t)tlasOff, 0u, st))
        e = cudaErrorLaunchFailure;
    if(e == cudaSuccess)
        e = cudaMemcpyAsync(c->dTlasLeaf, tlas.leafIds, sizeof(uint32_t) * ni, cudaMemcpyDeviceToDevice, st);
    std::vector<mrg::HostInstRecord> recs(ni);
    for(int k = 0; k < 3; k++) { c->sceneBoxExact[k] = 3.0e38f; c->sceneBoxExact[3 + k] = -3.0e38f; }
    for(uint32_t i = 0; i < ni; i++)
    {
        const auto& in = c->insts[i];
        std::memcpy(recs[i].inv, in.inv, sizeof(in.inv));
        recs[i].keys[0] = in.lm;
        recs[i].keys[1] = in.trans;
        recs[i].keys[2] = in.accel;
        recs[i].keys[3] = c->meshes[in.mesh].rootNode |
                          ((in.flags & MRG_INSTANCE_CULL_BACKFACE) ? 0x80000000u : 0u);
        float wb[6];
        mrg::transform_box_exact(in.m, c->meshes[in.mesh].box, wb);
        for(int k = 0; k < 3; k++)
        {
            recs[i].wmin[k] = wb[k]; recs[i].wmax[k] = wb[3 + k];
            c->sceneBoxExact[k] = std::min(c->sceneBoxExact[k], wb[k]);
            c->sceneBoxExact[3 + k] = std::max(c->sceneBoxExact[3 + k], wb[3 + k]);
        }
        recs[i].wmin[3] = 0.0f; recs[i].wmax[3] = 0.0f;
    }
    if(e == cudaSuccess)
        e = cudaMemcpyAsync(c->dInsts, recs.data(), sizeof(mrg::HostInstRecord) * ni, cudaMemcpyHostToDevice, st);
    if(e == cudaSuccess) e = cudaStreamSynchronize(st);
    free_pieces();
    cudaFree(tlas.nodes); cudaFree(tlas.leafIds);
    if(e != cudaSuccess) { free_accel(c); return cuda_fail(e, "mrg_build: placement"); }

    c->blasNodes = totalNodes - tlas.nodeCount;
    c->blasTris = totalTris;
    c->tlasNodes = tlas.nodeCount;
    c->scene.nodes = static_cast<const mrg::WideNode*>(c->dNodes);
    c->scene.tris = static_cast<const mrg::TriRecord*>(c->dTris);
    c->scene.insts = static_cast<const mrg::InstRecord*>(c->dInsts);
    c->scene.tlasLeaf = c->dTlasLeaf;
    c->scene.tlasRoot = (uint32_t)tlasOff;
    c->scene.instCount = ni;
    c->scene.nodeCount = (uint32_t)totalNodes;
    c->scene.triCount = (uint32_t)totalTris;
    c->scene.watertight = c->watertight ? 1u : 0u;
    c->built = true;
    c->buildMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return MRG_OK;
}

mrg_status mrg_cast_local(mrg_ctx* c, mrg_ray* dRays, const uint32_t* dIdx, const uint32_t* dInst, uint32_t n,
                          mrg_hit_keys* dHits, mrg_meta_hit* dMeta, void* stream)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_local: null context");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_cast_local: call mrg_build first");
    if(n == 0) return MRG_OK;
    if(!dRays || !dInst || !dHits || !dMeta) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_local: null buffer");
    if(reinterpret_cast<uintptr_t>(dRays) % 32 != 0 || reinterpret_cast<uintptr_t>(dHits) % 16 != 0 ||
       reinterpret_cast<uintptr_t>(dMeta) % 8 != 0)
        return fail(MRG_ERR_INVALID_ARG, "mrg_cast_local: misaligned buffer");
    DeviceGuard g(c->device);
    MRG_TRY(mrg::launch_local(c->scene, scratch_of(c), dRays, dIdx, dInst, n, dHits, dMeta, c->smCount,
                              static_cast<cudaStream_t>(stream)), "mrg_cast_local");
    return MRG_OK;
}

mrg_status mrg_cast_closest(mrg_ctx* c, mrg_ray* dRays, const uint32_t* dIdx, uint32_t n,
                            mrg_hit_keys* dHits, mrg_meta_hit* dMeta, void* stream)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest: null context");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_cast_closest: call mrg_build first");
    if(n == 0) return MRG_OK;
    if(!dRays || !dHits || !dMeta) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest: null buffer");
    if(reinterpret_cast<uintptr_t>(dRays) % 32 != 0 || reinterpret_cast<uintptr_t>(dHits) % 16 != 0 ||
       reinterpret_cast<uintptr_t>(dMeta) % 8 != 0)
        return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest: misaligned buffer");
    DeviceGuard g(c->device);
    const uint32_t* order = dIdx;
    if(cast_sort_enabled() && n >= kCoherenceSortMin)
    {
        // coherence sort: an index permutation only, results are per ray
        const size_t words = 4ull * n + mrg::multisplit_hist_words(n, 8);
        mrg_status s = mrg::partition_scratch(c, words);
        if(s != MRG_OK) return s;
        uint32_t* base = c->dPartScratch;
        uint32_t* sorted = nullptr;
        cudaError_t e = mrg::ray_coherence_order(dRays, dIdx, n, c->sceneBoxExact, base, base + n, base + 2ull * n,
                                                 base + 3ull * n, base + 4ull * n, sorted, c->smCount,
                                                 static_cast<cudaStream_t>(stream));
        if(e != cudaSuccess) return cuda_fail(e, "mrg_cast_closest: coherence sort");
        order = sorted;
    }
    cudaError_t e = mrg::launch_closest(c->scene, scratch_of(c), dRays, order, n, dHits, dMeta,
                                        c->smCount, static_cast<cudaStream_t>(stream));
    if(e != cudaSuccess) return cuda_fail(e, "mrg_cast_closest");
    return MRG_OK;
}

mrg_status mrg_cast_visibility(mrg_ctx* c, uint32_t* dVis, const mrg_ray* dRays,
                               const uint32_t* dIdx, uint32_t n, void* stream)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_visibility: null context");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_cast_visibility: call mrg_build first");
    if(n == 0) return MRG_OK;
    if(!dRays || !dVis) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_visibility: null buffer");
    if(reinterpret_cast<uintptr_t>(dRays) % 32 != 0 || reinterpret_cast<uintptr_t>(dVis) % 4 != 0)
        return fail(MRG_ERR_INVALID_ARG, "mrg_cast_visibility: misaligned buffer");
    DeviceGuard g(c->device);
    cudaError_t e = mrg::launch_visibility(c->scene, scratch_of(c), dVis, dRays, dIdx, n,
                                           c->smCount, static_cast<cudaStream_t>(stream));
    if(e != cudaSuccess) return cuda_fail(e, "mrg_cast_visibility");
    return MRG_OK;
}

mrg_status mrg_cast_closest_host(mrg_ctx* c, mrg_ray* hRays, uint32_t n, mrg_hit_keys* hHits,
                                 mrg_meta_hit* hMeta)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host: null context");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_cast_closest_host: call mrg_build first");
    if(n == 0) return MRG_OK;
    if(!hRays || !hHits || !hMeta) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host: null buffer");
    DeviceGuard g(c->device);
    if(n > c->stageCap)
    {
        cudaFree(c->dStageRays); cudaFree(c->dStageHits); cudaFree(c->dStageMeta);
        c->dStageRays = nullptr; c->dStageHits = nullptr; c->dStageMeta = nullptr; c->stageCap = 0;
        MRG_TRY(cudaMalloc(&c->dStageRays, sizeof(mrg_ray) * (size_t)n), "mrg_cast_closest_host: staging");
        MRG_TRY(cudaMalloc(&c->dStageHits, sizeof(mrg_hit_keys) * (size_t)n), "mrg_cast_closest_host: staging");
        MRG_TRY(cudaMalloc(&c->dStageMeta, sizeof(mrg_meta_hit) * (size_t)n), "mrg_cast_closest_host: staging");
        c->stageCap = n;
    }
    if(!c->hostStreams[0])
    {
        for(cudaStream_t& q : c->hostStreams)
            MRG_TRY(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking), "mrg_cast_closest_host: streams");
        for(cudaEvent_t& q : c->hostEvents)
            MRG_TRY(cudaEventCreateWithFlags(&q, cudaEventDisableTiming), "mrg_cast_closest_host: events");
        MRG_TRY(cudaMalloc(&c->dHostCounters, sizeof(uint32_t) * mrg_ctx::kHostMaxChunks), "mrg_cast_closest_host: counters");
    }
    // The ray set goes through in chunks: while chunk k is cast, chunk k+1
    // is copied in and chunk k-1 copied out (copy engines in both directions
    // run beside the SMs).  Casts alternate between two streams, each chunk
    // with its own ray-claim counter, so chunk k+1's blocks take the SMs that
    // chunk k's last rays leave idle.  Each chunk owns its slice of the
    // staging buffers.
    const uint32_t chunks = host_chunks(n);
    cudaStream_t sIn = c->hostStreams[0], sOut = c->hostStreams[3];
    // Chunk k covers rays [edge(k), edge(k + 1)).  With three or more chunks the
    // first and last weigh a quarter of the others: the copy-in before the
    // first cast and the copy-out after the last one are not overlapped.
    const double wEnd = (chunks >= 3) ? 0.25 : 1.0;
    const double wSum = (chunks >= 3) ? 2.0 * wEnd + (double)(chunks - 2) : (double)chunks;
    auto edge = [&](uint32_t k) -> size_t {
        if(k == 0) return 0;
        if(k >= chunks) return n;
        const double w = (chunks >= 3) ? wEnd + (double)(k - 1) : (double)k;
        return std::min((size_t)n, (size_t)((double)n * w / wSum));
    };
    for(uint32_t k = 0; k < chunks; k++)
    {
        cudaStream_t sCast = c->hostStreams[1 + (k & 1u)];
        mrg::TraceScratch scr = scratch_of(c);
        scr.workCounter = c->dHostCounters + k;
        const size_t off = edge(k), cnt = edge(k + 1) - off;
        if(cnt == 0) continue;
        cudaEvent_t copied = c->hostEvents[2 * k], cast = c->hostEvents[2 * k + 1];
        MRG_TRY(cudaMemcpyAsync(c->dStageRays + off, hRays + off, sizeof(mrg_ray) * cnt, cudaMemcpyHostToDevice, sIn), "H2D rays");
        MRG_TRY(cudaMemcpyAsync(c->dStageHits + off, hHits + off, sizeof(mrg_hit_keys) * cnt, cudaMemcpyHostToDevice, sIn), "H2D hits");
        MRG_TRY(cudaMemcpyAsync(c->dStageMeta + off, hMeta + off, sizeof(mrg_meta_hit) * cnt, cudaMemcpyHostToDevice, sIn), "H2D meta");
        MRG_TRY(cudaEventRecord(copied, sIn), "event");
        MRG_TRY(cudaStreamWaitEvent(sCast, copied, 0), "event wait");
        MRG_TRY(mrg::launch_closest(c->scene, scr, c->dStageRays + off, nullptr, (uint32_t)cnt,
                                    c->dStageHits + off, c->dStageMeta + off, c->smCount, sCast), "cast");
        MRG_TRY(cudaEventRecord(cast, sCast), "event");
        MRG_TRY(cudaStreamWaitEvent(sOut, cast, 0), "event wait");
        MRG_TRY(cudaMemcpyAsync(hRays + off, c->dStageRays + off, sizeof(mrg_ray) * cnt, cudaMemcpyDeviceToHost, sOut), "D2H rays");
        MRG_TRY(cudaMemcpyAsync(hHits + off, c->dStageHits + off, sizeof(mrg_hit_keys) * cnt, cudaMemcpyDeviceToHost, sOut), "D2H hits");
        MRG_TRY(cudaMemcpyAsync(hMeta + off, c->dStageMeta + off, sizeof(mrg_meta_hit) * cnt, cudaMemcpyDeviceToHost, sOut), "D2H meta");
    }
    return mrg_sync_status(c, sOut);
}

mrg_status mrg_scene_aabb(mrg_ctx* c, float out[6])
{
    if(!c || !out) return fail(MRG_ERR_INVALID_ARG, "mrg_scene_aabb: null pointer");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_scene_aabb: call mrg_build first");
    std::memcpy(out, c->sceneBoxExact, sizeof(c->sceneBoxExact));
    return MRG_OK;
}

mrg_status mrg_get_stats(mrg_ctx* c, mrg_accel_stats* out)
{
    if(!c || !out) return fail(MRG_ERR_INVALID_ARG, "mrg_get_stats: null pointer");
    out->blasNodes = c->blasNodes;
    out->blasTriangles = c->blasTris;
    out->tlasNodes = c->tlasNodes;
    out->instances = c->insts.size();
    out->deviceBytes = mrg::kWideNodeBytes * (c->blasNodes + c->tlasNodes) +
                       mrg::kTriRecordBytes * c->blasTris +
                       (sizeof(mrg::HostInstRecord) + 4) * c->insts.size();
    out->buildMs = c->buildMs;
    out->accelerators = c->built ? c->meshes.size() : 0;
    return MRG_OK;
}

mrg_status mrg_sync_status(mrg_ctx* c, void* stream)
{
    if(!c) return fail(MRG_ERR_INVALID_ARG, "mrg_sync_status: null context");
    DeviceGuard g(c->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MRG_TRY(cudaStreamSynchronize(st), "mrg_sync_status: stream");
    uint32_t flag = 0;
    MRG_TRY(cudaMemcpy(&flag, c->dScratch + 1, sizeof(flag), cudaMemcpyDeviceToHost), "mrg_sync_status: read flag");
    if(flag)
    {
        MRG_TRY(cudaMemset(c->dScratch + 1, 0, sizeof(uint32_t)), "mrg_sync_status: clear flag");
        if(flag & mrg::kNrcWaitTimeout)
            return fail(MRG_ERR_CUDA, "a tensor-core kernel's barrier wait ran out");
        return fail(MRG_ERR_TRAVERSAL, (flag & mrg::kTraceStackOverflow) ? "traversal stack overflow"
                                       : (flag & mrg::kTraceBadIndex) ? "traversal read an out-of-range index"
                                                                      : "traversal step cap reached");
    }
    return MRG_OK;
}

mrg_status mrg_cast_closest_stats(mrg_ctx* c, const mrg_ray* dRays, uint32_t n,
                                  uint64_t out[8], void* stream)
{
    if(!c || !out) return fail(MRG_ERR_INVALID_ARG, "mrg_cast_closest_stats: null pointer");
    if(!c->built) return fail(MRG_ERR_NOT_BUILT, "mrg_cast_closest_stats: call mrg_build first");
    DeviceGuard g(c->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MRG_TRY(mrg::launch_closest_stats(c->scene, scratch_of(c), dRays, n, c->smCount, st), "stats cast");
    unsigned long long h[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    MRG_TRY(cudaMemcpyAsync(h, c->dStats, sizeof(h), cudaMemcpyDeviceToHost, st), "stats read");
    MRG_TRY(cudaStreamSynchronize(st), "stats sync");
    for(int i = 0; i < 8; i++) out[i] = h[i];
    return MRG_OK;
}

} // extern "C"
