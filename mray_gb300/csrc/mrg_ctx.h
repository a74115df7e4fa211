// mrg_ctx.h -- private definition of the C-ABI context (shared by the
// translation units that implement include/mray_gb300.h).
#pragma once
#include "mray_gb300.h"
#include "mrg_build.h"
#include "mrg_pt.h"
#include "mrg_guide.h"
#include "mrg_partition.h"
#include "mrg_nrc.h"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace mrg {

// Device-side record layouts, mirrored on the host for uploads.
struct HostInstRecord
{
    float    inv[12];
    uint32_t keys[4];
    float    wmin[4];
    float    wmax[4];
};
static_assert(sizeof(HostInstRecord) == 96, "instance record is 96 bytes");
constexpr size_t kWideNodeBytes = MRG_NODE_F16 ? 128 : 80;
constexpr size_t kTriRecordBytes = 48;

} // namespace mrg

struct mrg_ctx
{
    int device = 0;
    int smCount = 0;
    bool watertight = false;          // triangle test: watertight instead of MRay's Moller-Trumbore
    cudaStream_t buildStream = nullptr;

    struct Mesh
    {
        std::vector<float>    pos;
        std::vector<uint32_t> idx;
        uint32_t              primKeyBase = 0;
        std::vector<float>    uv;             // per-vertex texture coordinates (optional)
        float                 box[6] = { 0, 0, 0, 0, 0, 0 };
        uint32_t              rootNode = 0;
    };
    struct Inst
    {
        uint32_t mesh = 0;
        float    m[12];
        float    inv[12];
        uint32_t flags = 0, lm = 0, trans = 0, accel = 0;
    };
    std::vector<Mesh> meshes;
    std::vector<Inst> insts;
    bool built = false;

    // accelerator (device)
    void*     dNodes = nullptr;
    void*     dTris = nullptr;
    void*     dInsts = nullptr;
    uint32_t* dTlasLeaf = nullptr;
    uint64_t  blasNodes = 0, blasTris = 0, tlasNodes = 0;
    mrg::TraceScene scene;
    float     sceneBox[6] = { 0, 0, 0, 0, 0, 0 };        // conservative (TLAS) box
    float     sceneBoxExact[6] = { 0, 0, 0, 0, 0, 0 };   // union of the exact instance boxes
    double    buildMs = 0.0;

    // scratch: [0] work counter, [1] error flag; stats in a separate block
    uint32_t*           dScratch = nullptr;
    unsigned long long* dStats = nullptr;

    // path tracer: per-instance surface description, device tables, path state
    struct PtSurfaceDesc
    {
        int      kind = 0;            // 0 unset, 1 material, 2 area light
        uint32_t material = 0;        // MRG_MAT_*
        float    albedo[3] = { 0, 0, 0 };
        float    roughness = 0, metallic = 0, specular = 0;
        float    iorFront = 1, iorBack = 1;
        float    radiance[3] = { 0, 0, 0 };
        uint32_t twoSided = 0;
        uint32_t texture = 0;         // albedo texture id + 1 (0: constant albedo)
        uint32_t paramTex[3] = { 0, 0, 0 };  // Unreal roughness / metallic / specular texture id + 1
    };
    struct PtTextureDesc
    {
        uint32_t             width = 0, height = 0, format = 0;   // 0 RGBA8 unorm, 1 RGBA f32
        std::vector<uint8_t> host;             // owned copy, or empty when borrowed
        const void*          borrowed = nullptr;
        float                mipRadius = 0.0f;  // > 0: a mip chain made with this Gaussian radius
        std::vector<std::vector<uint8_t>> given;  // mip level -> texels set by the caller (level 0 unused)
    };
    std::vector<PtTextureDesc> ptTextures;
    void*     dPtTexTable = nullptr;           // PtTexture per texture
    void*     dPtTexData = nullptr;            // owned texel copies
    void*     dPtMipData = nullptr;            // mip levels 1.. of the textures that have a chain
    void*     dPtUvs = nullptr;                // 2 float4 per primitive
    void*     dPtRadTotal = nullptr;           // adjoint: primal radiance per path slot
    uint32_t  ptRadTotalCap = 0;
    std::vector<PtSurfaceDesc> ptDesc;       // indexed by instance
    bool      ptDirty = true;
    void*     dPtSurfaces = nullptr;
    void*     dPtLights = nullptr;
    void*     dPtTris = nullptr;
    uint32_t  ptSurfaceCount = 0, ptLightCount = 0, ptTriCount = 0;
    uint32_t  ptMaterialGroups = 0;          // distinct material groups among surfaces
    mrg::PtPaths ptPaths{};
    // shadow casts of bounce d overlap the closest-hit cast of bounce d + 1
    cudaStream_t ptSideStream = nullptr;
    cudaEvent_t  ptEvShaded = nullptr, ptEvResolved = nullptr;
    // second pass pipeline of mrg_pt_render: its own path state, streams,
    // events; ptEvFilm orders the film writes of consecutive passes
    mrg::PtPaths ptPaths2{};
    void*        ptPathMem2 = nullptr;
    cudaStream_t ptStream2 = nullptr, ptSideStream2 = nullptr;
    cudaEvent_t  ptEvShaded2 = nullptr, ptEvResolved2 = nullptr;
    cudaEvent_t  ptEvFilm = nullptr, ptEvStart = nullptr, ptEvDone2 = nullptr;
    void*        dPtRadTotal2 = nullptr;      // adjoint: primal radiance of the second pipeline
    uint32_t     ptRadTotalCap2 = 0;
    double*      dPtGradEmission = nullptr;   // adjoint: FP64 emission-gradient sums, RGBA per instance
    uint32_t*    dZsTables = nullptr;         // ZSobol sampler: matrices and digit permutations
    uint32_t*    dZsSeeds = nullptr;          // ZSobol sampler: per-pixel seeds of (zsW, zsH, zsSeed)
    uint32_t     zsW = 0, zsH = 0, zsSeed = 0;
    uint32_t     ptGradEmissionCap = 0;       // instances
    void*     ptPathMem = nullptr;
    // skysphere boundary light: host copy of the radiance map and transform,
    // device block [texels | cdfX | cdfY]
    bool               ptEnvSet = false;
    uint32_t           ptEnvW = 0, ptEnvH = 0;
    std::vector<float> ptEnvTexels;          // RGBA per texel
    float              ptEnvM[12] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0 };
    void*              dPtEnv = nullptr;
    mrg::PtEnv         ptEnv{};
    // spectral context: device block [lut | observer | illuminant]
    void*              dPtSpec = nullptr;
    mrg::PtSpectral    ptSpec{};

    // guided path tracing: the hash grid block (codes, counter, chain and
    // irradiance state) and the per-slot guided path state
    bool               guideOn = false;
    mrg_guide_params   guidePrm{};
    void*              dGuideGrid = nullptr;
    mrg::GuideGrid     guide{};
    bool               guideCamSet = false;
    void*              dGuidePaths = nullptr;
    mrg::GuidePaths    guideQ{};
    uint32_t           guideCap = 0;              // slots the path state holds
    bool               guideBkValid = false;      // backup streams of (guideBkSeed, W, H, slots)
    uint32_t           guideBkSeed = 0, guideBkW = 0, guideBkH = 0;

    // radiance cache (one per context) and its path-tracer buffers
    void*              dPtCacheBuf = nullptr;
    size_t             ptCacheBufBytes = 0;
    bool               cacheOn = false;
    mrg::NrcState      cache{};
    std::vector<void*> cacheAllocs;

    // ray partitioner scratch (grow-only)
    uint32_t* dPartScratch = nullptr;
    size_t    partScratchWords = 0;

    // staging for the host-buffer cast
    mrg_ray*      dStageRays = nullptr;
    mrg_hit_keys* dStageHits = nullptr;
    mrg_meta_hit* dStageMeta = nullptr;
    size_t        stageCap = 0;
    // host-buffer cast pipeline: copy-in, cast and copy-out streams, and the
    // events that chain one chunk through them
    static constexpr int kHostMaxChunks = 32;
    cudaStream_t  hostStreams[4] = { nullptr, nullptr, nullptr, nullptr };   // in, cast A, cast B, out
    cudaEvent_t   hostEvents[2 * kHostMaxChunks] = {};
    uint32_t*     dHostCounters = nullptr;       // one ray-claim counter per chunk
};

namespace mrg {

// Records the calling thread's last error message (mrg_last_error) and
// returns the status.
mrg_status set_error(mrg_status s, const std::string& msg);
// Grows the context's partitioner scratch to `words` 32-bit words.
mrg_status partition_scratch(mrg_ctx* c, size_t words);
// Called by mrg_create with `device` current: loads the module that holds the
// allocation-free cast's static array and the closest-hit kernel (both are
// allocated by the driver when their module loads) and records the array's
// device address, so that mrg_cast_closest_host_noalloc itself never makes the
// driver allocate.
mrg_status noalloc_prepare(int device);

} // namespace mrg
