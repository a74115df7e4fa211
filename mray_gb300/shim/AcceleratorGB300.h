// AcceleratorGB300.h -- MRay-side adapter: a BaseAcceleratorI (Source/Tracer/
// AcceleratorC.h:375-430) that forwards every cast to the mray_gb300 C ABI.
//
// This header is compiled inside MRay's TracerDLL (it includes MRay's own
// headers); it is not part of libmray_gb300.so.  It is registered as an
// accelerator type by a generator line in Tracer::AddAccelGenerators
// (Source/TracerDLL/Tracer.cu:139-169) under the HARDWARE slot.
//
// Construct turns MRay's scene description into the library's meshes and
// instances the way MRay's accelerators read it (BaseAccelerator /
// AcceleratorGroup::LinearizeSurfaceData, Source/Tracer/AcceleratorCommon.cu:
// 280-370): each primitive batch of a surface becomes one instance of that
// batch's triangle mesh (meshes are shared between surfaces that use the same
// batch), with MRay's keys -- transform key = the surface's TransformId, light
// or material key = CombinedKey(IS_MAT_KEY_FLAG, material batch, index), or
// the light flag and the light's key for a primitive-backed light surface,
// primitive keys = CombinedKey(primitive group, index in the group) -- and the
// surface's back-face culling flag.  Triangle data and transforms are read
// from MRay's groups (PrimGroupTriangle::SoA after Finalize made the indices
// group-global; TransformGroupSingle::SoA), copied to the host once per build.
#pragma once

#include "Tracer/AcceleratorC.h"
#include "Tracer/PrimitiveDefaultTriangle.h"
#include "Tracer/TransformsDefault.h"
#include "Tracer/LightC.h"

#include "mray_gb300.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#ifdef MRAY_GPU_BACKEND_CUDA
#include <cuda_runtime.h>
#endif

// The C ABI's records are MRay's own layouts; the casts reinterpret the
// caller's spans in place.
static_assert(sizeof(RayGMem) == sizeof(mrg_ray) && alignof(RayGMem) == 32,
              "RayGMem must be the 32-byte record mrg_ray describes");
static_assert(offsetof(RayGMem, pos) == offsetof(mrg_ray, pos) && offsetof(RayGMem, tMin) == offsetof(mrg_ray, tMin) &&
              offsetof(RayGMem, dir) == offsetof(mrg_ray, dir) && offsetof(RayGMem, tMax) == offsetof(mrg_ray, tMax),
              "RayGMem field offsets");
static_assert(sizeof(HitKeyPack) == sizeof(mrg_hit_keys), "HitKeyPack must be the 16-byte record mrg_hit_keys describes");
static_assert(offsetof(HitKeyPack, primKey) == offsetof(mrg_hit_keys, primKey) &&
              offsetof(HitKeyPack, lightOrMatKey) == offsetof(mrg_hit_keys, lightOrMatKey) &&
              offsetof(HitKeyPack, transKey) == offsetof(mrg_hit_keys, transKey) &&
              offsetof(HitKeyPack, accelKey) == offsetof(mrg_hit_keys, accelKey),
              "HitKeyPack field order");
static_assert(sizeof(MetaHit) >= sizeof(mrg_meta_hit), "a triangle MetaHit holds the two barycentrics");
static_assert(sizeof(PrimitiveKey) == 4 && sizeof(LightOrMatKey) == 4 && sizeof(TransformKey) == 4 &&
              sizeof(AcceleratorKey) == 4, "32-bit keys");
static_assert(sizeof(Matrix3x4) == 12 * sizeof(float), "row-major 3x4 transforms");

class BaseAcceleratorGB300 final : public BaseAcceleratorI
{
    mrg_ctx*                ctx = nullptr;
    std::vector<uint32_t>   accelKeyToInstance;     // AcceleratorKey index portion -> library instance
    uint32_t*               dInstOfKey = nullptr;   // the same table on the device (CastLocalRays)

    static void Check(mrg_status s, const char* what)
    {
        if(s != MRG_OK) throw MRayError("mray_gb300: {}: {}", what, mrg_last_error());
    }

    static void* StreamOf([[maybe_unused]] const GPUQueue& q)
    {
        #ifdef MRAY_GPU_BACKEND_CUDA
            return static_cast<void*>(mray::cuda::ToHandleCUDA(q));
        #else
            return nullptr;
        #endif
    }

    // Device spans of the CUDA backend are device pointers; the host
    // backend's are host memory.
    static void ToHost(void* dst, const void* src, size_t bytes)
    {
        #ifdef MRAY_GPU_BACKEND_CUDA
            if(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
                throw MRayError("mray_gb300: reading MRay's scene data from the device failed");
        #else
            std::memcpy(dst, src, bytes);
        #endif
    }

    static Matrix3x4 TransformOf(const BaseAccelConstructParams& p, TransformKey tk)
    {
        auto it = p.transformGroups.find(TransGroupId(tk.FetchBatchPortion()));
        if(it == p.transformGroups.end()) throw MRayError("mray_gb300: unknown transform group");
        const GenericGroupTransformT* tg = it->second.get();
        if(dynamic_cast<const TransformGroupIdentity*>(tg)) return Matrix3x4::Identity();
        if(const auto* ts = dynamic_cast<const TransformGroupSingle*>(tg))
        {
            Matrix3x4 m;
            ToHost(&m, ts->SoA().transforms.data() + tk.FetchIndexPortion(), sizeof(Matrix3x4));
            return m;
        }
        throw MRayError("mray_gb300: only identity and single transforms are supported");
    }

    // The batch's triangles as a local mesh (vertices rebased to the batch's
    // used range), uploaded once; primitive keys start at the batch's first
    // group-wide primitive index.
    uint32_t MeshOf(const BaseAccelConstructParams& p, PrimBatchKey bk, std::map<CommonKey, uint32_t>& meshes)
    {
        const CommonKey id = std::bit_cast<CommonKey>(bk);
        if(auto it = meshes.find(id); it != meshes.end()) return it->second;
        auto git = p.primGroups.find(PrimGroupId(bk.FetchBatchPortion()));
        if(git == p.primGroups.end()) throw MRayError("mray_gb300: unknown primitive group");
        const auto* tri = dynamic_cast<const PrimGroupTriangle*>(git->second.get());
        if(!tri) throw MRayError("mray_gb300: only triangle primitive groups are supported");
        const Vector2ui range = tri->BatchRange(bk);
        const uint32_t nt = range[1] - range[0];
        const DefaultTriangleDetail::TriangleData soa = tri->SoA();
        std::vector<Vector3ui> idx(nt);
        ToHost(idx.data(), soa.indexList.data() + range[0], sizeof(Vector3ui) * nt);
        uint32_t lo = ~0u, hi = 0u;
        for(const Vector3ui& t : idx)
            for(uint32_t k = 0; k < 3; k++) { lo = std::min(lo, t[k]); hi = std::max(hi, t[k]); }
        const uint32_t nv = hi - lo + 1u;
        std::vector<Vector3> pos(nv);
        ToHost(pos.data(), soa.positions.data() + lo, sizeof(Vector3) * nv);
        std::vector<uint32_t> local(3 * size_t(nt));
        for(uint32_t i = 0; i < nt; i++)
            for(uint32_t k = 0; k < 3; k++) local[3 * size_t(i) + k] = idx[i][k] - lo;
        const PrimitiveKey base = PrimitiveKey::CombinedKey(bk.FetchBatchPortion(), range[0]);
        uint32_t mesh = 0;
        Check(mrg_upload_mesh(ctx, reinterpret_cast<const float*>(pos.data()), nv, local.data(), nt,
                              std::bit_cast<uint32_t>(base), &mesh), "mrg_upload_mesh");
        meshes.emplace(id, mesh);
        return mesh;
    }

    void AddInstance(uint32_t mesh, const Matrix3x4& m, bool cull, LightOrMatKey lmk, TransformKey tk)
    {
        const uint32_t n = uint32_t(accelKeyToInstance.size());
        const AcceleratorKey ak = AcceleratorKey::CombinedKey(0, n);
        uint32_t inst = 0;
        Check(mrg_add_instance(ctx, mesh, reinterpret_cast<const float*>(&m), cull ? MRG_INSTANCE_CULL_BACKFACE : 0u,
                               std::bit_cast<uint32_t>(lmk), std::bit_cast<uint32_t>(tk),
                               std::bit_cast<uint32_t>(ak), &inst), "mrg_add_instance");
        accelKeyToInstance.push_back(inst);
    }

    public:
    explicit BaseAcceleratorGB300(int device = 0, uint32_t triangleTest = MRG_TRI_MOLLER_TRUMBORE)
    {
        mrg_params p{};
        p.device = device;
        p.triangle_test = triangleTest;
        Check(mrg_create(&p, &ctx), "mrg_create");
    }
    ~BaseAcceleratorGB300() override
    {
        #ifdef MRAY_GPU_BACKEND_CUDA
            cudaFree(dInstOfKey);
        #endif
        mrg_destroy(ctx);
    }
    BaseAcceleratorGB300(const BaseAcceleratorGB300&) = delete;
    BaseAcceleratorGB300& operator=(const BaseAcceleratorGB300&) = delete;

    // BaseAccelerator::Construct (AcceleratorCommon.cu:709-805)
    void Construct(BaseAccelConstructParams p) override
    {
        std::map<CommonKey, uint32_t> meshes;
        accelKeyToInstance.clear();
        for(const auto& [surfId, surf] : p.mSurfList)
        {
            const TransformKey tk = std::bit_cast<TransformKey>(surf.transformId);
            const Matrix3x4 m = TransformOf(p, tk);
            for(size_t i = 0; i < surf.primBatches.size(); i++)
            {
                const PrimBatchKey bk = std::bit_cast<PrimBatchKey>(surf.primBatches[i]);
                const MaterialKey mk = std::bit_cast<MaterialKey>(surf.materials[i]);
                const LightOrMatKey lmk = LightOrMatKey::CombinedKey(IS_MAT_KEY_FLAG, mk.FetchBatchPortion(),
                                                                     mk.FetchIndexPortion());
                AddInstance(MeshOf(p, bk, meshes), m, surf.cullFaceFlags[i], lmk, tk);
            }
        }
        for(const auto& [lSurfId, lSurf] : p.lSurfList)
        {
            const LightKey lk = std::bit_cast<LightKey>(lSurf.lightId);
            auto lit = p.lightGroups.find(LightGroupId(lk.FetchBatchPortion()));
            if(lit == p.lightGroups.end() || !lit->second->IsPrimitiveBacked()) continue;   // no geometry
            const PrimBatchKey bk = lit->second->LightPrimBatch(lk);
            const TransformKey tk = std::bit_cast<TransformKey>(lSurf.transformId);
            const LightOrMatKey lmk = LightOrMatKey::CombinedKey(IS_LIGHT_KEY_FLAG, lk.FetchBatchPortion(),
                                                                 lk.FetchIndexPortion());
            // lights are ray sinks seen from both sides
            AddInstance(MeshOf(p, bk, meshes), TransformOf(p, tk), false, lmk, tk);
        }
        Check(mrg_build(ctx), "mrg_build");
        #ifdef MRAY_GPU_BACKEND_CUDA
            cudaFree(dInstOfKey);
            dInstOfKey = nullptr;
            const size_t bytes = sizeof(uint32_t) * std::max<size_t>(1, accelKeyToInstance.size());
            if(cudaMalloc(&dInstOfKey, bytes) != cudaSuccess ||
               cudaMemcpy(dInstOfKey, accelKeyToInstance.data(), sizeof(uint32_t) * accelKeyToInstance.size(),
                          cudaMemcpyHostToDevice) != cudaSuccess)
                throw MRayError("mray_gb300: instance table upload failed");
        #endif
    }

    // AllocateForTraversal: the casts need no per-ray scratch
    void AllocateForTraversal(size_t) override {}

    // CastRays (AcceleratorC.h:391-398).  Volume indices and the backup RNG
    // states are left untouched (no media; no stochastic alpha).
    void CastRays(Span<VolumeIndex>, Span<HitKeyPack> dHitIds, Span<MetaHit> dHitParams,
                  Span<BackupRNGState>, Span<RayGMem> dRays, Span<const RayIndex> dRayIndices,
                  bool, const GPUQueue& q) override
    {
        Check(mrg_cast_closest(ctx, reinterpret_cast<mrg_ray*>(dRays.data()),
                               reinterpret_cast<const uint32_t*>(dRayIndices.data()),
                               uint32_t(dRayIndices.size()), reinterpret_cast<mrg_hit_keys*>(dHitIds.data()),
                               reinterpret_cast<mrg_meta_hit*>(dHitParams.data()), StreamOf(q)),
              "mrg_cast_closest");
    }

    // CastVisibilityRays (AcceleratorC.h:400-405)
    void CastVisibilityRays(Bitspan<uint32_t> dIsVisible, Span<BackupRNGState>, Span<const RayGMem> dRays,
                            Span<const RayIndex> dRayIndices, const GPUQueue& q) override
    {
        Check(mrg_cast_visibility(ctx, dIsVisible.Data(), reinterpret_cast<const mrg_ray*>(dRays.data()),
                                  reinterpret_cast<const uint32_t*>(dRayIndices.data()),
                                  uint32_t(dRayIndices.size()), StreamOf(q)),
              "mrg_cast_visibility");
    }

    // CastLocalRays (AcceleratorC.h:407-421): the accelerator keys this
    // adapter assigned index the instance table it uploaded in Construct.
    // The library's local cast takes instance indices; on the CUDA backend a
    // gather of dAccelKeys through that table precedes it (one small kernel
    // of the TracerDLL); the host backend gathers on the host.
    void CastLocalRays(Span<VolumeIndex>, Span<HitKeyPack> dHitIds, Span<MetaHit> dHitParams,
                       Span<BackupRNGState>, Span<RayGMem> dRays, Span<const RayIndex> dRayIndices,
                       Span<const AcceleratorKey> dAccelKeys, CommonKey, bool, const GPUQueue& q) override
    {
        const uint32_t n = uint32_t(dRayIndices.size());
        #ifdef MRAY_GPU_BACKEND_CUDA
            uint32_t* dInst = GatherInstances(dAccelKeys, q);
        #else
            std::vector<uint32_t> inst(n);
            for(uint32_t i = 0; i < n; i++)
            {
                const uint32_t k = dAccelKeys[i].FetchIndexPortion();
                inst[i] = (k < accelKeyToInstance.size()) ? accelKeyToInstance[k] : ~0u;
            }
            const uint32_t* dInst = inst.data();
        #endif
        Check(mrg_cast_local(ctx, reinterpret_cast<mrg_ray*>(dRays.data()),
                             reinterpret_cast<const uint32_t*>(dRayIndices.data()), dInst, n,
                             reinterpret_cast<mrg_hit_keys*>(dHitIds.data()),
                             reinterpret_cast<mrg_meta_hit*>(dHitParams.data()), StreamOf(q)),
              "mrg_cast_local");
    }

    #ifdef MRAY_GPU_BACKEND_CUDA
    // Defined in the TracerDLL's CUDA translation unit beside the adapter:
    // out[i] = dInstOfKey[dAccelKeys[i].FetchIndexPortion()] on q's stream.
    uint32_t* GatherInstances(Span<const AcceleratorKey> dAccelKeys, const GPUQueue& q);
    #endif

    // SceneAABB / GPUMemoryUsage / TotalAccelCount / TotalInstanceCount
    // (AcceleratorC.h:416-428)
    AABB3 SceneAABB() const override
    {
        float b[6];
        Check(mrg_scene_aabb(ctx, b), "mrg_scene_aabb");
        return AABB3(Vector3(b[0], b[1], b[2]), Vector3(b[3], b[4], b[5]));
    }
    size_t GPUMemoryUsage() const override { return Stats().deviceBytes; }
    size_t TotalAccelCount() const override { return Stats().accelerators; }
    size_t TotalInstanceCount() const override { return Stats().instances; }
    std::string_view Name() const override { return "GB300"; }

    mrg_accel_stats Stats() const
    {
        mrg_accel_stats s{};
        Check(mrg_get_stats(ctx, &s), "mrg_get_stats");
        return s;
    }
    // The adapter's instance index of an accelerator key it assigned.
    uint32_t InstanceOf(AcceleratorKey k) const
    {
        const uint32_t i = k.FetchIndexPortion();
        return (i < accelKeyToInstance.size()) ? accelKeyToInstance[i] : ~0u;
    }
};
