// noalloc.cu -- closest-hit cast on host buffers that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they cast rays: a
// host application that owns every device allocation through its own
// memory manager (MRay's GPUSystem/DeviceMemory hands out all device memory),
// or a real-time or plugin thread that is not allowed to grow the device heap
// between frames.  For them this entry point keeps its device staging (rays,
// hit keys, meta hits) and its control words (work counter, error flag) in
// one file-scope __device__ array that is part of the library image.  The
// accelerator itself still comes from mrg_build.
#include "mrg_ctx.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

namespace {

constexpr size_t kCtrlBytes = 256;
constexpr size_t kRayBytes = sizeof(mrg_ray);            // 32
constexpr size_t kHitBytes = sizeof(mrg_hit_keys);       // 16
constexpr size_t kMetaBytes = sizeof(mrg_meta_hit);      // 8
constexpr size_t kMaxRays = MRG_NOALLOC_MAX_RAYS;
constexpr size_t kScratchBytes = kCtrlBytes + kMaxRays * (kRayBytes + kHitBytes + kMetaBytes);

// Layout: [0, 256) control words (u32 work counter, u32 error flag);
// then rays[kMaxRays], hits[kMaxRays], meta[kMaxRays].  The driver allocates
// these ~14 MiB on a device when the module loads there (at the latest in the
// first mrg_create on that device) and holds them until the process exits.
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setupMutex;
unsigned char* g_scratchAddr[kMaxDevices] = {};

// Looks up the device address of g_noallocScratch on `device` (which must be
// current) and records it.  In host code the symbol name is only a host-side
// stand-in, so kernels and copies must use this address.  The lookup also
// loads the module that holds the array, which is when the driver allocates
// it.  mrg_create calls this for every new context, so a context created
// after a device reset sees the re-loaded array's address.
mrg_status resolve_scratch(int device)
{
    if(device < 0 || device >= kMaxDevices)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host_noalloc: device ordinal out of range");
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if(e != cudaSuccess || p == nullptr)
    {
        cudaGetLastError();
        return mrg::set_error(MRG_ERR_CUDA, std::string("mrg_cast_closest_host_noalloc: "
                              "cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    }
    std::lock_guard<std::mutex> lock(g_setupMutex);
    g_scratchAddr[device] = static_cast<unsigned char*>(p);
    return MRG_OK;
}

mrg_status scratch_address(int device, unsigned char** out)
{
    if(device < 0 || device >= kMaxDevices)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host_noalloc: device ordinal out of range");
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        *out = g_scratchAddr[device];
    }
    if(*out == nullptr)   // every context comes from mrg_create, which resolves it
        return mrg::set_error(MRG_ERR_CUDA, "mrg_cast_closest_host_noalloc: staging array not set up on this device");
    return MRG_OK;
}

mrg_status cuda_err(cudaError_t e, const char* what)
{
    cudaGetLastError();
    return mrg::set_error(MRG_ERR_CUDA, std::string("mrg_cast_closest_host_noalloc: ") + what + ": " +
                          cudaGetErrorString(e));
}

} // namespace

mrg_status mrg::noalloc_prepare(int device)
{
    mrg_status s = resolve_scratch(device);
    if(s != MRG_OK) return s;
    cudaError_t e = mrg::preload_closest();
    if(e != cudaSuccess) return cuda_err(e, "loading the closest-hit kernel");
    return MRG_OK;
}

extern "C" mrg_status mrg_cast_closest_host_noalloc(mrg_ctx* c, mrg_ray* hRays, uint32_t n,
                                                    mrg_hit_keys* hHits, mrg_meta_hit* hMeta)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host_noalloc: null context");
    if(!c->built) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cast_closest_host_noalloc: call mrg_build first");
    if(n == 0) return MRG_OK;
    if(!hRays || !hHits || !hMeta)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cast_closest_host_noalloc: null buffer");
    if(n > kMaxRays)
        return mrg::set_error(MRG_ERR_LIMIT, "mrg_cast_closest_host_noalloc: " + std::to_string(n) +
                              " rays exceed the static staging capacity of " + std::to_string(kMaxRays) +
                              " (MRG_NOALLOC_MAX_RAYS); split the batch or use mrg_cast_closest_host");

    int prev = -1;
    if(cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if(prev != c->device) cudaSetDevice(c->device);
    struct Restore { int d; ~Restore() { if(d >= 0) cudaSetDevice(d); } } restore{ prev };

    unsigned char* base = nullptr;
    mrg_status s = scratch_address(c->device, &base);
    if(s != MRG_OK) return s;
    uint32_t* ctrl = reinterpret_cast<uint32_t*>(base);
    mrg_ray* dRays = reinterpret_cast<mrg_ray*>(base + kCtrlBytes);
    mrg_hit_keys* dHits = reinterpret_cast<mrg_hit_keys*>(base + kCtrlBytes + kMaxRays * kRayBytes);
    mrg_meta_hit* dMeta = reinterpret_cast<mrg_meta_hit*>(base + kCtrlBytes + kMaxRays * (kRayBytes + kHitBytes));

    cudaStream_t st = c->buildStream;
    cudaError_t e;
    // The array keeps the previous call's contents: clear the error flag
    // (the work counter is cleared by the launch).
    if((e = cudaMemsetAsync(ctrl + 1, 0, sizeof(uint32_t), st)) != cudaSuccess) return cuda_err(e, "clear flag");
    if((e = cudaMemcpyAsync(dRays, hRays, kRayBytes * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_err(e, "H2D rays");
    if((e = cudaMemcpyAsync(dHits, hHits, kHitBytes * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_err(e, "H2D hits");
    if((e = cudaMemcpyAsync(dMeta, hMeta, kMetaBytes * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_err(e, "H2D meta");
    mrg::TraceScratch scr;
    scr.workCounter = ctrl;
    scr.errorFlag = ctrl + 1;
    scr.stats = nullptr;
    if((e = mrg::launch_closest(c->scene, scr, dRays, nullptr, n, dHits, dMeta, c->smCount, st)) != cudaSuccess)
        return cuda_err(e, "launch");
    if((e = cudaMemcpyAsync(hRays, dRays, kRayBytes * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e, "D2H rays");
    if((e = cudaMemcpyAsync(hHits, dHits, kHitBytes * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e, "D2H hits");
    if((e = cudaMemcpyAsync(hMeta, dMeta, kMetaBytes * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e, "D2H meta");
    uint32_t flag = 0;
    if((e = cudaMemcpyAsync(&flag, ctrl + 1, sizeof(flag), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_err(e, "read flag");
    if((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_err(e, "synchronize");
    if(flag)
        return mrg::set_error(MRG_ERR_TRAVERSAL, "mrg_cast_closest_host_noalloc: traversal error flag " +
                              std::to_string(flag));
    return MRG_OK;
}
