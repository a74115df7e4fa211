// nrc_api.cpp -- C ABI of the radiance cache (include/mray_gb300.h, "Radiance
// cache"): allocation, seeded initialisation, query / train enqueue and
// parameter transfer.
#include "mrg_ctx.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace {

mrg_status nrc_cuda(cudaError_t e, const char* what)
{
    cudaGetLastError();
    return mrg::set_error(e == cudaErrorMemoryAllocation ? MRG_ERR_OUT_OF_MEMORY : MRG_ERR_CUDA,
                          std::string(what) + ": " + cudaGetErrorString(e));
}

template<class T>
cudaError_t alloc(mrg_ctx* c, T*& p, size_t count)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if(e == cudaSuccess)
    {
        c->cacheAllocs.push_back(q);
        e = cudaMemset(q, 0, sizeof(T) * (count ? count : 1));
    }
    p = static_cast<T*>(q);
    return e;
}

struct DevScope
{
    int prev = -1;
    explicit DevScope(int d) { if(cudaGetDevice(&prev) != cudaSuccess) prev = -1; if(prev != d) cudaSetDevice(d); }
    ~DevScope() { if(prev >= 0) cudaSetDevice(prev); }
};

// The cache kernels' bounded waits report through the context's error word.
mrg_status wait_flag(mrg_ctx* c, const char* what)
{
    uint32_t flag = 0;
    cudaError_t e = cudaMemcpy(&flag, c->cache.err, sizeof(flag), cudaMemcpyDeviceToHost);
    if(e != cudaSuccess) return nrc_cuda(e, what);
    if(flag & mrg::kNrcWaitTimeout)
    {
        const uint32_t rest = flag & ~mrg::kNrcWaitTimeout;
        e = cudaMemcpy(c->cache.err, &rest, sizeof(rest), cudaMemcpyHostToDevice);
        if(e != cudaSuccess) return nrc_cuda(e, what);
        return mrg::set_error(MRG_ERR_CUDA, std::string(what) + ": a tensor-core kernel's barrier wait ran out");
    }
    return MRG_OK;
}

} // namespace

extern "C" {

mrg_status mrg_cache_create(mrg_ctx* c, const mrg_cache_params* p)
{
    if(!c || !p) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_create: null pointer");
    if(p->levels == 0 || p->levels > 16 || p->log2_table_size < 8 || p->log2_table_size > 24 ||
       p->base_resolution < 2 || p->max_resolution < p->base_resolution || p->max_batch == 0 ||
       p->max_batch > (1u << 20) || !(p->learning_rate > 0.0f))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_create: parameters out of range");
    DevScope g(c->device);
    for(void* q : c->cacheAllocs) cudaFree(q);
    c->cacheAllocs.clear();
    c->cacheOn = false;
    mrg::NrcState& S = c->cache;
    S = mrg::NrcState{};
    mrg::nrc_make_grid(S.grid, p->levels, p->log2_table_size, p->base_resolution, p->max_resolution, p->aabb);
    const size_t nt = mrg::nrc_table_entries(S.grid) * 2;
    const size_t nw = mrg::kNrcWeightCount;
    S.cap = p->max_batch;
    cudaError_t e = cudaSuccess;
    if(e == cudaSuccess) e = alloc(c, S.w32, nw);
    if(e == cudaSuccess) e = alloc(c, S.w16, nw);
    if(e == cudaSuccess) e = alloc(c, S.mW, nw);
    if(e == cudaSuccess) e = alloc(c, S.vW, nw);
    if(e == cudaSuccess) e = alloc(c, S.gW, nw);
    if(e == cudaSuccess) e = alloc(c, S.t32, nt);
    if(e == cudaSuccess) e = alloc(c, S.t16, nt);
    if(e == cudaSuccess) e = alloc(c, S.mT, nt);
    if(e == cudaSuccess) e = alloc(c, S.vT, nt);
    if(e == cudaSuccess) e = alloc(c, S.gT, nt);
    if(e == cudaSuccess) e = alloc(c, S.acts, (size_t)S.cap * mrg::kNrcLayers * mrg::kNrcWidth);
    if(e == cudaSuccess) e = alloc(c, S.g16, (size_t)S.cap * mrg::kNrcLayers * mrg::kNrcWidth);
    if(e == cudaSuccess) e = alloc(c, S.y, (size_t)S.cap);
    if(e == cudaSuccess) e = alloc(c, S.loss, 1);
    S.partCtas = (uint32_t)std::max(1, c->smCount);
    if(e == cudaSuccess) e = alloc(c, S.wgPart, (size_t)S.partCtas * mrg::kNrcWeightCount);
    // the gradient rows' unused columns (output slot, 16..63) must read as zero
    if(e == cudaSuccess) e = cudaMemset(S.g16, 0, sizeof(uint16_t) * (size_t)S.cap * mrg::kNrcLayers * mrg::kNrcWidth);
    if(e == cudaSuccess) e = cudaMemset(S.acts, 0, sizeof(uint16_t) * (size_t)S.cap * mrg::kNrcLayers * mrg::kNrcWidth);
    if(e == cudaSuccess) e = mrg::nrc_make_tensor_maps(S);
    if(e != cudaSuccess) return nrc_cuda(e, "mrg_cache_create");
    S.err = c->dScratch + 1;
    S.lr = p->learning_rate;
    S.beta1 = p->beta1; S.beta2 = p->beta2; S.eps = p->epsilon;
    S.step = 0;
    // Xavier-uniform MLP weights; hash features uniform in [-1e-4, 1e-4]
    std::mt19937 rng(p->seed);
    std::vector<float> w(nw);
    const float lim = std::sqrt(6.0f / (64.0f + 64.0f)), limOut = std::sqrt(6.0f / (64.0f + 16.0f));
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    const size_t hiddenWeights = (size_t)mrg::kNrcHidden * mrg::kNrcWidth * mrg::kNrcWidth;
    for(size_t i = 0; i < nw; i++) w[i] = U(rng) * (i < hiddenWeights ? lim : limOut);
    std::vector<float> t(nt);
    for(size_t i = 0; i < nt; i++) t[i] = U(rng) * 1e-4f;
    e = cudaMemcpy(S.w32, w.data(), sizeof(float) * nw, cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemcpy(S.t32, t.data(), sizeof(float) * nt, cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = mrg::nrc_sync_copies(S, nullptr);
    if(e == cudaSuccess) e = cudaDeviceSynchronize();
    if(e != cudaSuccess) return nrc_cuda(e, "mrg_cache_create: initialisation");
    c->cacheOn = true;
    return MRG_OK;
}

mrg_status mrg_cache_query(mrg_ctx* c, const float* dIn, uint32_t n, float* dOut, void* stream)
{
    if(!c || (n && (!dIn || !dOut))) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_query: null pointer");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cache_query: call mrg_cache_create first");
    if(n == 0) return MRG_OK;
    DevScope g(c->device);
    cudaError_t e = mrg::nrc_query(c->cache, reinterpret_cast<const float4*>(dIn), nullptr, n,
                                   reinterpret_cast<float4*>(dOut), c->smCount, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? MRG_OK : nrc_cuda(e, "mrg_cache_query");
}

mrg_status mrg_cache_train(mrg_ctx* c, const float* dIn, const float* dTarget, uint32_t n, float* hLoss, void* stream)
{
    if(!c || (n && (!dIn || !dTarget))) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_train: null pointer");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cache_train: call mrg_cache_create first");
    if(n > c->cache.cap) return mrg::set_error(MRG_ERR_LIMIT, "mrg_cache_train: more samples than max_batch");
    if(n == 0) { if(hLoss) *hLoss = 0.0f; return MRG_OK; }
    DevScope g(c->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = mrg::nrc_train(c->cache, reinterpret_cast<const float4*>(dIn),
                                   reinterpret_cast<const float4*>(dTarget), nullptr, n, c->smCount, st);
    if(e == cudaSuccess && hLoss)
    {
        e = cudaMemcpyAsync(hLoss, c->cache.loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        if(e == cudaSuccess) e = cudaStreamSynchronize(st);
        if(e == cudaSuccess) return wait_flag(c, "mrg_cache_train");
    }
    return e == cudaSuccess ? MRG_OK : nrc_cuda(e, "mrg_cache_train");
}

mrg_status mrg_cache_gradients(mrg_ctx* c, const float* dIn, const float* dTarget, uint32_t n, float* hGW,
                               float* hGT, float* hLoss)
{
    if(!c || !dIn || !dTarget) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_gradients: null pointer");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cache_gradients: no cache");
    if(n == 0 || n > c->cache.cap) return mrg::set_error(MRG_ERR_LIMIT, "mrg_cache_gradients: batch size");
    DevScope g(c->device);
    mrg::NrcState& S = c->cache;
    const size_t nt = mrg::nrc_table_entries(S.grid) * 2;
    cudaError_t e = mrg::nrc_gradients(S, reinterpret_cast<const float4*>(dIn), reinterpret_cast<const float4*>(dTarget),
                                       nullptr, n, c->smCount, nullptr);
    if(e == cudaSuccess) e = cudaDeviceSynchronize();
    if(e == cudaSuccess && hGW) e = cudaMemcpy(hGW, S.gW, sizeof(float) * mrg::kNrcWeightCount, cudaMemcpyDeviceToHost);
    if(e == cudaSuccess && hGT) e = cudaMemcpy(hGT, S.gT, sizeof(float) * nt, cudaMemcpyDeviceToHost);
    if(e == cudaSuccess && hLoss) e = cudaMemcpy(hLoss, S.loss, sizeof(float), cudaMemcpyDeviceToHost);
    if(e == cudaSuccess) e = cudaMemset(S.gW, 0, sizeof(float) * mrg::kNrcWeightCount);
    if(e == cudaSuccess) e = cudaMemset(S.gT, 0, sizeof(float) * nt);
    return e == cudaSuccess ? wait_flag(c, "mrg_cache_gradients") : nrc_cuda(e, "mrg_cache_gradients");
}

mrg_status mrg_cache_get_params(mrg_ctx* c, float* hW, float* hT)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_get_params: null context");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cache_get_params: no cache");
    DevScope g(c->device);
    cudaError_t e = cudaDeviceSynchronize();
    if(e == cudaSuccess && hW) e = cudaMemcpy(hW, c->cache.w32, sizeof(float) * mrg::kNrcWeightCount, cudaMemcpyDeviceToHost);
    if(e == cudaSuccess && hT)
        e = cudaMemcpy(hT, c->cache.t32, sizeof(float) * mrg::nrc_table_entries(c->cache.grid) * 2, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? MRG_OK : nrc_cuda(e, "mrg_cache_get_params");
}

mrg_status mrg_cache_set_params(mrg_ctx* c, const float* hW, const float* hT)
{
    if(!c) return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_cache_set_params: null context");
    if(!c->cacheOn) return mrg::set_error(MRG_ERR_NOT_BUILT, "mrg_cache_set_params: no cache");
    DevScope g(c->device);
    cudaError_t e = cudaDeviceSynchronize();
    if(e == cudaSuccess && hW) e = cudaMemcpy(c->cache.w32, hW, sizeof(float) * mrg::kNrcWeightCount, cudaMemcpyHostToDevice);
    if(e == cudaSuccess && hT)
        e = cudaMemcpy(c->cache.t32, hT, sizeof(float) * mrg::nrc_table_entries(c->cache.grid) * 2, cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = mrg::nrc_sync_copies(c->cache, nullptr);
    if(e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? MRG_OK : nrc_cuda(e, "mrg_cache_set_params");
}

} // extern "C"
