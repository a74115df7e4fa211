// partition_api.cpp -- C ABI of the ray partitioner (include/mray_gb300.h,
// "Ray partitioning"): argument checks, scratch, and the enqueue of
// mrg::multi_partition.
#include "mrg_ctx.h"

#include <cuda_runtime.h>

#include <string>

namespace mrg {

// Grows the context's partitioner scratch to hold `words` words.
mrg_status partition_scratch(mrg_ctx* c, size_t words)
{
    if(c->partScratchWords >= words && c->dPartScratch) return MRG_OK;
    cudaFree(c->dPartScratch);
    c->dPartScratch = nullptr;
    c->partScratchWords = 0;
    cudaError_t e = cudaMalloc(&c->dPartScratch, sizeof(uint32_t) * words);
    if(e != cudaSuccess)
    {
        cudaGetLastError();
        return set_error(e == cudaErrorMemoryAllocation ? MRG_ERR_OUT_OF_MEMORY : MRG_ERR_CUDA,
                         std::string("partition scratch: ") + cudaGetErrorString(e));
    }
    c->partScratchWords = words;
    return MRG_OK;
}

} // namespace mrg

extern "C" {

mrg_status mrg_multi_partition(mrg_ctx* c, const uint32_t* dKeys, const uint32_t* dIndices, uint32_t n,
                               const uint32_t dataBits[2], const uint32_t batchBits[2],
                               uint32_t onlyBatches, uint32_t* dSortedKeys, uint32_t* dSortedIdx,
                               uint32_t* dCount, uint32_t* dOffsets, uint32_t* dBinKeys,
                               uint32_t maxPartitions, void* stream)
{
    if(!c || !dataBits || !batchBits || !dCount || !dOffsets || !dBinKeys)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: null pointer");
    if(n > 0 && (!dKeys || !dSortedKeys || !dSortedIdx))
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: null pointer");
    if(n > (1u << 28)) return mrg::set_error(MRG_ERR_LIMIT, "mrg_multi_partition: more than 2^28 pairs");
    if(batchBits[0] >= batchBits[1] || batchBits[1] > 32)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: empty or out-of-range batch bit range");
    uint32_t dataShift = 0, dataWidth = 0;
    if(!onlyBatches)
    {
        if(dataBits[0] >= dataBits[1] || dataBits[1] > 32)
            return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: empty or out-of-range data bit range");
        if(dataBits[0] < batchBits[1] && batchBits[0] < dataBits[1])
            return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: data and batch bit ranges overlap");
        dataShift = dataBits[0];
        dataWidth = dataBits[1] - dataBits[0];
    }
    const uint32_t batchWidth = batchBits[1] - batchBits[0];
    if(batchWidth + dataWidth > 32)
        return mrg::set_error(MRG_ERR_INVALID_ARG, "mrg_multi_partition: more than 32 key bits");
    int prev = -1;
    cudaGetDevice(&prev);
    if(prev != c->device) cudaSetDevice(c->device);
    const size_t words = mrg::multi_partition_scratch_words(n);
    mrg_status s = mrg::partition_scratch(c, words);
    if(s == MRG_OK)
    {
        uint32_t* tmpKeys = c->dPartScratch;
        uint32_t* tmpIdx = tmpKeys + std::max<uint32_t>(n, 1u);
        uint32_t* hist = tmpIdx + std::max<uint32_t>(n, 1u);
        cudaError_t e = mrg::multi_partition(dKeys, dIndices, nullptr, n, dataShift, dataWidth, batchBits[0],
                                             batchWidth, dSortedKeys, dSortedIdx, tmpKeys, tmpIdx, hist, dCount,
                                             dOffsets, dBinKeys, maxPartitions, c->smCount,
                                             static_cast<cudaStream_t>(stream));
        if(e != cudaSuccess)
        {
            cudaGetLastError();
            s = mrg::set_error(MRG_ERR_CUDA, std::string("mrg_multi_partition: ") + cudaGetErrorString(e));
        }
    }
    if(prev >= 0 && prev != c->device) cudaSetDevice(prev);
    return s;
}

} // extern "C"
