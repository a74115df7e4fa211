// mrg_partition.h -- stable multi-split radix passes and MultiPartition.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace mrg {

// One radix digit of the composite key
//   c = bits(key, batch) << dataWidth | bits(key, data)   (dataWidth may be 0)
// digit = bits(c, digitShift, digitBits), digitBits in [1, 8].
struct DigitSpec
{
    uint32_t batchShift = 0, batchWidth = 0;
    uint32_t dataShift = 0, dataWidth = 0;
    uint32_t digitShift = 0, digitBits = 0;
};

// Words of the (bucket, tile) count table of one pass.
size_t multisplit_hist_words(uint32_t nMax, uint32_t digitBits);

// Words of scratch multi_partition needs for up to nMax elements.
inline size_t multi_partition_scratch_words(uint32_t nMax)
{
    return 3ull * std::max<uint32_t>(nMax, 1u) + multisplit_hist_words(nMax, 8);
}

// Stable scatter of (key, index) pairs by one digit.  idxIn == nullptr means
// the element's position.  The count is *nDevice when given, else nMax.
cudaError_t multisplit_pass(const uint32_t* keysIn, const uint32_t* idxIn, uint32_t* keysOut, uint32_t* idxOut,
                            const uint32_t* nDevice, uint32_t nMax, const DigitSpec& spec, uint32_t* hist,
                            cudaStream_t st);

// RayPartitioner::MultiPartition: stable sort by (batch, data) bits, then the
// start offset and key of every run of equal batch bits.  scratch holds
// multi_partition_scratch_words(nMax) words.
cudaError_t multi_partition(const uint32_t* keys, const uint32_t* indices, const uint32_t* nDevice, uint32_t nMax,
                            uint32_t dataShift, uint32_t dataWidth, uint32_t batchShift, uint32_t batchWidth,
                            uint32_t* sortedKeys, uint32_t* sortedIdx, uint32_t* tmpKeys, uint32_t* tmpIdx,
                            uint32_t* hist, uint32_t* count, uint32_t* offsets, uint32_t* binKeys,
                            uint32_t maxPartitions, int smCount, cudaStream_t st);

// Index order that groups rays by direction octant, then by origin (Morton
// code in `box`): a coherence sort before a cast.  Scratch: 4 arrays of n
// words and a count table of multisplit_hist_words(n, 8); `order` points at
// the sorted indices (one of the scratch arrays).
cudaError_t ray_coherence_order(const void* rays, const uint32_t* idx, uint32_t n, const float box[6],
                                uint32_t* keysA, uint32_t* valsA, uint32_t* keysB, uint32_t* valsB,
                                uint32_t* hist, uint32_t*& order, int smCount, cudaStream_t st);

} // namespace mrg
