// partition.cu -- stable multi-split radix sort of (key, index) pairs and the
// partition (split) search of MRay's RayPartitioner::MultiPartition
// (Source/Tracer/RayPartitioner.cu:263-411, split kernels :19-75).
//
// MRay sorts with CUB's radix sort and finds the splits with a binary
// partition, waiting on the host in between.  Here one radix digit (up to 8
// bits, 256 buckets) is one pass of three kernels:
//   hist     per-tile bucket counts (shared-memory, warp-aggregated atomics)
//   scan     exclusive scan of the bucket-major (bucket, tile) count table
//   scatter  stable ranks inside each tile (warp match + per-warp counts in
//            shared memory), written to the bucket's global offset
// The element count may live in device memory (a path tracer's alive count),
// so a pass is enqueued without knowing it; the grid is sized for an upper
// bound and tiles past the count contribute nothing.
#include "mrg_partition.h"

namespace mrg {

namespace {

constexpr int kMsTPB = 256;
constexpr int kMsItems = 8;
constexpr int kMsTile = kMsTPB * kMsItems;     // 2048 elements per tile
constexpr int kMsWarps = kMsTPB / 32;
constexpr int kScanTPB = 1024;

__device__ __forceinline__ uint32_t bits_of(uint32_t v, uint32_t shift, uint32_t width)
{
    return (width >= 32u) ? (v >> shift) : ((v >> shift) & ((1u << width) - 1u));
}

// Composite sort key: batch bits above data bits (or batch bits alone).
__device__ __forceinline__ uint32_t digit_of(const DigitSpec& s, uint32_t key)
{
    uint32_t c = bits_of(key, s.batchShift, s.batchWidth);
    if(s.dataWidth) c = (c << s.dataWidth) | bits_of(key, s.dataShift, s.dataWidth);
    return bits_of(c, s.digitShift, s.digitBits);
}

__device__ __forceinline__ uint32_t count_of(const uint32_t* nDevice, uint32_t nHost)
{
    return nDevice ? *nDevice : nHost;
}

__global__ void __launch_bounds__(kMsTPB)
k_ms_hist(const uint32_t* __restrict__ keys, const uint32_t* nDevice, uint32_t nHost, DigitSpec spec,
          uint32_t* __restrict__ hist, uint32_t numTiles)
{
    __shared__ uint32_t sHist[256];
    const uint32_t nb = 1u << spec.digitBits;
    for(uint32_t b = threadIdx.x; b < nb; b += kMsTPB) sHist[b] = 0u;
    __syncthreads();
    const uint32_t n = count_of(nDevice, nHost);
    const uint32_t tileStart = blockIdx.x * (uint32_t)kMsTile;
    for(int r = 0; r < kMsItems; r++)
    {
        const uint32_t e = tileStart + (uint32_t)r * kMsTPB + threadIdx.x;
        const bool valid = e < n;
        const uint32_t d = valid ? digit_of(spec, __ldg(&keys[e])) : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t lane = threadIdx.x & 31u;
        if(valid && (__ffs(peers) - 1) == (int)lane) atomicAdd(&sHist[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for(uint32_t b = threadIdx.x; b < nb; b += kMsTPB) hist[(size_t)b * numTiles + blockIdx.x] = sHist[b];
}

// Exclusive scan of len counts in place; one block (len <= 256 * 2^16).
__global__ void __launch_bounds__(kScanTPB)
k_ms_scan(uint32_t* __restrict__ hist, uint32_t len)
{
    __shared__ uint32_t sPart[kScanTPB];
    const uint32_t per = (len + kScanTPB - 1) / kScanTPB;
    const uint32_t beg = min(len, threadIdx.x * per), end = min(len, beg + per);
    uint32_t sum = 0;
    for(uint32_t i = beg; i < end; i++) sum += hist[i];
    sPart[threadIdx.x] = sum;
    __syncthreads();
    // Hillis-Steele inclusive scan of the per-thread sums
    for(uint32_t off = 1; off < kScanTPB; off <<= 1)
    {
        const uint32_t v = (threadIdx.x >= off) ? sPart[threadIdx.x - off] : 0u;
        __syncthreads();
        sPart[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = sPart[threadIdx.x] - sum;
    for(uint32_t i = beg; i < end; i++)
    {
        const uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// Large count tables: a three-kernel scan (per-block sums, one-block scan of
// the sums, per-block exclusive scan plus its offset), kScanChunk entries per
// block, 4 per thread.
constexpr uint32_t kScanChunk = 4u * kScanTPB;
constexpr uint32_t kSingleBlockScan = 65536u;   // at most this many entries: k_ms_scan

// Exclusive scan of v across the block; the block's total in *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t sWarp[kScanTPB / 32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if(lane >= (uint32_t)o) x += y;
    }
    if(lane == 31u) sWarp[warp] = x;
    __syncthreads();
    if(warp == 0)
    {
        uint32_t w = (lane < kScanTPB / 32) ? sWarp[lane] : 0u;
#pragma unroll
        for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if(lane >= (uint32_t)o) w += y;
        }
        if(lane < kScanTPB / 32) sWarp[lane] = w;
    }
    __syncthreads();
    const uint32_t before = (warp ? sWarp[warp - 1] : 0u) + x - v;
    if(total) *total = sWarp[kScanTPB / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kScanTPB)
k_scan_sums(const uint32_t* __restrict__ hist, uint32_t len, uint32_t* __restrict__ sums)
{
    const uint32_t base = blockIdx.x * kScanChunk + 4u * threadIdx.x;
    uint32_t v = 0;
#pragma unroll
    for(uint32_t k = 0; k < 4u; k++) v += (base + k < len) ? hist[base + k] : 0u;
    uint32_t total;
    block_exclusive(v, &total);
    if(threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanTPB)
k_scan_top(uint32_t* __restrict__ sums, uint32_t n)
{
    uint32_t carry = 0;
    for(uint32_t b = 0; b < n; b += kScanTPB)
    {
        const uint32_t i = b + threadIdx.x;
        const uint32_t v = (i < n) ? sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive(v, &total);
        if(i < n) sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanTPB)
k_scan_apply(uint32_t* __restrict__ hist, uint32_t len, const uint32_t* __restrict__ sums)
{
    const uint32_t base = blockIdx.x * kScanChunk + 4u * threadIdx.x;
    uint32_t a[4];
#pragma unroll
    for(uint32_t k = 0; k < 4u; k++) a[k] = (base + k < len) ? hist[base + k] : 0u;
    uint32_t run = sums[blockIdx.x] + block_exclusive(a[0] + a[1] + a[2] + a[3], nullptr);
#pragma unroll
    for(uint32_t k = 0; k < 4u; k++)
        if(base + k < len) { hist[base + k] = run; run += a[k]; }
}

__global__ void __launch_bounds__(kMsTPB)
k_ms_scatter(const uint32_t* __restrict__ keysIn, const uint32_t* __restrict__ idxIn,
             uint32_t* __restrict__ keysOut, uint32_t* __restrict__ idxOut,
             const uint32_t* nDevice, uint32_t nHost, DigitSpec spec,
             const uint32_t* __restrict__ hist, uint32_t numTiles)
{
    __shared__ uint32_t sBase[256];
    __shared__ uint32_t sWarp[kMsWarps][256];
    const uint32_t nb = 1u << spec.digitBits;
    const uint32_t n = count_of(nDevice, nHost);
    const uint32_t tileStart = blockIdx.x * (uint32_t)kMsTile;
    if(tileStart >= n) return;                              // block-uniform
    for(uint32_t b = threadIdx.x; b < nb; b += kMsTPB) sBase[b] = hist[(size_t)b * numTiles + blockIdx.x];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t lowerMask = (1u << lane) - 1u;
    for(int r = 0; r < kMsItems; r++)
    {
        for(uint32_t i = threadIdx.x; i < (uint32_t)kMsWarps * nb; i += kMsTPB) sWarp[i / nb][i % nb] = 0u;
        __syncthreads();
        const uint32_t e = tileStart + (uint32_t)r * kMsTPB + threadIdx.x;
        const bool valid = e < n;
        uint32_t key = 0, idx = 0, d = 0xFFFFFFFFu;
        if(valid)
        {
            key = keysIn[e];
            idx = idxIn ? idxIn[e] : e;
            d = digit_of(spec, key);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = (uint32_t)__popc(peers & lowerMask);
        if(valid && rank == 0u) sWarp[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        if(valid)
        {
            uint32_t pos = sBase[d] + rank;
            for(uint32_t w = 0; w < warp; w++) pos += sWarp[w][d];
            keysOut[pos] = key;
            idxOut[pos] = idx;
        }
        __syncthreads();
        for(uint32_t b = threadIdx.x; b < nb; b += kMsTPB)
        {
            uint32_t t = 0;
            for(int w = 0; w < kMsWarps; w++) t += sWarp[w][b];
            sBase[b] += t;
        }
        __syncthreads();
    }
}

// KCFindSplits: mark 1 where the batch portion changes (and at 0).
__global__ void k_find_splits(const uint32_t* __restrict__ sortedKeys, const uint32_t* nDevice, uint32_t nHost,
                              uint32_t batchShift, uint32_t batchWidth, uint32_t* __restrict__ marks)
{
    const uint32_t n = count_of(nDevice, nHost);
    for(uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    {
        const uint32_t k = bits_of(sortedKeys[j], batchShift, batchWidth);
        marks[j] = (j == 0u) ? 1u : (k != bits_of(sortedKeys[j - 1], batchShift, batchWidth) ? 1u : 0u);
    }
}

// KCFindBinMatIds: partition start offsets and keys from the compacted split
// positions (bucket 1 of a one-bit multi-split of the marks).
__global__ void k_bins(const uint32_t* __restrict__ splitPos, const uint32_t* __restrict__ sortedKeys,
                       const uint32_t* nDevice, uint32_t nHost, const uint32_t* __restrict__ scannedHist,
                       uint32_t numTiles, uint32_t maxPartitions,
                       uint32_t* __restrict__ count, uint32_t* __restrict__ offsets, uint32_t* __restrict__ binKeys)
{
    const uint32_t n = count_of(nDevice, nHost);
    // bucket 1 starts after every zero mark
    const uint32_t ones = (n == 0u) ? 0u : n - scannedHist[(size_t)1 * numTiles];
    const uint32_t first = n - ones;
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ones && i < maxPartitions;
        i += gridDim.x * blockDim.x)
    {
        const uint32_t p = splitPos[first + i];
        offsets[i] = p;
        binKeys[i] = sortedKeys[p];
    }
    if(blockIdx.x == 0 && threadIdx.x == 0)
    {
        *count = ones;
        if(ones <= maxPartitions) offsets[ones] = n;
    }
}

} // namespace

namespace {

// Coherence key of a ray: direction octant above a 27-bit Morton code of the
// origin quantised (9 bits per axis) in the scene box.
__global__ void k_ray_keys(const float4* __restrict__ rays, const uint32_t* __restrict__ idx, uint32_t n,
                           float3 lo, float3 scale, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    for(uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t r = idx ? idx[i] : i;
        const float4 o = __ldg(rays + 2 * (size_t)r), d = __ldg(rays + 2 * (size_t)r + 1);
        auto q = [](float v, float l, float s) {
            const float t = fminf(fmaxf((v - l) * s, 0.0f), 511.0f);
            uint32_t x = (uint32_t)t;
            x = (x | (x << 16)) & 0x030000FFu;
            x = (x | (x << 8)) & 0x0300F00Fu;
            x = (x | (x << 4)) & 0x030C30C3u;
            x = (x | (x << 2)) & 0x09249249u;
            return x;
        };
        const uint32_t m = q(o.x, lo.x, scale.x) | (q(o.y, lo.y, scale.y) << 1) | (q(o.z, lo.z, scale.z) << 2);
        const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
        keys[i] = (oct << 27) | m;
        vals[i] = r;
    }
}

} // namespace

cudaError_t ray_coherence_order(const void* rays, const uint32_t* idx, uint32_t n, const float box[6],
                                uint32_t* keysA, uint32_t* valsA, uint32_t* keysB, uint32_t* valsB,
                                uint32_t* hist, uint32_t*& order, int smCount, cudaStream_t st)
{
    float3 lo = make_float3(box[0], box[1], box[2]), sc;
    const float ext[3] = { box[3] - box[0], box[4] - box[1], box[5] - box[2] };
    sc.x = ext[0] > 0.0f ? 511.0f / ext[0] : 0.0f;
    sc.y = ext[1] > 0.0f ? 511.0f / ext[1] : 0.0f;
    sc.z = ext[2] > 0.0f ? 511.0f / ext[2] : 0.0f;
    k_ray_keys<<<std::max(1, smCount * 8), 256, 0, st>>>(static_cast<const float4*>(rays), idx, n, lo, sc, keysA, valsA);
    cudaError_t e = cudaGetLastError();
    uint32_t* kin = keysA; uint32_t* vin = valsA;
    uint32_t* kout = keysB; uint32_t* vout = valsB;
    for(uint32_t p = 0; p < 4 && e == cudaSuccess; p++)
    {
        DigitSpec s;
        s.batchShift = 0; s.batchWidth = 30;
        s.digitShift = 8u * p; s.digitBits = (p == 3) ? 6u : 8u;
        e = multisplit_pass(kin, vin, kout, vout, nullptr, n, s, hist, st);
        std::swap(kin, kout); std::swap(vin, vout);
    }
    order = vin;
    return e;
}

size_t multisplit_hist_words(uint32_t nMax, uint32_t digitBits)
{
    const uint32_t tiles = (nMax + kMsTile - 1) / kMsTile;
    const size_t len = (size_t)(tiles ? tiles : 1u) << digitBits;
    // the count table, then the block sums of its scan
    return len + (len + kScanChunk - 1) / kScanChunk;
}

cudaError_t multisplit_pass(const uint32_t* keysIn, const uint32_t* idxIn, uint32_t* keysOut, uint32_t* idxOut,
                            const uint32_t* nDevice, uint32_t nMax, const DigitSpec& spec, uint32_t* hist,
                            cudaStream_t st)
{
    if(spec.digitBits == 0 || spec.digitBits > 8) return cudaErrorInvalidValue;
    uint32_t tiles = (nMax + kMsTile - 1) / kMsTile;
    if(tiles == 0) tiles = 1;
    const uint32_t len = tiles << spec.digitBits;
    k_ms_hist<<<tiles, kMsTPB, 0, st>>>(keysIn, nDevice, nMax, spec, hist, tiles);
    if(len <= kSingleBlockScan) k_ms_scan<<<1, kScanTPB, 0, st>>>(hist, len);
    else
    {
        const uint32_t blocks = (len + kScanChunk - 1) / kScanChunk;
        uint32_t* sums = hist + len;
        k_scan_sums<<<blocks, kScanTPB, 0, st>>>(hist, len, sums);
        k_scan_top<<<1, kScanTPB, 0, st>>>(sums, blocks);
        k_scan_apply<<<blocks, kScanTPB, 0, st>>>(hist, len, sums);
    }
    k_ms_scatter<<<tiles, kMsTPB, 0, st>>>(keysIn, idxIn, keysOut, idxOut, nDevice, nMax, spec, hist, tiles);
    return cudaGetLastError();
}

cudaError_t multi_partition(const uint32_t* keys, const uint32_t* indices, const uint32_t* nDevice, uint32_t nMax,
                            uint32_t dataShift, uint32_t dataWidth, uint32_t batchShift, uint32_t batchWidth,
                            uint32_t* sortedKeys, uint32_t* sortedIdx, uint32_t* tmpKeys, uint32_t* tmpIdx,
                            uint32_t* hist, uint32_t* count, uint32_t* offsets, uint32_t* binKeys,
                            uint32_t maxPartitions, int smCount, cudaStream_t st)
{
    const uint32_t total = batchWidth + dataWidth;
    const uint32_t passes = (total + 7u) / 8u;
    // ping-pong so that the last pass lands in the outputs
    const uint32_t* kIn = keys;
    const uint32_t* iIn = indices;
    for(uint32_t p = 0; p < passes; p++)
    {
        const bool toOut = ((passes - 1u - p) & 1u) == 0u;
        uint32_t* kOut = toOut ? sortedKeys : tmpKeys;
        uint32_t* iOut = toOut ? sortedIdx : tmpIdx;
        DigitSpec s;
        s.batchShift = batchShift; s.batchWidth = batchWidth;
        s.dataShift = dataShift; s.dataWidth = dataWidth;
        s.digitShift = 8u * p;
        s.digitBits = std::min(8u, total - 8u * p);
        cudaError_t e = multisplit_pass(kIn, iIn, kOut, iOut, nDevice, nMax, s, hist, st);
        if(e != cudaSuccess) return e;
        kIn = kOut; iIn = iOut;
    }
    // splits of the batch portion, compacted in order with a one-bit pass
    k_find_splits<<<std::max(1, smCount * 4), 256, 0, st>>>(sortedKeys, nDevice, nMax, batchShift, batchWidth, tmpKeys);
    DigitSpec m;
    m.batchShift = 0; m.batchWidth = 1; m.dataShift = 0; m.dataWidth = 0;
    m.digitShift = 0; m.digitBits = 1;
    uint32_t* marksOut = hist + multisplit_hist_words(nMax, 8);      // past the widest count table
    cudaError_t e = multisplit_pass(tmpKeys, nullptr, marksOut, tmpIdx, nDevice, nMax, m, hist, st);
    if(e != cudaSuccess) return e;
    uint32_t tiles = (nMax + kMsTile - 1) / kMsTile;
    if(tiles == 0) tiles = 1;
    k_bins<<<std::max(1, smCount), 256, 0, st>>>(tmpIdx, sortedKeys, nDevice, nMax, hist, tiles, maxPartitions,
                                                 count, offsets, binKeys);
    return cudaGetLastError();
}

} // namespace mrg
