// mrg_nrc.h -- radiance cache: multiresolution hash-grid encoding + fully
// fused MLP of 5 hidden 64-wide ReLU layers and a 16-wide output layer
// (BF16 tensor cores, FP32 accumulation),
// trained online with Adam.  No reference counterpart.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace mrg {

constexpr int kNrcWidth = 64;          // hidden width = input width
constexpr int kNrcOut = 16;            // output rows (RGB in the first 3)
constexpr int kNrcHidden = 5;          // hidden layers, each 64x64 with ReLU
constexpr int kNrcLayers = kNrcHidden + 1;   // + the 16x64 output layer
constexpr int kNrcHashFeatures = 32;   // levels * features per level
constexpr int kNrcInputFloats = 16;    // per sample: pos, rough | dir | normal | albedo
constexpr int kNrcWeightCount = kNrcHidden * kNrcWidth * kNrcWidth + kNrcOut * kNrcWidth;   // 21,504

struct NrcGrid
{
    uint32_t levels;          // 16
    uint32_t featuresPerLevel;// 2
    uint32_t log2Table;       // 19
    float    scale[32];       // per level: N_min * b^l - 1
    uint32_t res[32];         // per level: grid resolution (ceil(scale) + 1)
    uint32_t dense[32];       // 1: direct indexing (res^3 <= table size)
    float    aabbMin[3], aabbInv[3];
};

// Device state of one cache.
struct NrcState
{
    NrcGrid   grid;
    // parameters: MLP master weights (fp32) + bf16 copies, table master (fp32) + fp16 copy
    float*    w32;            // kNrcWeightCount: W0..W4 [64][64] row-major (out, in), W5 [16][64]
    uint16_t* w16;            // bf16 bits of w32
    float*    t32;            // levels * 2^log2Table * featuresPerLevel
    uint16_t* t16;            // fp16 bits of t32
    // Adam moments and gradients
    float*    mW;  float* vW;  float* gW;
    float*    mT;  float* vT;  float* gT;
    uint32_t  step;
    float     lr, beta1, beta2, eps;
    // training scratch (capacity samples)
    uint16_t* acts;           // [cap][6][64] bf16: x0, a1 .. a5
    uint16_t* g16;            // [cap][6][64] bf16: g_z1..g_z5, then dL/dy in columns 0..15 (16..63 stay 0)
    float4*   y;              // [cap] forward outputs of the training batch
    float*    loss;           // [1]
    float*    wgPart;         // [partCtas][kNrcWeightCount]: per-CTA weight-gradient partials
    uint32_t* err;            // sticky error word (a bounded wait that ran out sets kNrcWaitTimeout)
    uint32_t  cap;
    uint32_t  partCtas;
    // TMA descriptors of g16 and acts as 2D [cap rows][320 bf16], 64 x 128 boxes, 128-byte swizzle
    CUtensorMap tmG16;
    CUtensorMap tmActs;
};

constexpr uint32_t kNrcWaitTimeout = 8u;   // error bit, shared with the traversal error word

size_t nrc_table_entries(const NrcGrid& g);
void nrc_make_grid(NrcGrid& g, uint32_t levels, uint32_t log2Table, uint32_t baseRes, uint32_t maxRes,
                   const float aabb[6]);

// out: 4 floats per sample (RGB, 0).  Inputs as described for the C ABI.
cudaError_t nrc_query(const NrcState& S, const float4* inputs, const uint32_t* nDevice, uint32_t nMax,
                      float4* out, int smCount, cudaStream_t st);
// Query for a path tracer: samples are listed slots (list[k], k < *count) of
// an input array; writes out[slot].
cudaError_t nrc_query_list(const NrcState& S, const float4* inputs, const uint32_t* list, const uint32_t* count,
                           uint32_t nMax, float4* out, int smCount, cudaStream_t st);
// One optimisation step on n (input, target) samples; loss (mean relative
// L2) is written to S.loss.
cudaError_t nrc_train(NrcState& S, const float4* inputs, const float4* targets, const uint32_t* nDevice,
                      uint32_t nMax, int smCount, cudaStream_t st);
// Forward + backward + weight gradients only (accumulated into gW / gT).
cudaError_t nrc_gradients(NrcState& S, const float4* inputs, const float4* targets, const uint32_t* nDevice,
                          uint32_t nMax, int smCount, cudaStream_t st);
// bf16 / fp16 copies from the fp32 masters (after the host set them).
cudaError_t nrc_sync_copies(const NrcState& S, cudaStream_t st);
// Encodes S.tmG16 / S.tmActs for the allocated buffers (after g16 / acts / cap are set).
cudaError_t nrc_make_tensor_maps(NrcState& S);

} // namespace mrg
