// mrg_guide.h -- device data and host launch interface of the guided path
// tracer (MRay's GuidedPTRenderer: Markov-chain mixtures on a
// spatio-directional hash grid, Source/TracerDLL/GuidedPTRenderer.{h,cu},
// GuidedPTRendererShaders.h; Source/Tracer/HashGrid.h).
//
// One pass renders samplesPerPass samples per pixel bounce by bounce.  Per
// bounce, in MRay's kernel order:
//   closest-hit cast
//   backprop   KCBackpropagateHashGridPath: irradiance sample of the previous
//              vertex, chain update and lift, lock by atomicMin(slot + 1)
//   write MC   KCWriteMarkovChains: the lock winners write their chains
//   shade      WorkFunction / LightWorkFunction: mixture load (8 stochastic
//              codes, inserted), mixture / BSDF MIS sample, Russian roulette,
//              NEE with both pdfs; light hits and misses end the path
//   visibility cast, resolve   KCAccumulateShadowRaysGPT
//   apply      KCBackpropagateIrradNEE / KCBackpropagateIrradLight and the
//              backprop kernel's irradiance averages
// MRay updates irradiance with a compare-and-swap loop (MCIrradiance::
// AtomicEMA), so its order, and its result, vary run to run.  Here every
// update of a bounce becomes a record (cell, value) at a fixed position, and
// the records are stably sorted by (cell, phase): each cell takes its updates
// in MRay's kernel order (path backprop, NEE, light), slot by slot, with the
// path backprop reading the values from before the bounce.  That is one of the
// schedules MRay's kernels allow, and it is reproducible.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mrg_pt.h"

namespace mrg {

// PermutedCG32's LCG (Source/Tracer/Random.h:762-790), the slots' backup streams
constexpr uint32_t kBackupPcgMult = 747796405u, kBackupPcgInc = 2891336453u;

// HashGridView (HashGrid.h:66-115) plus the chain and irradiance state per
// table slot (GuidedPTRenderer.h: dMCStates, dMCCounts, dMCLocks, dMCIrradiances).
struct GuideGrid
{
    unsigned long long* codes;      // SpatioDirCode per slot, ~0 when empty
    uint32_t* counter;              // entries allocated
    uint32_t  tableMask;            // table size - 1 (a power of two)
    float3    cam;                  // camera position
    float3    rmin;                 // region (scene box) minimum
    float     baseDelta;            // baseRegionDelta
    uint32_t  baseDim;              // baseRegionDim
    float     normalDelta;
    uint32_t  normalDim;
    uint32_t  maxLevelOffset;
    uint32_t  maxEntryLimit;        // table size * 0.6
    float     tanConeHalfTimes2;
    float     lobeProb;             // lobeProbablity
    uint32_t  fixZeroWeight;        // 1: no mixture sample where the chosen lobe has weight 0
    float4*   mcA;                  // MCState target xyz, cosine
    float*    mcW;                  // MCState weight
    uint32_t* mcN;                  // MCCount
    uint32_t* lock;                 // MCLock (slot + 1 of the winner)
    float2*   irr;                  // MCIrradiance: value, count (bits)
};

// Per-slot guided path state (RayState of GuidedPTRDetail) and the bounce's
// irradiance records.
struct GuidePaths
{
    uint32_t* bk;                   // backup RNG state (PermutedCG32)
    uint32_t* lifted;               // dLiftedMCIndices
    float*    prevRefl;             // dPrevPathReflectanceOrOutRadiance
    float*    scoreSum;             // dScoreSums
    float2*   prevNormal;           // dPrevNormals (concentric octahedral)
    float*    shadowOut;            // dShadowPrevPathOutRadiance
    float4*   tmpA;                 // TransientMCState: target xyz, cosine
    float2*   tmpB;                 //                   weight, count (bits)
    uint32_t* recKey;               // 2 * slots: cell << 1 | light, ~0 = none
    float*    recVal;               // 2 * slots
    uint32_t* sortKeysA;            // radix-sort buffers, 2 * slots each
    uint32_t* sortIdxA;
    uint32_t* sortKeysB;
    uint32_t* sortIdxB;
    uint32_t* sortHist;
    uint2*    longRuns;             // runs of one cell longer than 32 records: (first position, cell)
    uint32_t* longCount;
    uint32_t  slots;
    uint32_t  keyBits;              // bits of a record key: log2(table) + 2
};

cudaError_t guide_backprop(const PtLaunch& L, const PtPaths& P, const GuideGrid& G, const GuidePaths& Q,
                           const PtSceneTables& T, const uint32_t* aliveList, const uint32_t* aliveCount,
                           int smCount, cudaStream_t st);
cudaError_t guide_write_mc(const PtPaths& P, const GuideGrid& G, const GuidePaths& Q, const PtSceneTables& T,
                           const uint32_t* aliveList, const uint32_t* aliveCount, int smCount, cudaStream_t st);
cudaError_t guide_shade(const PtLaunch& L, const PtPaths& P, const GuideGrid& G, const GuidePaths& Q,
                        const PtSceneTables& T, const uint32_t* aliveList, const uint32_t* aliveCount,
                        uint32_t* nextList, uint32_t* nextCount, int smCount, cudaStream_t st);
cudaError_t guide_resolve(const PtPaths& P, const GuidePaths& Q, int smCount, cudaStream_t st);
// Sorts the bounce's records by (cell, phase) and applies them to the
// irradiance averages; then marks every record empty for the next bounce.
cudaError_t guide_apply(const GuideGrid& G, const GuidePaths& Q, int smCount, cudaStream_t st);

} // namespace mrg
