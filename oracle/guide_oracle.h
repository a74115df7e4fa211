/* guide_oracle.h -- TEST INFRASTRUCTURE ONLY: CPU restatement of the
 * building blocks of MRay's guided path tracer (Markov-chain mixtures on a
 * spatio-directional hash grid; see guide_oracle.c for the reference lines).
 * Never linked into the product. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_GUIDE_EMPTY   0xFFFFFFFFFFFFFFFFull
#define ORC_GUIDE_INVALID 0xFFFFFFFFu
#define ORC_GUIDE_LOBES   8u

/* HashGridView (Source/Tracer/HashGrid.h:66-115) */
typedef struct orc_guide_grid
{
    uint64_t* codes;             /* table (power of two), ORC_GUIDE_EMPTY when free */
    uint32_t  tableSize;
    uint32_t  counter;           /* entries allocated */
    float     cam[3];
    float     rmin[3];           /* hash-grid region min (the region max is not read) */
    float     baseDelta;         /* baseRegionDelta */
    uint32_t  baseDim;           /* baseRegionDim */
    float     normalDelta;
    uint32_t  normalDim;
    uint32_t  maxLevelOffset;
    uint32_t  maxEntryLimit;
    float     tanConeHalfTimes2;
} orc_guide_grid;

/* GaussianLobe (Source/Tracer/DistributionFunctions.h:75-99, 230-380) */
typedef struct orc_lobe { float dir[3]; float kappa, alpha; } orc_lobe;
/* MCState (TracerDLL/GuidedPTRendererShaders.h:22-38) */
typedef struct orc_mc_state { float target[3]; float cosine, weight; } orc_mc_state;

/* PermutedCG32 as the backup RNG: ToFloat01(Next()). */
float    orc_guide_next_float(uint32_t* state);

/* HashGrid::View numbers from the grid's settings (HashGrid.h:410-440). */
void     orc_guide_view(orc_guide_grid* g, const float aabb[6], const float cam[3], uint32_t posBits,
                        uint32_t normalBits, uint32_t maxLevelOffset, float coneApertureDeg, uint32_t tableSize);
uint64_t orc_guide_gen_code(const orc_guide_grid* g, const float pos[3], const float normal[3]);
uint64_t orc_guide_gen_code_stochastic(const orc_guide_grid* g, const float pos[3], const float normal[3],
                                       uint32_t* rng);
uint32_t orc_guide_search(const orc_guide_grid* g, uint64_t code);       /* ORC_GUIDE_INVALID if absent */
uint32_t orc_guide_try_insert(orc_guide_grid* g, uint64_t code, int* inserted);

void     orc_dir_to_conc_octa(const float d[3], float st[2]);
void     orc_conc_octa_to_dir(const float st[2], float d[3]);

orc_lobe orc_lobe_make(const float dir[3], float kappa);
float    orc_lobe_pdf(const orc_lobe* l, const float w[3]);
void     orc_lobe_sample(const orc_lobe* l, float xi0, float xi1, float out[3]);
float    orc_x_over_exp1m(float x);

void     orc_mc_target(const orc_mc_state* s, float out[3]);
void     orc_mc_direction(const orc_mc_state* s, const float pos[3], float out[3]);
float    orc_mc_mean_cosine(const orc_mc_state* s, const float pos[3], uint32_t n);
uint32_t orc_mc_ema(orc_mc_state* s, const float pos[3], const float newTarget[3], float newWeight, uint32_t n);
orc_lobe orc_mc_to_lobe(const orc_mc_state* s, uint32_t n, const float pos[3]);
/* MCIrradiance::AtomicEMA's update (GuidedPTRendererShaders.h:330-345) */
void     orc_irr_ema(float* irrad, uint32_t* n, float radEst);

/* batch forms (fixture tests) */
void     orc_guide_lobe_batch(const float* in7, const float* w3, float* out8, uint32_t n);
void     orc_conc_octa_batch(const float* dir3, float* st2, const float* stIn, float* dirOut, uint32_t n);
void     orc_guide_codes_batch(const float* view15, const float* in6, uint32_t* rng, uint64_t* out2, uint32_t n);
void     orc_guide_table_batch(const uint64_t* codes, uint32_t n, const uint64_t* probe, uint32_t m, uint32_t size,
                               uint32_t* slots, uint32_t* found);

#ifdef __cplusplus
}
#endif
