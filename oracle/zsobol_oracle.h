/* zsobol_oracle.h -- TEST INFRASTRUCTURE ONLY: CPU restatement of MRay's
 * ZSobol and independent (PCG32) random-number groups (see zsobol_oracle.c
 * for the reference lines). */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* matrices: 3 x 52 uint32 (Sobol dims 0-2); perms: 24 x 4 bytes. */
void     orc_zs_tables(uint32_t* matrices, uint8_t* perms);
void     orc_mt19937(uint32_t seed, uint32_t count, uint32_t* out);
uint32_t orc_zs_res_max_bits(uint32_t width, uint32_t height);
/* Per-pixel seeds (row-major) of a width x height group. */
void     orc_zs_seeds(uint32_t width, uint32_t height, uint64_t seed, uint32_t* out);
/* The numbers of one sample of every pixel: request r (2 bits each of
 * `requests`, 1..3 numbers) reads dimension dimStart + (numbers before it);
 * out[pixel + width * height * k] = number k. */
int      orc_zs_generate(uint32_t width, uint32_t height, const uint32_t* seeds, uint32_t initialMaxSpp,
                         uint32_t sampleIndex, uint32_t dimStart, uint64_t requests, uint32_t requestCount,
                         uint32_t* out);

/* Component comp of the size-number request at dimension dim of one
 * pixel's sample (ZSobol::Next / Next2D / Next3D); owen != 0 reverses the
 * scrambled value's bits back (Laine-Karras Owen scrambling as published). */
uint32_t orc_zs_number(uint32_t px, uint32_t py, uint32_t seed, uint32_t sampleIndex, uint32_t initialMaxSpp,
                       uint32_t resMaxBits, uint32_t dim, uint32_t size, uint32_t comp, int owen);

/* MRay's independent sampler (PermutedCG32): the state GenerateState makes
 * of a per-pixel seed, and number n of that state's stream
 * (Permute(Step^n(state)), the jump by Brown's arbitrary-stride method). */
uint32_t orc_pcg32_state(uint32_t seed);
uint32_t orc_pcg32_advance(uint32_t state, uint32_t delta);
uint32_t orc_pcg32_permute(uint32_t state);
/* out[i] = number delta[i] of the stream seeded by seeds[i]. */
void     orc_pcg32_numbers(const uint32_t* seeds, const uint32_t* delta, uint32_t count, uint32_t* out);

#ifdef __cplusplus
}
#endif
