/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Counter-based random stream used by the
 * CPU oracle (kk_oracle.c) and by the RNG hook that feeds the reference's own
 * sampler (ref/kk_ref_driver.cpp).  The product has its own device copy of the
 * same definitions; this file is the checker's copy and is never linked into
 * the product.
 *
 * Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel
 * Random Numbers: As Easy as 1, 2, 3" (SC'11): a 10-round substitution-
 * permutation network over a 128-bit counter with a 64-bit key, using the
 * paper's multipliers 0xD2511F53 / 0xCD9E8D57 and Weyl key increments
 * 0x9E3779B9 / 0xBB67AE85.
 *
 * Stream layout (the project's definition, shared with the device):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (walker_id, step, draw_idx >> 2, stream)
 *   word    = output[draw_idx & 3]
 * draw_idx counts the draws a walker makes within one step, in program order,
 * across all rejection trials of that step.  stream 0 = walk, 1 = walker
 * init state, 2 = walker start vertex.
 *
 * Sampling mappings (replacing std::uniform_int_distribution /
 * std::uniform_real_distribution of include/util.hpp:60-69):
 *   gen(ub)       = (uint32)(((uint64)word * ub) >> 32)          in [0, ub)
 *   gen_float(ub) = ((float)(word >> 8) * 2^-24) * ub  (one IEEE multiply)
 */
#ifndef KK_ORACLE_RNG_H
#define KK_ORACLE_RNG_H

#include <stdint.h>

#define KKO_STREAM_WALK 0u
#define KKO_STREAM_INIT_STATE 1u
#define KKO_STREAM_INIT_DIST 2u

static inline void kko_philox4x32_10(const uint32_t ctr_in[4], uint64_t seed, uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; r++)
    {
        if (r != 0)
        {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Per-walker draw cursor.  Caches the current Philox block. */
typedef struct
{
    uint64_t seed;
    uint32_t walker;
    uint32_t step;
    uint32_t stream;
    uint32_t draw;
    uint32_t block_idx; /* block held in buf, or 0xffffffff */
    uint32_t buf[4];
} kko_rng;

static inline void kko_rng_enter(kko_rng *g, uint64_t seed, uint32_t walker, uint32_t step, uint32_t stream, uint32_t draw)
{
    g->seed = seed;
    g->walker = walker;
    g->step = step;
    g->stream = stream;
    g->draw = draw;
    g->block_idx = 0xffffffffu;
}

static inline uint32_t kko_rng_word(kko_rng *g)
{
    uint32_t blk = g->draw >> 2;
    if (blk != g->block_idx)
    {
        uint32_t ctr[4] = {g->walker, g->step, blk, g->stream};
        kko_philox4x32_10(ctr, g->seed, g->buf);
        g->block_idx = blk;
    }
    uint32_t w = g->buf[g->draw & 3u];
    g->draw++;
    return w;
}

static inline uint32_t kko_map_gen(uint32_t word, uint32_t ub)
{
    return (uint32_t)(((uint64_t)word * (uint64_t)ub) >> 32);
}

static inline float kko_map_gen_float(uint32_t word, float ub)
{
    /* (word >> 8) * 2^-24 is exact; the product with ub is the single rounding.
     * Every oracle file is compiled with -ffp-contract=off so that no caller
     * fuses this multiply with a following add. */
    float u = (float)(word >> 8) * (1.0f / 16777216.0f);
    return u * ub;
}

static inline uint32_t kko_gen(kko_rng *g, uint32_t ub)
{
    return kko_map_gen(kko_rng_word(g), ub);
}

static inline float kko_gen_float(kko_rng *g, float ub)
{
    return kko_map_gen_float(kko_rng_word(g), ub);
}

#endif
