/*
 * ORACLE / TEST INFRASTRUCTURE ONLY: CPU restatement of KnightKing's walker-step
 * path (include/walk.hpp) and of its four apps' functors (the src/apps headers).
 *
 * This library is the checker for the CUDA product and the CPU baseline that
 * bench.py times.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * load it.  It is pinned against the reference itself: tests/golden/ holds
 * paths and alias tables produced by the reference's own engine (compiled with
 * a Philox RNG hook), and tests/test_oracle_golden.py checks this library
 * reproduces them bit for bit.
 */
#ifndef KK_ORACLE_H
#define KK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KO_APP_DEEPWALK 0
#define KO_APP_PPR 1
#define KO_APP_NODE2VEC 2
#define KO_APP_METAPATH 3
#define KO_APP_TAGWALK 4
#define KO_APP_DYNWALK 5 /* the return-edge-doubling walk of src/examples/dynamic_walk.cpp:52-93 */

#define KO_MAX_SCHEMES 16
#define KO_MAX_SCHEME_LEN 16

#define KO_OK 0
#define KO_ERR_INVALID 1
#define KO_ERR_PATH_CAPACITY 2

typedef struct
{
    uint32_t V;
    uint64_t E;
    const int64_t *off;   /* V+1 */
    const uint32_t *nbr;  /* E */
    const float *w;       /* E or NULL */
    const uint8_t *etype; /* E or NULL (metapath type / tagwalk edge tag) */
} ko_graph;

typedef struct
{
    int app;
    int weighted; /* static component = edge weight (alias tables) */
    uint64_t seed;
    uint32_t walker_begin;
    uint32_t walker_num;
    uint32_t walk_length;
    float terminate_prob; /* PPR */
    float p, q;           /* node2vec */
    /* metapath */
    int n_schemes;
    int scheme_len[KO_MAX_SCHEMES];
    uint8_t scheme_mask[KO_MAX_SCHEMES][KO_MAX_SCHEME_LEN];
    int scheme_round_robin; /* 0: scheme = gen(n) on stream 1 (src/apps/metapath.hpp:91-95) */
    /* tagwalk */
    int tag_num;
    float vertex_tag_weight;
    float outlier_amplifier;
    int order;   /* 1 or 2 */
    int outlier; /* 0: bound form, 1: outlier form */
    const int32_t *vertex_tag;
    /* optional start list (PPR, src/apps/ppr.hpp:37-51) */
    const uint32_t *start;
    uint32_t n_start;
} ko_walk_params;

/* Alias tables, include/walk.hpp:538-652.  p/p_idx/q_idx sized E (bucket j of
 * vertex v at off[v]+j, indices local to v's adjacency, q_idx = 0xffffffff for
 * a null alias); sum sized V (the sequential float sum, regular_area). */
void ko_alias_build(const ko_graph *g, float *p, uint32_t *p_idx, uint32_t *q_idx, float *sum, int threads);

/* Sorts each adjacency by neighbour, carrying weights and types, as
 * node2vec() does before walking (src/apps/node2vec.hpp:122-125).  In place. */
void ko_sort_adjacency(uint32_t V, const int64_t *off, uint32_t *nbr, float *w, uint8_t *etype);

/* Walks walkers [walker_begin, walker_begin + walker_num).  Walker i of the
 * call writes its length to out_len[i] and its vertices to
 * out_path[i * cap ...] (out_path may be NULL: lengths only).  Returns KO_OK,
 * KO_ERR_INVALID or KO_ERR_PATH_CAPACITY (a path longer than cap). */
int ko_walk(const ko_graph *g, const ko_walk_params *prm, uint32_t cap, uint32_t *out_len, uint32_t *out_path,
            int threads, uint64_t *total_steps);

/* ko_walk with the weight alias tables (and sums) of this graph built
 * beforehand by ko_alias_build, instead of building them in the call as the
 * reference's random_walk does (include/walk.hpp:538-652); NULL tables build
 * them as ko_walk does.  For many calls on one large graph. */
int ko_walk_alias(const ko_graph *g, const ko_walk_params *prm, uint32_t cap, uint32_t *out_len, uint32_t *out_path,
                  int threads, uint64_t *total_steps, const float *alias_p, const uint32_t *alias_pi,
                  const uint32_t *alias_qi, const float *alias_sum);

/* Seconds spent in the alias build and in the walk by the last ko_walk call. */
void ko_last_timing(double *alias_seconds, double *walk_seconds);

/* Synthetic inputs (the project's seeded R-MAT, see graphs.py): raw draws as
 * (min << 32 | max) keys, ~0 for self-loops; and per-edge pair data. */
void ko_rmat_draw(uint32_t scale, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc, uint64_t seed, uint64_t *keys,
                  int threads);
void ko_radix_sort_u64(uint64_t n, uint64_t *keys, uint64_t *tmp, int bits, int threads);
void ko_pair_data(uint64_t n, const uint32_t *src, const uint32_t *dst, uint64_t seed, int weights, uint32_t types,
                  float *w, uint8_t *t, int threads);

/* n Philox4x32-10 blocks of the oracle's generator: ctr[4i..4i+3] in,
 * out[4i..4i+3] out, key = seed (low word k0, high word k1). */
void ko_philox_blocks(uint64_t seed, uint64_t n, const uint32_t *ctr, uint32_t *out);

#ifdef __cplusplus
}
#endif

#endif
