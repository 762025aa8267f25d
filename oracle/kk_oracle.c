/*
 * ORACLE / TEST INFRASTRUCTURE ONLY: plain-C restatement of KnightKing's
 * walker-step path.  See kk_oracle.h for what it is for and how it is pinned.
 *
 * Compile with -ffp-contract=off: every float operation below is one IEEE
 * rounding, in the order the reference performs it.
 *
 * Per walker the reference's semi-asynchronous superstep loop reduces to a
 * sequential loop: walkers interact only through the random stream, and the
 * Philox stream is keyed per walker, so each walker's draws and decisions are
 * those of the superstep engine (include/walk.hpp:946-1067 first order,
 * :1146-1379 second order) in the same order.
 */
#include "kk_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "kk_oracle_rng.h"

#define KO_NONE 0xffffffffu

static double g_alias_seconds = 0.0;
static double g_walk_seconds = 0.0;

static double ko_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

void ko_last_timing(double *alias_seconds, double *walk_seconds)
{
    *alias_seconds = g_alias_seconds;
    *walk_seconds = g_walk_seconds;
}

/* ---- alias tables: include/walk.hpp:538-652 ----------------------------- */

static void ko_alias_vertex(const ko_graph *g, uint32_t v, float *prob, uint32_t *p_set, uint32_t *q_set, float *P,
                            uint32_t *PI, uint32_t *QI, float *sum_out)
{
    int64_t b = g->off[v];
    uint32_t deg = (uint32_t)(g->off[v + 1] - b);
    if (deg == 0)
    {
        return;
    }
    /* sequential float sum in CSR order (:579-584) */
    float sum = 0.0f;
    for (uint32_t e = 0; e < deg; e++)
    {
        prob[e] = g->w[b + e];
        sum += prob[e];
    }
    if (sum_out != NULL)
    {
        sum_out[v] = sum;
    }
    float ave = sum / (float)deg; /* :589 */
    uint32_t ph = 0, pt = 0, qh = 0, qt = 0;
    for (uint32_t e = 0; e < deg; e++) /* :594-603 */
    {
        if (prob[e] < ave)
        {
            p_set[pt++] = e;
        }
        else
        {
            q_set[qt++] = e;
        }
    }
    uint64_t out = (uint64_t)b;
    while (pt != ph) /* :605-630, FIFO pairing */
    {
        uint32_t pi = p_set[ph++];
        if (qt != qh)
        {
            uint32_t qi = q_set[qh++];
            PI[out] = pi;
            P[out] = prob[pi] / ave;
            QI[out] = qi;
            float diff = ave - prob[pi];
            prob[qi] -= diff;
            if (prob[qi] < ave)
            {
                p_set[pt++] = qi;
            }
            else
            {
                q_set[qt++] = qi;
            }
        }
        else
        {
            PI[out] = pi;
            P[out] = 1.0f;
            QI[out] = KO_NONE;
        }
        out++;
    }
    while (qt != qh) /* :631-638 */
    {
        uint32_t qi = q_set[qh++];
        PI[out] = qi;
        P[out] = 1.0f;
        QI[out] = KO_NONE;
        out++;
    }
}

void ko_alias_build(const ko_graph *g, float *P, uint32_t *PI, uint32_t *QI, float *sum, int threads)
{
    uint32_t max_deg = 0;
    for (uint32_t v = 0; v < g->V; v++)
    {
        uint32_t d = (uint32_t)(g->off[v + 1] - g->off[v]);
        if (d > max_deg)
        {
            max_deg = d;
        }
    }
    if (threads <= 0)
    {
        threads = omp_get_max_threads();
    }
#pragma omp parallel num_threads(threads)
    {
        float *prob = (float *)malloc(sizeof(float) * (max_deg + 1));
        uint32_t *p_set = (uint32_t *)malloc(sizeof(uint32_t) * (max_deg + 1));
        uint32_t *q_set = (uint32_t *)malloc(sizeof(uint32_t) * (max_deg + 1));
#pragma omp for schedule(dynamic, 128)
        for (int64_t v = 0; v < (int64_t)g->V; v++)
        {
            ko_alias_vertex(g, (uint32_t)v, prob, p_set, q_set, P, PI, QI, sum);
        }
        free(prob);
        free(p_set);
        free(q_set);
    }
}

/* ---- node2vec adjacency sort: src/apps/node2vec.hpp:122-125 ------------- */

typedef struct
{
    uint32_t nbr;
    float w;
    uint8_t t;
} ko_unit;

static int ko_unit_cmp(const void *a, const void *b)
{
    uint32_t x = ((const ko_unit *)a)->nbr, y = ((const ko_unit *)b)->nbr;
    return x < y ? -1 : (x > y ? 1 : 0);
}

void ko_sort_adjacency(uint32_t V, const int64_t *off, uint32_t *nbr, float *w, uint8_t *etype)
{
    for (uint32_t v = 0; v < V; v++)
    {
        int64_t b = off[v];
        uint32_t d = (uint32_t)(off[v + 1] - b);
        int sorted = 1;
        for (uint32_t i = 1; i < d; i++)
        {
            if (nbr[b + i - 1] > nbr[b + i])
            {
                sorted = 0;
                break;
            }
        }
        if (sorted)
        {
            continue;
        }
        ko_unit *u = (ko_unit *)malloc(sizeof(ko_unit) * d);
        for (uint32_t i = 0; i < d; i++)
        {
            u[i].nbr = nbr[b + i];
            u[i].w = w ? w[b + i] : 0.0f;
            u[i].t = etype ? etype[b + i] : 0;
        }
        qsort(u, d, sizeof(ko_unit), ko_unit_cmp);
        for (uint32_t i = 0; i < d; i++)
        {
            nbr[b + i] = u[i].nbr;
            if (w)
                w[b + i] = u[i].w;
            if (etype)
                etype[b + i] = u[i].t;
        }
        free(u);
    }
}

/* ---- per-call derived data --------------------------------------------- */

typedef struct
{
    const ko_graph *g;
    const ko_walk_params *prm;
    /* alias tables (weighted) */
    float *ap;
    uint32_t *api, *aqi;
    float *sum;
    /* dynamic component bounds (include/walk.hpp:499-536) */
    int dynamic;
    int has_lb;
    int outlier;
    float *ub, *lb, *ra; /* ra: regular_area (:750-781) */
    /* node2vec constants (src/apps/node2vec.hpp:126-139) */
    float n2v_ub, n2v_lb, n2v_overflow, inv_p, inv_q;
    /* metapath (src/apps/metapath.hpp:77-88) */
    uint8_t *vmask;
    /* tagwalk: per (vertex, tag) range of the tag-grouped adjacency */
    uint32_t *tag_begin, *tag_end;
} ko_ctx;

typedef struct
{
    uint32_t a; /* node2vec: previous vertex; metapath: scheme id; tagwalk: tag; dynwalk: last vertex */
    uint32_t b; /* metapath: state; tagwalk: previous vertex */
} ko_state;

static inline float ko_weight(const ko_ctx *c, uint64_t e)
{
    return c->g->w[e];
}

/* ---- functors ----------------------------------------------------------- */

/* extension_comp (deepwalk.hpp:36-38, ppr.hpp:56-58, node2vec.hpp:145-148,
 * metapath.hpp:102-105) */
static inline float ko_ext(const ko_ctx *c, const ko_state *s, uint32_t step, uint32_t v)
{
    const ko_walk_params *p = c->prm;
    switch (p->app)
    {
    case KO_APP_PPR:
        return 1.0f - p->terminate_prob;
    case KO_APP_METAPATH:
        return (step >= p->walk_length || !(c->vmask[v] & p->scheme_mask[s->a][s->b])) ? 0.0f : 1.0f;
    default:
        return step >= p->walk_length ? 0.0f : 1.0f;
    }
}

/* lower_bound of x in v's sorted adjacency, as a local index (deg if none) */
static inline uint32_t ko_lower_bound(const ko_graph *g, uint32_t v, uint32_t x)
{
    int64_t b = g->off[v];
    uint32_t lo = 0, hi = (uint32_t)(g->off[v + 1] - b);
    while (lo < hi)
    {
        uint32_t mid = lo + (hi - lo) / 2;
        if (g->nbr[b + mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

static inline int ko_adjacent(const ko_graph *g, uint32_t u, uint32_t x)
{
    uint32_t i = ko_lower_bound(g, u, x);
    return i < (uint32_t)(g->off[u + 1] - g->off[u]) && g->nbr[g->off[u] + i] == x;
}

/* outlier_upperbound (node2vec.hpp:47-83; tag walk) */
static inline void ko_outlier_ub(const ko_ctx *c, const ko_state *s, uint32_t step, uint32_t v, float *ob, uint32_t *on)
{
    const ko_walk_params *p = c->prm;
    if (p->app == KO_APP_NODE2VEC)
    {
        if (c->prm->weighted)
        {
            uint32_t i = ko_lower_bound(c->g, v, s->a);
            uint32_t deg = (uint32_t)(c->g->off[v + 1] - c->g->off[v]);
            /* The reference reads past the adjacency when the previous vertex
             * is not a neighbour (directed graphs); here the area is empty. */
            *ob = i < deg ? ko_weight(c, c->g->off[v] + i) * c->n2v_overflow : 0.0f;
        }
        else
        {
            *ob = c->n2v_overflow;
        }
        *on = 1;
        return;
    }
    /* tag walk, outlier form */
    if (step != 0)
    {
        int T = p->tag_num;
        uint32_t b = c->tag_begin[(uint64_t)v * T + s->a], e = c->tag_end[(uint64_t)v * T + s->a];
        float pu = 0.0f;
        for (uint32_t i = b; i < e; i++)
        {
            float wt = p->weighted ? ko_weight(c, c->g->off[v] + i) : 1.0f;
            float cand = (float)T * (p->outlier_amplifier - 1.0f) * wt;
            if (pu < cand)
                pu = cand;
        }
        *ob = pu;
        *on = e - b;
    }
    else
    {
        *ob = 0.0f;
        *on = 0;
    }
}

/* outlier_search: local edge index or KO_NONE */
static inline uint32_t ko_outlier_search(const ko_ctx *c, const ko_state *s, uint32_t v, uint32_t idx)
{
    if (c->prm->app == KO_APP_NODE2VEC)
    {
        uint32_t i = ko_lower_bound(c->g, v, s->a);
        uint32_t deg = (uint32_t)(c->g->off[v + 1] - c->g->off[v]);
        return i < deg ? i : KO_NONE;
    }
    int T = c->prm->tag_num;
    return c->tag_begin[(uint64_t)v * T + s->a] + idx;
}

/* first-order dynamic_comp (metapath.hpp:107-116; tag walk) */
static inline float ko_dyn1(const ko_ctx *c, const ko_state *s, uint32_t step, uint32_t v, uint64_t e)
{
    const ko_walk_params *p = c->prm;
    if (p->app == KO_APP_METAPATH)
    {
        uint8_t t = c->g->etype[e];
        return ((p->scheme_mask[s->a][s->b] >> t) & 1u) ? 1.0f : 0.0f;
    }
    if (p->app == KO_APP_DYNWALK)
    {
        /* src/examples/dynamic_walk.cpp:72-88: 1 at step 0, 2 back to the last vertex, else 1 */
        if (step == 0)
            return 1.0f;
        return c->g->nbr[e] == s->a ? 2.0f : 1.0f;
    }
    /* tag walk */
    int T = p->tag_num;
    if (step == 0)
        return (float)T;
    int et = (int)c->g->etype[e];
    float temp = 1.0f + (float)((p->vertex_tag[s->b] + (int)s->a + et) % T);
    if (p->outlier)
    {
        if ((int)s->a == et)
            temp *= p->outlier_amplifier;
    }
    else
    {
        temp += (float)p->vertex_tag[v] * p->vertex_tag_weight;
    }
    return temp;
}

/* second-order dynamic_comp with the response (node2vec.hpp:167-185; tag walk) */
static inline float ko_dyn2(const ko_ctx *c, const ko_state *s, uint32_t step, int32_t resp, uint32_t v, uint64_t e)
{
    const ko_walk_params *p = c->prm;
    if (p->app == KO_APP_NODE2VEC)
    {
        if (step == 0)
            return c->n2v_ub;
        uint32_t nb = c->g->nbr[e];
        if (s->a == nb)
            return c->inv_p;
        if (resp)
            return 1.0f;
        return c->inv_q;
    }
    int T = p->tag_num;
    if (step == 0)
        return (float)T;
    int et = (int)c->g->etype[e];
    float temp = 1.0f + (float)((resp + (int)s->a + et) % T);
    if (p->outlier)
    {
        if ((int)s->a == et)
            temp *= p->outlier_amplifier;
    }
    else
    {
        temp += (float)p->vertex_tag[v] * p->vertex_tag_weight;
    }
    return temp;
}

/* respond_query: node2vec binary_search (node2vec.hpp:158-166); tag walk:
 * the previous vertex's tag.  Called only when post_query emitted (step != 0). */
static inline int32_t ko_respond(const ko_ctx *c, const ko_state *s, uint64_t e)
{
    if (c->prm->app == KO_APP_NODE2VEC)
    {
        return ko_adjacent(c->g, s->a, c->g->nbr[e]);
    }
    return c->prm->vertex_tag[s->b];
}

static inline void ko_update(const ko_ctx *c, ko_state *s, uint32_t v)
{
    switch (c->prm->app)
    {
    case KO_APP_NODE2VEC:
        s->a = v;
        break;
    case KO_APP_METAPATH:
        s->b = (s->b + 1) % (uint32_t)c->prm->scheme_len[s->a];
        break;
    case KO_APP_TAGWALK:
        s->a = (s->a + 1) % (uint32_t)c->prm->tag_num;
        s->b = v;
        break;
    case KO_APP_DYNWALK:
        s->a = v; /* dynamic_walk.cpp:62-65 */
        break;
    default:
        break;
    }
}

/* candidate pick: uniform (:1016-1018) or alias (:1020-1028) */
static inline uint32_t ko_pick(const ko_ctx *c, kko_rng *g, uint32_t v, uint32_t deg)
{
    if (c->ap == NULL)
    {
        return kko_gen(g, deg);
    }
    uint64_t j = (uint64_t)c->g->off[v] + kko_gen(g, deg);
    if (c->aqi[j] == KO_NONE || kko_gen_float(g, 1.0f) < c->ap[j])
    {
        return c->api[j];
    }
    return c->aqi[j];
}

/* ---- one walker --------------------------------------------------------- */

static int ko_walk_one(const ko_ctx *c, uint32_t id, uint32_t cap, uint32_t *len_out, uint32_t *path)
{
    const ko_walk_params *p = c->prm;
    const ko_graph *g = c->g;
    kko_rng rng;
    ko_state s = {0, 0};
    uint32_t v;
    /* start vertex (include/walk.hpp:403-411, ppr.hpp:37-51) */
    if (p->start != NULL && p->n_start > 0)
        v = p->start[id % p->n_start];
    else
        v = id % g->V;
    /* init state (metapath.hpp:91-95; tag walk) */
    if (p->app == KO_APP_METAPATH)
    {
        if (p->scheme_round_robin)
        {
            s.a = id % (uint32_t)p->n_schemes;
        }
        else
        {
            kko_rng_enter(&rng, p->seed, id, 0, KKO_STREAM_INIT_STATE, 0);
            s.a = kko_gen(&rng, (uint32_t)p->n_schemes);
        }
        s.b = 0;
    }
    else if (p->app == KO_APP_TAGWALK)
    {
        s.a = id % (uint32_t)p->tag_num;
    }
    else if (p->app == KO_APP_DYNWALK)
    {
        s.a = 0xffffffffu; /* dynamic_walk.cpp:57-61: no last vertex yet */
    }
    uint32_t step = 0;
    uint32_t len = 1;
    if (path != NULL)
    {
        if (cap < 1)
            return KO_ERR_PATH_CAPACITY;
        path[0] = v;
    }
    int second = (p->app == KO_APP_NODE2VEC) || (p->app == KO_APP_TAGWALK && p->order == 2);
    for (;;)
    {
        int64_t base = g->off[v];
        uint32_t deg = (uint32_t)(g->off[v + 1] - base);
        if (deg == 0)
            break;
        kko_rng_enter(&rng, p->seed, id, step, KKO_STREAM_WALK, 0);
        uint32_t ac = KO_NONE;
        if (!second)
        {
            float ext = ko_ext(c, &s, step, v);
            if (ext == 0.0f || (ext < 1.0f && kko_gen_float(&rng, 1.0f) > ext))
                break;
            while (ac == KO_NONE)
            {
                if (c->outlier)
                {
                    float ob;
                    uint32_t on;
                    ko_outlier_ub(c, &s, step, v, &ob, &on);
                    if (ob > 0.0f && on > 0)
                    {
                        float r = kko_gen_float(&rng, ob * (float)on + c->ra[v]) - c->ra[v];
                        if (r > 0.0f)
                        {
                            uint32_t oi = (uint32_t)(r / ob);
                            if (oi + 1 > on)
                                oi = on - 1;
                            uint32_t cand = ko_outlier_search(c, &s, v, oi);
                            if (cand != KO_NONE)
                            {
                                float sc = p->weighted ? ko_weight(c, base + cand) : 1.0f;
                                float r2 = (r - (float)oi * ob) / sc + c->ub[v];
                                if (r2 <= ko_dyn1(c, &s, step, v, base + cand))
                                    ac = cand;
                            }
                            continue;
                        }
                    }
                }
                uint32_t cand = ko_pick(c, &rng, v, deg);
                if (c->dynamic)
                {
                    float dart = kko_gen_float(&rng, c->ub[v]);
                    if ((c->has_lb && dart <= c->lb[v]) || dart <= ko_dyn1(c, &s, step, v, base + cand))
                        ac = cand;
                }
                else
                {
                    ac = cand;
                }
            }
        }
        else
        {
            /* second order: each pass of this loop is one superstep's trial */
            int terminated = 0;
            for (;;)
            {
                float ext = ko_ext(c, &s, step, v);
                if (ext == 0.0f || (ext < 1.0f && kko_gen_float(&rng, 1.0f) > ext))
                {
                    terminated = 1;
                    break;
                }
                uint32_t cand = KO_NONE;
                float randval = 0.0f;
                int accepted = 0;
                for (;;) /* include/walk.hpp:1176-1258 */
                {
                    int in_app = 0;
                    if (c->outlier)
                    {
                        float ob;
                        uint32_t on;
                        ko_outlier_ub(c, &s, step, v, &ob, &on);
                        if (ob > 0.0f && on > 0)
                        {
                            float r = kko_gen_float(&rng, ob * (float)on + c->ra[v]) - c->ra[v];
                            if (r > 0.0f)
                            {
                                in_app = 1;
                                uint32_t oi = (uint32_t)(r / ob);
                                if (oi + 1 > on)
                                    oi = on - 1;
                                cand = ko_outlier_search(c, &s, v, oi);
                                if (cand != KO_NONE)
                                {
                                    float sc = p->weighted ? ko_weight(c, base + cand) : 1.0f;
                                    randval = (r - (float)oi * ob) / sc + c->ub[v];
                                    break; /* query posted */
                                }
                            }
                        }
                    }
                    if (!in_app)
                    {
                        cand = ko_pick(c, &rng, v, deg);
                        randval = kko_gen_float(&rng, c->ub[v]);
                        if (c->has_lb && randval <= c->lb[v])
                            accepted = 1;
                        break;
                    }
                }
                if (accepted)
                {
                    ac = cand;
                    break;
                }
                int32_t resp = 0;
                if (step != 0)
                    resp = ko_respond(c, &s, base + cand);
                if (randval <= ko_dyn2(c, &s, step, resp, v, base + cand))
                {
                    ac = cand;
                    break;
                }
            }
            if (terminated)
                break;
        }
        uint32_t nv = g->nbr[base + ac];
        step++;
        ko_update(c, &s, v);
        if (path != NULL)
        {
            if (len >= cap)
                return KO_ERR_PATH_CAPACITY;
            path[len] = nv;
        }
        len++;
        v = nv;
    }
    *len_out = len;
    return KO_OK;
}

/* ---- call setup: include/walk.hpp:698-781 and the apps' bounds ---------- */

int ko_walk(const ko_graph *g, const ko_walk_params *p, uint32_t cap, uint32_t *out_len, uint32_t *out_path, int threads,
            uint64_t *total_steps)
{
    return ko_walk_alias(g, p, cap, out_len, out_path, threads, total_steps, NULL, NULL, NULL, NULL);
}

int ko_walk_alias(const ko_graph *g, const ko_walk_params *p, uint32_t cap, uint32_t *out_len, uint32_t *out_path,
                  int threads, uint64_t *total_steps, const float *alias_p, const uint32_t *alias_pi,
                  const uint32_t *alias_qi, const float *alias_sum)
{
    ko_ctx c;
    memset(&c, 0, sizeof(c));
    c.g = g;
    c.prm = p;
    if (threads <= 0)
        threads = omp_get_max_threads();
    if (p->weighted && g->w == NULL)
        return KO_ERR_INVALID;
    if ((p->app == KO_APP_METAPATH || p->app == KO_APP_TAGWALK) && g->etype == NULL)
        return KO_ERR_INVALID;
    if (p->app == KO_APP_METAPATH && (p->n_schemes <= 0 || p->n_schemes > KO_MAX_SCHEMES))
        return KO_ERR_INVALID;
    if (p->app == KO_APP_TAGWALK && (p->tag_num <= 0 || p->vertex_tag == NULL))
        return KO_ERR_INVALID;
    uint32_t V = g->V;

    /* bounds (include/walk.hpp:499-536) */
    if (p->app == KO_APP_NODE2VEC)
    {
        double inv_q = 1.0 / (double)p->q;
        double inv_p = 1.0 / (double)p->p;
        c.n2v_ub = (float)(inv_q > 1.0 ? inv_q : 1.0);
        double lbd = inv_q < 1.0 ? inv_q : 1.0;
        c.n2v_lb = (float)(inv_p < lbd ? inv_p : lbd);
        c.n2v_overflow = (float)(inv_p - (double)c.n2v_ub);
        c.inv_p = 1.0f / p->p;
        c.inv_q = 1.0f / p->q;
        c.dynamic = 1;
        c.has_lb = 1;
        c.outlier = c.n2v_overflow > 0.0f;
    }
    else if (p->app == KO_APP_DYNWALK)
    {
        c.dynamic = 1; /* upper bound 2, no lower bound, no outlier (dynamic_walk.cpp:89-92) */
    }
    else if (p->app == KO_APP_METAPATH)
    {
        c.dynamic = 1;
        c.vmask = (uint8_t *)calloc(V, 1);
        for (uint32_t v = 0; v < V; v++)
            for (int64_t e = g->off[v]; e < g->off[v + 1]; e++)
                c.vmask[v] |= (uint8_t)(1u << g->etype[e]);
    }
    else if (p->app == KO_APP_TAGWALK)
    {
        c.dynamic = 1;
        c.has_lb = 1;
        c.outlier = p->outlier;
        if (p->outlier)
        {
            int T = p->tag_num;
            c.tag_begin = (uint32_t *)calloc((size_t)V * T, 4);
            c.tag_end = (uint32_t *)calloc((size_t)V * T, 4);
            for (uint32_t v = 0; v < V; v++)
                for (int64_t e = g->off[v]; e < g->off[v + 1]; e++)
                {
                    int t = g->etype[e];
                    uint32_t li = (uint32_t)(e - g->off[v]);
                    if (c.tag_begin[(uint64_t)v * T + t] == c.tag_end[(uint64_t)v * T + t])
                        c.tag_begin[(uint64_t)v * T + t] = li;
                    c.tag_end[(uint64_t)v * T + t] = li + 1;
                }
        }
    }
    if (c.dynamic)
    {
        c.ub = (float *)malloc(sizeof(float) * V);
        c.lb = (float *)malloc(sizeof(float) * V);
        for (uint32_t v = 0; v < V; v++)
        {
            if (p->app == KO_APP_NODE2VEC)
            {
                c.ub[v] = c.n2v_ub;
                c.lb[v] = c.n2v_lb;
            }
            else if (p->app == KO_APP_METAPATH)
            {
                c.ub[v] = 1.0f;
                c.lb[v] = 0.0f;
            }
            else if (p->app == KO_APP_DYNWALK)
            {
                c.ub[v] = 2.0f;
                c.lb[v] = 0.0f;
            }
            else if (p->outlier)
            {
                c.ub[v] = (float)p->tag_num;
                c.lb[v] = 1.0f;
            }
            else
            {
                c.ub[v] = (float)p->tag_num + (float)p->vertex_tag[v] * p->vertex_tag_weight;
                c.lb[v] = (float)p->vertex_tag[v] * p->vertex_tag_weight;
            }
        }
    }
    double t0 = ko_now();
    const int own_alias = p->weighted && alias_p == NULL;
    if (own_alias)
    {
        c.ap = (float *)malloc(sizeof(float) * g->E);
        c.api = (uint32_t *)malloc(sizeof(uint32_t) * g->E);
        c.aqi = (uint32_t *)malloc(sizeof(uint32_t) * g->E);
        c.sum = (float *)calloc(V, sizeof(float));
        ko_alias_build(g, c.ap, c.api, c.aqi, c.sum, threads);
    }
    else if (p->weighted)
    {
        /* tables the caller built with ko_alias_build on this graph */
        c.ap = (float *)alias_p;
        c.api = (uint32_t *)alias_pi;
        c.aqi = (uint32_t *)alias_qi;
        c.sum = (float *)alias_sum;
    }
    if (c.outlier)
    {
        /* regular_area (include/walk.hpp:750-781) */
        c.ra = (float *)calloc(V, sizeof(float));
        for (uint32_t v = 0; v < V; v++)
        {
            if (p->weighted)
                c.ra[v] = c.sum[v] * c.ub[v];
            else
                c.ra[v] = (float)(uint32_t)(g->off[v + 1] - g->off[v]) * c.ub[v];
        }
    }
    double t1 = ko_now();
    int status = KO_OK;
    uint64_t steps = 0;
#pragma omp parallel for schedule(dynamic, 128) num_threads(threads) reduction(+ : steps)
    for (int64_t i = 0; i < (int64_t)p->walker_num; i++)
    {
        uint32_t len = 0;
        int st = ko_walk_one(&c, p->walker_begin + (uint32_t)i, cap, &len,
                             out_path ? out_path + (uint64_t)i * cap : NULL);
        if (st != KO_OK)
        {
#pragma omp atomic write
            status = st;
        }
        if (out_len)
            out_len[i] = len;
        steps += len - 1;
    }
    double t2 = ko_now();
    g_alias_seconds = t1 - t0;
    g_walk_seconds = t2 - t1;
    if (total_steps)
        *total_steps = steps;
    if (own_alias)
    {
        free(c.ap);
        free(c.api);
        free(c.aqi);
        free(c.sum);
    }
    free(c.ub);
    free(c.lb);
    free(c.ra);
    free(c.vmask);
    free(c.tag_begin);
    free(c.tag_end);
    return status;
}

/* ---- synthetic inputs: the project's seeded R-MAT (see graphs.py) ------- */

void ko_rmat_draw(uint32_t scale, uint64_t m, uint64_t ta, uint64_t tab, uint64_t tabc, uint64_t seed, uint64_t *keys,
                  int threads)
{
    if (threads <= 0)
        threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)m; i++)
    {
        uint64_t src = 0, dst = 0;
        for (uint32_t blk = 0; blk * 4 < scale; blk++)
        {
            uint32_t ctr[4] = {(uint32_t)i, 0, blk, 3}, w4[4];
            kko_philox4x32_10(ctr, seed, w4);
            for (uint32_t j = 0; j < 4 && blk * 4 + j < scale; j++)
            {
                uint64_t w = w4[j];
                uint64_t sbit = w >= tab;
                uint64_t dbit = ((w >= ta) && (w < tab)) || (w >= tabc);
                src = (src << 1) | sbit;
                dst = (dst << 1) | dbit;
            }
        }
        uint64_t lo = src < dst ? src : dst, hi = src < dst ? dst : src;
        keys[i] = (src == dst) ? ~0ull : ((lo << 32) | hi);
    }
}

/* Per directed edge (s, d): data of the unordered pair (min, max).  weights:
 * 1 uniform [1,5), 2 lognormal(0,1) (Box-Muller); types > 0: edge type. */
void ko_pair_data(uint64_t n, const uint32_t *src, const uint32_t *dst, uint64_t seed, int weights, uint32_t types,
                  float *w, uint8_t *t, int threads)
{
    if (threads <= 0)
        threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t i = 0; i < (int64_t)n; i++)
    {
        uint32_t s = src[i], d = dst[i];
        uint32_t ctr[4] = {s < d ? s : d, s < d ? d : s, 0, 4}, r[4];
        kko_philox4x32_10(ctr, seed, r);
        if (w != NULL)
        {
            if (weights == 1)
            {
                w[i] = 1.0f + kko_map_gen_float(r[0], 1.0f) * 4.0f;
            }
            else
            {
                float u1 = (float)((r[2] >> 8) + 1) * (1.0f / 16777216.0f);
                float u2 = (float)(r[3] >> 8) * (1.0f / 16777216.0f);
                w[i] = expf(sqrtf(-2.0f * logf(u1)) * cosf(6.283185307179586f * u2));
            }
        }
        if (t != NULL)
            t[i] = (uint8_t)(((uint64_t)r[1] * types) >> 32);
    }
}

/* Stable LSD radix sort of the low `bits` bits of n keys (11-bit digits),
 * parallel histograms and scatter; the result ends in keys. */
void ko_radix_sort_u64(uint64_t n, uint64_t *keys, uint64_t *tmp, int bits, int threads)
{
    if (threads <= 0)
        threads = omp_get_max_threads();
    const int D = 11, R = 1 << 11;
    uint64_t *hist = (uint64_t *)calloc((size_t)threads * R, sizeof(uint64_t));
    uint64_t *src = keys, *dst = tmp;
    for (int shift = 0; shift < bits; shift += D)
    {
        memset(hist, 0, (size_t)threads * R * sizeof(uint64_t));
#pragma omp parallel num_threads(threads)
        {
            int t = omp_get_thread_num();
            uint64_t lo = n * t / threads, hi = n * (t + 1) / threads;
            uint64_t *h = hist + (size_t)t * R;
            for (uint64_t i = lo; i < hi; i++)
                h[(src[i] >> shift) & (R - 1)]++;
#pragma omp barrier
#pragma omp single
            {
                uint64_t run = 0;
                for (int d = 0; d < R; d++)
                    for (int u = 0; u < threads; u++)
                    {
                        uint64_t c = hist[(size_t)u * R + d];
                        hist[(size_t)u * R + d] = run;
                        run += c;
                    }
            }
            for (uint64_t i = lo; i < hi; i++)
                dst[h[(src[i] >> shift) & (R - 1)]++] = src[i];
        }
        uint64_t *x = src;
        src = dst;
        dst = x;
    }
    if (src != keys)
        memcpy(keys, src, n * sizeof(uint64_t));
    free(hist);
}

void ko_philox_blocks(uint64_t seed, uint64_t n, const uint32_t *ctr, uint32_t *out)
{
    for (uint64_t i = 0; i < n; i++)
        kko_philox4x32_10(ctr + 4 * i, seed, out + 4 * i);
}
