/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Runs KnightKing's own walk engine (include/walk.hpp, include/graph.hpp,
 * include/path.hpp) and app functors (the src/apps headers), unmodified and compiled
 * from where they lie, as a single process through the MPI shim in shim/.
 * The reference's per-thread std::mt19937 generator (include/util.hpp:45-70)
 * is replaced by a Philox hook (kk_oracle_rng.h) keyed by
 * (seed, walker id, step, draw index), so that its paths can be compared bit
 * for bit with this project's kernels and with the C restatement.
 *
 * Built by oracle/Makefile into oracle/_ref/ (never into the product).  With
 * -DKK_STOCK_RNG the hook is left out and the reference's own mt19937 runs;
 * that build is only used to time the reference.
 *
 * Usage: kk_ref <cmd> --graph FILE --v V --kind KIND [options] --out FILE
 *   cmd  = alias | deepwalk | ppr | node2vec | metapath | tagwalk | dynwalk
 *   kind = none | f32 | meta | meta_f32 | tag | tag_f32
 * Output files are little-endian binary, read by tests/golden/make_golden.py:
 *   paths: "KKP1", u32 n, u32 len[n], u32 vertices[sum(len)] (walker id order)
 *   alias: "KKA1", u32 V, u64 E, f32 p[E], u32 p_idx[E], u32 q_idx[E], f32 sum[V]
 */
#include <assert.h>
#include <limits.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/resource.h>
#include <sys/time.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <iostream>
#include <map>
#include <mutex>
#include <random>
#include <set>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

#include "../kk_oracle_rng.h"

/* ---- RNG hook -------------------------------------------------------- */

#ifndef KK_STOCK_RNG
#define StdRandNumGenerator KKStockRandNumGenerator
#include "util.hpp"
#undef StdRandNumGenerator

namespace kkhook
{
static uint64_t g_seed = 0;
static std::vector<uint32_t> g_saved_step;
static std::vector<uint32_t> g_saved_draw;

struct Ctx
{
    bool valid;
    uint32_t walker, step, stream, draw;
    kko_rng rng;
};
static thread_local Ctx t_ctx = {false, 0, 0, 0, 0, {}};

static void reset(uint64_t seed, size_t walker_num)
{
    g_seed = seed;
    g_saved_step.assign(walker_num, 0xffffffffu);
    g_saved_draw.assign(walker_num, 0);
}

/* Called by the wrapped extension functor at the start of every step (first
 * order, include/walk.hpp:963) and of every trial (second order,
 * include/walk.hpp:1167).  A trial of the same (walker, step) resumes the
 * draw index where the previous trial left it. */
static void enter_walk(uint32_t walker, uint32_t step)
{
    assert(walker < g_saved_step.size());
    uint32_t draw = (g_saved_step[walker] == step) ? g_saved_draw[walker] : 0;
    g_saved_step[walker] = step;
    g_saved_draw[walker] = draw;
    t_ctx.valid = true;
    t_ctx.walker = walker;
    t_ctx.step = step;
    t_ctx.stream = KKO_STREAM_WALK;
    kko_rng_enter(&t_ctx.rng, g_seed, walker, step, KKO_STREAM_WALK, draw);
}

static void enter_aux(uint32_t walker, uint32_t stream)
{
    t_ctx.valid = true;
    t_ctx.walker = walker;
    t_ctx.step = 0;
    t_ctx.stream = stream;
    kko_rng_enter(&t_ctx.rng, g_seed, walker, 0, stream, 0);
}

static void leave()
{
    t_ctx.valid = false;
}

static uint32_t word()
{
    if (!t_ctx.valid)
    {
        fprintf(stderr, "kk_ref: random draw outside a walker context\n");
        abort();
    }
    uint32_t w = kko_rng_word(&t_ctx.rng);
    if (t_ctx.stream == KKO_STREAM_WALK)
    {
        g_saved_draw[t_ctx.walker] = t_ctx.rng.draw;
    }
    return w;
}
} // namespace kkhook

class KKPhiloxHookRNG : public RandNumGenerator
{
public:
    vertex_id_t gen(vertex_id_t upper_bound)
    {
        return kko_map_gen(kkhook::word(), upper_bound);
    }
    float gen_float(float upper_bound)
    {
        return kko_map_gen_float(kkhook::word(), upper_bound);
    }
};
#define StdRandNumGenerator KKPhiloxHookRNG
#endif /* KK_STOCK_RNG */

/* Test-only access to the engine's alias tables (include/walk.hpp:538-652). */
#define private public
#define protected public
#include "walk.hpp"
#undef private
#undef protected

#include "deepwalk.hpp"
#include "metapath.hpp"
#include "node2vec.hpp"
#include "ppr.hpp"
#include "static_comp.hpp"

/* ---- Tag walks: custom functors for the generic hook API ---------------
 * Modelled on the bound and outlier tag walks of src/tests/test_bound.cpp:105-193
 * and src/tests/test_outlier.cpp:105-252.  Edge data carries an int tag (and a
 * weight in the weighted form); every vertex has a tag.  The outlier form
 * expects each adjacency grouped by edge tag (the input file is written sorted
 * by (src, tag, dst)), so no sort is needed here. */
struct KKTag
{
    int tag;
    real_t get_weight() { return 1.0; }
};
struct KKWeightedTag
{
    int tag;
    real_t weight;
    real_t get_weight() { return weight; }
};
struct KKTagState
{
    int tag;
    vertex_id_t previous_vertex;
};
struct KKTagConf
{
    walker_id_t walker_num;
    step_t walk_length;
    int tag_num;
    real_t vertex_tag_weight;
    real_t outlier_amplifier;
};

template <typename E>
std::function<real_t(vertex_id_t, AdjUnit<E> *)> kk_tag_static_comp();
template <>
std::function<real_t(vertex_id_t, AdjUnit<KKTag> *)> kk_tag_static_comp<KKTag>()
{
    return nullptr;
}
template <>
std::function<real_t(vertex_id_t, AdjUnit<KKWeightedTag> *)> kk_tag_static_comp<KKWeightedTag>()
{
    return [](vertex_id_t, AdjUnit<KKWeightedTag> *e) { return e->data.weight; };
}

template <typename E>
void kk_tagwalk(WalkEngine<E, KKTagState> *graph, KKTagConf conf, std::vector<int> &vtag, int order, bool outlier, WalkConfig *walk_conf)
{
    const int T = conf.tag_num;
    std::vector<vertex_id_t> tag_begin, tag_end;
    if (outlier)
    {
        vertex_id_t V = graph->get_vertex_num();
        tag_begin.assign((size_t)V * T, 0);
        tag_end.assign((size_t)V * T, 0);
        for (vertex_id_t v = 0; v < V; v++)
        {
            AdjUnit<E> *b = graph->csr->adj_lists[v].begin, *e = graph->csr->adj_lists[v].end;
            for (AdjUnit<E> *p = b; p < e; p++)
            {
                int c = p->data.tag;
                if (tag_begin[(size_t)v * T + c] == tag_end[(size_t)v * T + c])
                {
                    tag_begin[(size_t)v * T + c] = (vertex_id_t)(p - b);
                }
                tag_end[(size_t)v * T + c] = (vertex_id_t)(p - b + 1);
            }
        }
    }
    WalkerConfig<E, KKTagState> walker_conf(
        conf.walker_num,
        [&](Walker<KKTagState> &w, vertex_id_t) { w.data.tag = w.id % T; },
        [&](Walker<KKTagState> &w, vertex_id_t cur, AdjUnit<E> *) {
            w.data.tag = (w.data.tag + 1) % T;
            w.data.previous_vertex = cur;
        });
    auto ext = [&](Walker<KKTagState> &w, vertex_id_t) { return w.step >= conf.walk_length ? 0.0 : 1.0; };
    std::function<real_t(vertex_id_t, AdjList<E> *)> ub, lb;
    if (outlier)
    {
        ub = [&](vertex_id_t, AdjList<E> *) { return (real_t)T; };
        lb = [&](vertex_id_t, AdjList<E> *) { return (real_t)1; };
    }
    else
    {
        ub = [&](vertex_id_t v, AdjList<E> *) { return (real_t)T + vtag[v] * conf.vertex_tag_weight; };
        lb = [&](vertex_id_t v, AdjList<E> *) { return (real_t)vtag[v] * conf.vertex_tag_weight; };
    }
    std::function<void(Walker<KKTagState> &, vertex_id_t, AdjList<E> *, real_t &, vertex_id_t &)> out_ub = nullptr;
    std::function<AdjUnit<E> *(Walker<KKTagState> &, vertex_id_t, AdjList<E> *, vertex_id_t)> out_search = nullptr;
    if (outlier)
    {
        out_ub = [&](Walker<KKTagState> &w, vertex_id_t v, AdjList<E> *adj, real_t &prob_ub, vertex_id_t &num_ub) {
            if (w.step != 0)
            {
                vertex_id_t b = tag_begin[(size_t)v * T + w.data.tag], e = tag_end[(size_t)v * T + w.data.tag];
                prob_ub = 0;
                num_ub = e - b;
                for (AdjUnit<E> *p = adj->begin + b; p < adj->begin + e; p++)
                {
                    prob_ub = std::max(prob_ub, T * (conf.outlier_amplifier - 1) * p->data.get_weight());
                }
            }
            else
            {
                prob_ub = 0;
                num_ub = 0;
            }
        };
        out_search = [&](Walker<KKTagState> &w, vertex_id_t v, AdjList<E> *adj, vertex_id_t idx) {
            return adj->begin + tag_begin[(size_t)v * T + w.data.tag] + idx;
        };
    }
    auto dyn_value = [&](KKTagState &s, step_t step, int prev_tag, vertex_id_t v, AdjUnit<E> *edge) {
        if (step == 0)
        {
            return (real_t)T;
        }
        real_t temp = (real_t)1 + (prev_tag + s.tag + edge->data.tag) % T;
        if (outlier)
        {
            if (s.tag == edge->data.tag)
            {
                temp *= conf.outlier_amplifier;
            }
        }
        else
        {
            temp += vtag[v] * conf.vertex_tag_weight;
        }
        return temp;
    };
    if (order == 1)
    {
        TransitionConfig<E, KKTagState> tr(
            ext, kk_tag_static_comp<E>(),
            [&](Walker<KKTagState> &w, vertex_id_t v, AdjUnit<E> *edge) {
                int prev_tag = w.step == 0 ? 0 : vtag[w.data.previous_vertex];
                return dyn_value(w.data, w.step, prev_tag, v, edge);
            },
            ub, lb, out_ub, out_search);
        graph->random_walk(&walker_conf, &tr, walk_conf);
    }
    else
    {
        SecondOrderTransitionConfig<E, KKTagState, EmptyData, int> tr(
            ext, kk_tag_static_comp<E>(),
            [&](Walker<KKTagState> &w, walker_id_t walker_idx, vertex_id_t cur, AdjUnit<E> *) {
                if (w.step != 0)
                {
                    stateQuery<EmptyData> q;
                    q.src_v = cur;
                    q.walker_idx = walker_idx;
                    graph->emit(w.data.previous_vertex, q);
                }
            },
            [&](vertex_id_t vtx, stateQuery<EmptyData> q, AdjList<E> *) {
                stateResponse<int> r;
                r.walker_idx = q.walker_idx;
                r.data = vtag[vtx];
                graph->emit(q.src_v, r);
            },
            [&](Walker<KKTagState> &w, stateResponse<int> &r, vertex_id_t v, AdjUnit<E> *edge) {
                return dyn_value(w.data, w.step, w.step == 0 ? 0 : r.data, v, edge);
            },
            ub, lb, out_ub, out_search);
        graph->random_walk(&walker_conf, &tr, walk_conf);
    }
}

/* ---- Dynamic walk: the configuration of src/examples/dynamic_walk.cpp:52-93 ----
 * Weighted first-order walk whose dynamic component doubles the return edge:
 * the walker remembers the vertex it came from (UINT_MAX before its first
 * step), dynamic_comp is 1 at step 0, 2 for an edge back to that vertex and 1
 * otherwise, with upper bound 2.  The lambdas are the example's, with its
 * fixed walker count made a parameter. */
struct KKDynWalkState
{
    vertex_id_t last_vertex;
};

template <typename E>
void kk_dynwalk(WalkEngine<E, KKDynWalkState> *graph, walker_id_t walker_num, step_t walk_length,
                WalkConfig *walk_conf)
{
    auto init_walker_func = [&](Walker<KKDynWalkState> &walker, vertex_id_t start_vertex) {
        walker.data.last_vertex = UINT_MAX;
    };
    auto update_walker_func = [&](Walker<KKDynWalkState> &walker, vertex_id_t current_v, AdjUnit<E> *edge) {
        walker.data.last_vertex = current_v;
    };
    WalkerConfig<E, KKDynWalkState> walker_conf(walker_num, init_walker_func, update_walker_func);
    auto extension_comp = [&](Walker<KKDynWalkState> &walker, vertex_id_t current_v) {
        return walker.step >= walk_length ? 0.0 : 1.0;
    };
    auto static_comp = [&](vertex_id_t v, AdjUnit<E> *edge) { return edge->data; };
    auto dynamic_comp = [&](Walker<KKDynWalkState> &walker, vertex_id_t current_v, AdjUnit<E> *edge) {
        if (walker.step == 0)
        {
            return 1.0;
        }
        else if (edge->neighbour == walker.data.last_vertex)
        {
            return 2.0;
        }
        else
        {
            return 1.0;
        }
    };
    auto dynamic_comp_upperbound = [&](vertex_id_t v_id, AdjList<E> *adj_lists) { return 2.0; };
    TransitionConfig<E, KKDynWalkState> tr_conf(extension_comp, static_comp, dynamic_comp, dynamic_comp_upperbound);
    graph->random_walk(&walker_conf, &tr_conf, walk_conf);
}

/* ---- Hooked random_walk ------------------------------------------------
 * Explicit specialisations of WalkEngine::random_walk (include/walk.hpp:423-436)
 * for every (edge, state, transition config) the apps use.  Each one wraps
 * the extension functor (sets the walker's draw context), the init-state
 * functor (value-initialises the walker state, then stream 1) and a custom
 * start-vertex functor (stream 2), then runs the engine unchanged.
 *
 * Value-initialising the state is the one behavioural choice: the reference
 * leaves Walker::data uninitialised (include/walk.hpp:464), and node2vec's
 * step-0 outlier bound reads walker.data.previous_vertex
 * (src/apps/node2vec.hpp:71-78), so an unset state would make weighted
 * node2vec with 1/p > max(1, 1/q) depend on stack contents.  Zero state makes
 * that read the vertex's first edge. */
#ifndef KK_STOCK_RNG
namespace kkhook
{
template <typename S>
inline void zero_state(Walker<S> &w)
{
    memset(&w.data, 0, sizeof(S));
}
template <>
inline void zero_state<EmptyData>(Walker<EmptyData> &)
{
}

template <typename E, typename S, typename TC>
void wrap(WalkerConfig<E, S> *wc, TC *tc)
{
    auto ext = tc->extension_comp_func;
    tc->extension_comp_func = [ext](Walker<S> &w, vertex_id_t v) {
        enter_walk(w.id, w.step);
        return ext(w, v);
    };
    auto init_state = wc->walker_init_state_func;
    wc->walker_init_state_func = [init_state](Walker<S> &w, vertex_id_t v) {
        zero_state<S>(w);
        enter_aux(w.id, KKO_STREAM_INIT_STATE);
        if (init_state != nullptr)
        {
            init_state(w, v);
        }
        leave();
    };
    auto init_dist = wc->walker_init_dist_func;
    if (init_dist != nullptr)
    {
        wc->walker_init_dist_func = [init_dist](walker_id_t id) {
            enter_aux(id, KKO_STREAM_INIT_DIST);
            vertex_id_t v = init_dist(id);
            leave();
            return v;
        };
    }
}
} // namespace kkhook

#define KK_HOOKED_RANDOM_WALK(E, S, TC)                                                                    \
    template <>                                                                                            \
    template <>                                                                                            \
    void WalkEngine<E, S>::random_walk<TC>(WalkerConfig<E, S> * wc, TC * tc, WalkConfig * walk_config_param) \
    {                                                                                                      \
        kkhook::wrap(wc, tc);                                                                              \
        WalkConfig *walk_config = walk_config_param;                                                       \
        if (walk_config == nullptr)                                                                        \
        {                                                                                                  \
            walk_config = new WalkConfig();                                                                \
        }                                                                                                  \
        internal_random_walk_wrap(wc, tc, walk_config);                                                    \
        if (walk_config_param == nullptr)                                                                  \
        {                                                                                                  \
            delete walk_config;                                                                            \
        }                                                                                                  \
    }


typedef TransitionConfig<EmptyData, EmptyData> kk_tc_ue;
typedef TransitionConfig<real_t, EmptyData> kk_tc_we;
typedef SecondOrderTransitionConfig<EmptyData, Node2vecState, vertex_id_t, bool> kk_tc_un2v;
typedef SecondOrderTransitionConfig<real_t, Node2vecState, vertex_id_t, bool> kk_tc_wn2v;
typedef TransitionConfig<UnweightedMetaData, MetapathState> kk_tc_um;
typedef TransitionConfig<WeightedMetaData, MetapathState> kk_tc_wm;
typedef TransitionConfig<KKTag, KKTagState> kk_tc_ut1;
typedef TransitionConfig<KKWeightedTag, KKTagState> kk_tc_wt1;
typedef SecondOrderTransitionConfig<KKTag, KKTagState, EmptyData, int> kk_tc_ut2;
typedef SecondOrderTransitionConfig<KKWeightedTag, KKTagState, EmptyData, int> kk_tc_wt2;
typedef TransitionConfig<real_t, KKDynWalkState> kk_tc_dyn;

KK_HOOKED_RANDOM_WALK(EmptyData, EmptyData, kk_tc_ue)
KK_HOOKED_RANDOM_WALK(real_t, EmptyData, kk_tc_we)
KK_HOOKED_RANDOM_WALK(EmptyData, Node2vecState, kk_tc_un2v)
KK_HOOKED_RANDOM_WALK(real_t, Node2vecState, kk_tc_wn2v)
KK_HOOKED_RANDOM_WALK(UnweightedMetaData, MetapathState, kk_tc_um)
KK_HOOKED_RANDOM_WALK(WeightedMetaData, MetapathState, kk_tc_wm)
KK_HOOKED_RANDOM_WALK(KKTag, KKTagState, kk_tc_ut1)
KK_HOOKED_RANDOM_WALK(KKWeightedTag, KKTagState, kk_tc_wt1)
KK_HOOKED_RANDOM_WALK(KKTag, KKTagState, kk_tc_ut2)
KK_HOOKED_RANDOM_WALK(KKWeightedTag, KKTagState, kk_tc_wt2)
KK_HOOKED_RANDOM_WALK(real_t, KKDynWalkState, kk_tc_dyn)
#else
namespace kkhook
{
static void reset(uint64_t, size_t) {}
} // namespace kkhook
#endif /* KK_STOCK_RNG */

/* ---- CLI ---------------------------------------------------------------- */

struct Args
{
    std::string cmd, graph, kind = "none", out, schemes, dump, variant = "bound", vtag;
    vertex_id_t v = 0;
    uint64_t seed = 1;
    walker_id_t walkers = 0;
    step_t len = 80;
    float term = 1.0f / 80, p = 1, q = 1, vtw = 0.5f, amp = 4.0f;
    double rate = 1.0;
    int threads = 0, order = 1, tag_num = 4, head = 0, time_only = 0, sort_adj = 0;
};

static void usage()
{
    fprintf(stderr, "usage: kk_ref <alias|deepwalk|ppr|node2vec|metapath|tagwalk|dynwalk> --graph F --v V --kind K [opts] --out F\n");
    exit(2);
}

static Args parse(int argc, char **argv)
{
    if (argc < 2)
    {
        usage();
    }
    Args a;
    a.cmd = argv[1];
    for (int i = 2; i < argc; i++)
    {
        std::string k = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc)
            {
                usage();
            }
            return argv[++i];
        };
        if (k == "--graph") a.graph = val();
        else if (k == "--v") a.v = (vertex_id_t)strtoul(val().c_str(), 0, 10);
        else if (k == "--kind") a.kind = val();
        else if (k == "--out") a.out = val();
        else if (k == "--seed") a.seed = strtoull(val().c_str(), 0, 10);
        else if (k == "--walkers") a.walkers = (walker_id_t)strtoul(val().c_str(), 0, 10);
        else if (k == "--len") a.len = (step_t)strtoul(val().c_str(), 0, 10);
        else if (k == "--term") a.term = strtof(val().c_str(), 0);
        else if (k == "--p") a.p = strtof(val().c_str(), 0);
        else if (k == "--q") a.q = strtof(val().c_str(), 0);
        else if (k == "--rate") a.rate = strtod(val().c_str(), 0);
        else if (k == "--threads") a.threads = atoi(val().c_str());
        else if (k == "--schemes") a.schemes = val();
        else if (k == "--dump") a.dump = val();
        else if (k == "--head") a.head = atoi(val().c_str());
        else if (k == "--variant") a.variant = val();
        else if (k == "--order") a.order = atoi(val().c_str());
        else if (k == "--tag-num") a.tag_num = atoi(val().c_str());
        else if (k == "--vtw") a.vtw = strtof(val().c_str(), 0);
        else if (k == "--amp") a.amp = strtof(val().c_str(), 0);
        else if (k == "--vtag") a.vtag = val();
        else if (k == "--time") a.time_only = 1;
        else usage();
    }
    if (a.graph.empty() || a.v == 0)
    {
        usage();
    }
    return a;
}

struct PathSink
{
    std::vector<std::vector<vertex_id_t> > paths;
    void consume(PathSet *ps)
    {
        for (int s = 0; s < ps->seg_num; s++)
        {
            for (walker_id_t i = 0; i < ps->path_num[s]; i++)
            {
                walker_id_t w = ps->walker_id[s][i];
                if (w >= paths.size())
                {
                    paths.resize((size_t)w + 1);
                }
                paths[w].assign(ps->path_begin[s][i], ps->path_begin[s][i] + ps->path_length[s][i]);
            }
        }
        delete ps;
    }
    void write(const std::string &fn, walker_id_t n)
    {
        FILE *f = fopen(fn.c_str(), "wb");
        assert(f != NULL);
        fwrite("KKP1", 1, 4, f);
        fwrite(&n, 4, 1, f);
        paths.resize(n);
        for (walker_id_t w = 0; w < n; w++)
        {
            uint32_t l = (uint32_t)paths[w].size();
            fwrite(&l, 4, 1, f);
        }
        for (walker_id_t w = 0; w < n; w++)
        {
            if (!paths[w].empty())
            {
                fwrite(paths[w].data(), 4, paths[w].size(), f);
            }
        }
        fclose(f);
    }
};

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename E, typename S>
static void setup_engine(WalkEngine<E, S> &g, const Args &a)
{
    if (a.threads > 0)
    {
        g.set_concurrency(a.threads);
    }
    g.load_graph(a.v, a.graph.c_str());
}

static WalkConfig *make_walk_conf(const Args &a, PathSink &sink)
{
    WalkConfig *wc = new WalkConfig();
    if (!a.time_only)
    {
        wc->set_output_consumer([&sink](PathSet *ps) { sink.consume(ps); });
    }
    if (!a.dump.empty())
    {
        wc->set_output_file(a.dump.c_str(), a.head != 0);
    }
    wc->set_walk_rate(a.rate);
    return wc;
}

template <typename E, typename S, typename RUN>
static int run_walk(const Args &a, RUN run)
{
    WalkEngine<E, S> g;
    setup_engine(g, a);
    walker_id_t n = a.walkers ? a.walkers : g.get_vertex_num();
    kkhook::reset(a.seed, n);
    PathSink sink;
    WalkConfig *wc = make_walk_conf(a, sink);
    double t0 = now_s();
    run(g, n, wc);
    double t1 = now_s();
    delete wc;
    if (a.time_only)
    {
        printf("{\"seconds\": %.6f, \"threads\": %d}\n", t1 - t0, g.get_worker_num());
    }
    else
    {
        sink.write(a.out, n);
    }
    return 0;
}

template <typename E>
static int run_alias(const Args &a)
{
    WalkEngine<E, EmptyData> g;
    setup_engine(g, a);
    vertex_id_t V = g.get_vertex_num();
    edge_id_t E_num = g.get_edge_num();
    std::vector<real_t> sum(V, 0.0f);
    AliasTableContainer<E> *tables = nullptr;
    auto static_comp = get_trivial_static_comp(&g);
    g.init_alias_tables(static_comp, tables, sum.data());
    std::vector<float> p(E_num);
    std::vector<uint32_t> pi(E_num), qi(E_num);
    for (vertex_id_t v = 0; v < V; v++)
    {
        AdjUnit<E> *begin = g.csr->adj_lists[v].begin;
        edge_id_t base = (edge_id_t)(tables->index[v] - tables->buckets);
        for (vertex_id_t j = 0; j < g.vertex_out_degree[v]; j++)
        {
            AliasBucket<E> &b = tables->index[v][j];
            p[base + j] = b.p;
            pi[base + j] = (uint32_t)(b.p_ptr - begin);
            qi[base + j] = b.q_ptr == nullptr ? 0xffffffffu : (uint32_t)(b.q_ptr - begin);
        }
    }
    g.free_alias_tables(tables);
    FILE *f = fopen(a.out.c_str(), "wb");
    assert(f != NULL);
    fwrite("KKA1", 1, 4, f);
    fwrite(&V, 4, 1, f);
    uint64_t e64 = E_num;
    fwrite(&e64, 8, 1, f);
    fwrite(p.data(), 4, E_num, f);
    fwrite(pi.data(), 4, E_num, f);
    fwrite(qi.data(), 4, E_num, f);
    fwrite(sum.data(), 4, V, f);
    fclose(f);
    return 0;
}

static std::vector<int> read_vtag(const Args &a)
{
    std::vector<int> t(a.v, 0);
    FILE *f = fopen(a.vtag.c_str(), "rb");
    assert(f != NULL);
    size_t r = fread(t.data(), 4, a.v, f);
    assert(r == a.v);
    fclose(f);
    return t;
}

template <typename E>
static int run_tagwalk(const Args &a)
{
    std::vector<int> vtag = read_vtag(a);
    return run_walk<E, KKTagState>(a, [&](WalkEngine<E, KKTagState> &g, walker_id_t n, WalkConfig *wc) {
        KKTagConf conf;
        conf.walker_num = n;
        conf.walk_length = a.len;
        conf.tag_num = a.tag_num;
        conf.vertex_tag_weight = a.vtw;
        conf.outlier_amplifier = a.amp;
        kk_tagwalk(&g, conf, vtag, a.order, a.variant == "outlier", wc);
    });
}

int main(int argc, char **argv)
{
    Args a = parse(argc, argv);
    const std::string &k = a.kind;
    if (a.cmd == "alias")
    {
        if (k == "f32") return run_alias<real_t>(a);
        usage();
    }
    if (a.cmd == "deepwalk" || a.cmd == "ppr")
    {
        bool dw = a.cmd == "deepwalk";
        if (k == "none")
            return run_walk<EmptyData, EmptyData>(a, [&](WalkEngine<EmptyData, EmptyData> &g, walker_id_t n, WalkConfig *wc) {
                if (dw) deepwalk(&g, n, a.len, wc);
                else ppr(&g, n, a.term, nullptr, wc);
            });
        if (k == "f32")
            return run_walk<real_t, EmptyData>(a, [&](WalkEngine<real_t, EmptyData> &g, walker_id_t n, WalkConfig *wc) {
                if (dw) deepwalk(&g, n, a.len, wc);
                else ppr(&g, n, a.term, nullptr, wc);
            });
        usage();
    }
    if (a.cmd == "node2vec")
    {
        if (k == "none")
            return run_walk<EmptyData, Node2vecState>(a, [&](WalkEngine<EmptyData, Node2vecState> &g, walker_id_t n, WalkConfig *wc) {
                Node2vecConf c;
                c.p = a.p;
                c.q = a.q;
                c.walker_num = n;
                c.walk_length = a.len;
                node2vec(&g, c, wc);
            });
        if (k == "f32")
            return run_walk<real_t, Node2vecState>(a, [&](WalkEngine<real_t, Node2vecState> &g, walker_id_t n, WalkConfig *wc) {
                Node2vecConf c;
                c.p = a.p;
                c.q = a.q;
                c.walker_num = n;
                c.walk_length = a.len;
                node2vec(&g, c, wc);
            });
        usage();
    }
    if (a.cmd == "metapath")
    {
        auto schemes = read_metapath_schemes(a.schemes.c_str());
        if (k == "meta")
            return run_walk<UnweightedMetaData, MetapathState>(a, [&](WalkEngine<UnweightedMetaData, MetapathState> &g, walker_id_t n, WalkConfig *wc) {
                metapath(&g, schemes, n, a.len, wc);
            });
        if (k == "meta_f32")
            return run_walk<WeightedMetaData, MetapathState>(a, [&](WalkEngine<WeightedMetaData, MetapathState> &g, walker_id_t n, WalkConfig *wc) {
                metapath(&g, schemes, n, a.len, wc);
            });
        usage();
    }
    if (a.cmd == "dynwalk")
    {
        if (k == "f32")
            return run_walk<real_t, KKDynWalkState>(a, [&](WalkEngine<real_t, KKDynWalkState> &g, walker_id_t n, WalkConfig *wc) {
                kk_dynwalk<real_t>(&g, n, a.len, wc);
            });
        usage();
    }
    if (a.cmd == "tagwalk")
    {
        if (k == "tag") return run_tagwalk<KKTag>(a);
        if (k == "tag_f32") return run_tagwalk<KKWeightedTag>(a);
        usage();
    }
    usage();
    return 2;
}
