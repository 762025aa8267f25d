/*
 * The reference's C++ classes over this engine, so that a KnightKing program
 * moves over by changing its includes and turning its lambdas into __device__
 * functors:
 *
 *   WalkEngine<E, S>  WalkEngine (include/walk.hpp:365-436) with GraphEngine's
 *                     load_graph (include/graph.hpp:408-530), set_concurrency,
 *                     get_vertex_num / get_edge_num and random_walk;
 *   WalkConfig        WalkConfig (include/walk.hpp:105-145): output file,
 *                     output consumer, walk rate (epochs);
 *   PathSet           PathSet (include/path.hpp:46-109): the paths of one
 *                     epoch in segments of the reference's layout, handed to
 *                     the output consumer, which owns it.
 *
 * WalkerConfig, TransitionConfig and SecondOrderTransitionConfig are the
 * functor-typed configs of walk.cuh; make_walker_config and
 * make_transition_config build them in the argument order of the reference's
 * constructors (include/walk.hpp:147-271).
 *
 * Differences a ported program sees:
 *   - hooks are __device__ functors; edge data is read through the device
 *     arrays the engine exposes (edge_weights(), edge_types(), neighbours(),
 *     offsets()) by the AdjUnit's global edge index, where the reference's
 *     lambdas dereference edge->data;
 *   - draws come from the counter-based Philox stream keyed by set_seed()'s
 *     seed (default 1) and the walker id, not from per-thread mt19937s, so
 *     paths do not depend on the thread count;
 *   - each walker's path has a fixed capacity on the device: the extension
 *     functor's walk_length member when it has one, else the engine's
 *     set_max_walk_length() (default 80); a longer walk fails the call;
 *   - failures throw kk::Error (the reference asserts or exits).
 * set_concurrency() keeps its meaning for the output: the number of segments
 * a PathSet holds and the order in which dumps write walkers.
 */
#pragma once

#include <stdio.h>

#include <functional>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "knightking_gb300.h"
#include "knightking_gb300/engine.cuh"

namespace kk
{

/* include/graph.hpp:123-127 */
enum GraphFormat
{
    GF_Binary,
    GF_Edgelist
};

/* The binary Edge<E> record kind of an edge data type (include/type.hpp:43-85):
 * EmptyData and real_t; specialise for other data types with a KK_EDGE_*
 * layout. */
template <typename E>
struct edge_kind;
template <>
struct edge_kind<EmptyData>
{
    static constexpr int value = KK_EDGE_UNWEIGHTED;
    static constexpr bool weighted = false;
};
template <>
struct edge_kind<real_t>
{
    static constexpr int value = KK_EDGE_F32;
    static constexpr bool weighted = true;
};

/* PathSet (include/path.hpp:46-109): seg_num segments; segment s holds
 * path_num[s] walkers, walker_id[s][i] with path_length[s][i] vertices at
 * path_begin[s][i] .. path_end[s][i] inside path_set[s]. */
struct PathSet
{
    int seg_num = 0;
    vertex_id_t **path_set = nullptr;
    walker_id_t **walker_id = nullptr;
    vertex_id_t ***path_begin = nullptr;
    vertex_id_t ***path_end = nullptr;
    step_t **path_length = nullptr;
    walker_id_t *path_num = nullptr;

    PathSet() = default;
    PathSet(const PathSet &) = delete;
    PathSet &operator=(const PathSet &) = delete;
    ~PathSet()
    {
        for (int s = 0; s < seg_num; s++)
        {
            delete[] path_set[s];
            delete[] walker_id[s];
            delete[] path_begin[s];
            delete[] path_end[s];
            delete[] path_length[s];
        }
        delete[] path_set;
        delete[] walker_id;
        delete[] path_begin;
        delete[] path_end;
        delete[] path_length;
        delete[] path_num;
    }

    /* The walkers [eb, eb + en) of p in seg_num segments, the reference's
     * segment order: segment t holds walkers eb + t, eb + t + seg_num, ...
     * (include/path.hpp:383-441). */
    static PathSet *from_epoch(const kk_paths *p, uint32_t eb, uint32_t en, int seg_num)
    {
        PathSet *ps = new PathSet();
        ps->seg_num = seg_num;
        ps->path_set = new vertex_id_t *[seg_num];
        ps->walker_id = new walker_id_t *[seg_num];
        ps->path_begin = new vertex_id_t **[seg_num];
        ps->path_end = new vertex_id_t **[seg_num];
        ps->path_length = new step_t *[seg_num];
        ps->path_num = new walker_id_t[seg_num];
        for (int t = 0; t < seg_num; t++)
        {
            const uint32_t n = en > (uint32_t)t ? (en - (uint32_t)t + (uint32_t)seg_num - 1) / (uint32_t)seg_num : 0;
            uint64_t total = 0;
            for (uint32_t k = 0; k < n; k++)
                total += p->length[eb + (uint32_t)t + k * (uint32_t)seg_num];
            ps->path_num[t] = n;
            ps->path_set[t] = new vertex_id_t[total > 0 ? total : 1];
            ps->walker_id[t] = new walker_id_t[n > 0 ? n : 1];
            ps->path_begin[t] = new vertex_id_t *[n > 0 ? n : 1];
            ps->path_end[t] = new vertex_id_t *[n > 0 ? n : 1];
            ps->path_length[t] = new step_t[n > 0 ? n : 1];
            uint64_t at = 0;
            for (uint32_t k = 0; k < n; k++)
            {
                const uint32_t w = eb + (uint32_t)t + k * (uint32_t)seg_num;
                const uint32_t len = p->length[w];
                const uint32_t *src = p->vertices + p->offset[w];
                for (uint32_t j = 0; j < len; j++)
                    ps->path_set[t][at + j] = src[j];
                ps->walker_id[t][k] = p->walker_begin + w;
                ps->path_length[t][k] = len;
                ps->path_begin[t][k] = ps->path_set[t] + at;
                ps->path_end[t][k] = ps->path_set[t] + at + len;
                at += len;
            }
        }
        return ps;
    }

    /* PathSet::dump (include/path.hpp:85-109) */
    void dump(const char *output_path, const char *fopen_mode, bool with_head_info) const
    {
        FILE *f = fopen(output_path, fopen_mode);
        if (f == nullptr)
            fail(KK_ERR_IO, std::string("cannot open ") + output_path);
        for (int s = 0; s < seg_num; s++)
            for (walker_id_t i = 0; i < path_num[s]; i++)
            {
                if (with_head_info)
                    fprintf(f, "%u %u", walker_id[s][i], path_length[s][i]);
                for (step_t k = 0; k < path_length[s][i]; k++)
                    fprintf(f, " %u", path_begin[s][i][k]);
                fprintf(f, "\n");
            }
        fclose(f);
    }
};

/* WalkConfig (include/walk.hpp:105-145) */
class WalkConfig
{
  public:
    bool output_file_flag = false;
    std::string output_path_prefix;
    bool print_with_head_info = false;
    bool output_consumer_flag = false;
    std::function<void(PathSet *)> output_consumer_func = nullptr;
    double rate = 1;

    void set_output_file(const char *output_path_prefix_param, bool with_head_info = false)
    {
        if (output_path_prefix_param == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "output_path_prefix is null");
        output_file_flag = true;
        output_path_prefix = output_path_prefix_param;
        print_with_head_info = with_head_info;
    }

    void set_output_consumer(std::function<void(PathSet *)> output_consumer_func_param)
    {
        if (output_consumer_func_param == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "output consumer is null");
        output_consumer_flag = true;
        output_consumer_func = output_consumer_func_param;
    }

    void set_walk_rate(double rate_param)
    {
        if (!(rate_param > 0 && rate_param <= 1))
            fail(KK_ERR_INVALID_CONFIG, "rate must be in (0, 1]");
        rate = rate_param;
    }
};

/* WalkerConfig in the argument order of the reference's constructor
 * (include/walk.hpp:155-171): walker count, init state, update state, start
 * distribution; NoHook{} for a nullptr. */
template <typename S, typename InitState = NoHook, typename Update = NoHook, typename InitDist = NoHook>
WalkerConfig<S, InitDist, InitState, Update> make_walker_config(walker_id_t walker_num, InitState init_state = {},
                                                                Update update = {}, InitDist init_dist = {})
{
    WalkerConfig<S, InitDist, InitState, Update> wc;
    wc.walker_num = walker_num;
    wc.walker_init_dist = init_dist;
    wc.walker_init_state = init_state;
    wc.walker_update_state = update;
    return wc;
}

/* TransitionConfig in the argument order of the reference's constructor
 * (include/walk.hpp:227-249). */
template <typename S, typename Ext, typename Static = NoHook, typename Dyn = NoHook, typename UB = NoHook,
          typename LB = NoHook, typename OutUB = NoHook, typename OutSearch = NoHook>
TransitionConfig<S, Ext, Static, Dyn, UB, LB, OutUB, OutSearch>
make_transition_config(Ext extension_comp, Static static_comp = {}, Dyn dynamic_comp = {}, UB upperbound = {},
                       LB lowerbound = {}, OutUB outlier_upperbound = {}, OutSearch outlier_search = {})
{
    TransitionConfig<S, Ext, Static, Dyn, UB, LB, OutUB, OutSearch> tc;
    tc.extension_comp = extension_comp;
    tc.static_comp = static_comp;
    tc.dynamic_comp = dynamic_comp;
    tc.dcomp_upperbound = upperbound;
    tc.dcomp_lowerbound = lowerbound;
    tc.outlier_upperbound = outlier_upperbound;
    tc.outlier_search = outlier_search;
    return tc;
}

/* Whether a functor declares the walk length it stops at (a walk_length member). */
template <typename F, typename = void>
struct has_walk_length : std::false_type
{
};
template <typename F>
struct has_walk_length<F, std::void_t<decltype(std::declval<const F &>().walk_length)>> : std::true_type
{
};

/* WalkEngine<edge data, walker state> (include/walk.hpp:365-436) on one CUDA
 * device; owns its kk_engine. */
template <typename E, typename S>
class WalkEngine
{
  public:
    explicit WalkEngine(int device = 0)
    {
        kk_status st = kk_engine_create(&e_, device);
        if (st != KK_OK)
            fail(st, "cannot create the engine");
    }
    ~WalkEngine()
    {
        if (e_)
            kk_engine_destroy(e_);
    }
    WalkEngine(const WalkEngine &) = delete;
    WalkEngine &operator=(const WalkEngine &) = delete;

    /* set_concurrency (include/walk.hpp:391-397): the segment count of the
     * output (PathSet segments, dump order); the GPU needs no thread count */
    void set_concurrency(int worker_num_param) { worker_num_ = worker_num_param > 0 ? worker_num_param : 1; }
    int get_worker_num() const { return worker_num_; }

    /* load_graph (include/graph.hpp:408-530) */
    void load_graph(vertex_id_t v_num_param, const char *graph_path, bool load_as_undirected = false,
                    GraphFormat graph_format = GF_Binary)
    {
        kk_status st = graph_format == GF_Binary
                           ? kk_graph_load_binary(e_, v_num_param, graph_path, edge_kind<E>::value, load_as_undirected)
                           : kk_graph_load_text(e_, v_num_param, graph_path, edge_kind<E>::weighted,
                                                load_as_undirected);
        check(st);
    }

    vertex_id_t get_vertex_num() const { return e_->V; }
    edge_id_t get_edge_num() const { return e_->E; }

    /* device arrays of the graph, for the hooks: per edge index (AdjUnit::index) */
    const float *edge_weights() const { return e_->d_w; }
    const uint8_t *edge_types() const { return e_->d_type; }
    const uint32_t *neighbours() const { return e_->d_nbr; }
    const int64_t *offsets() const { return e_->d_off; }

    /* the Philox key of the walks' random stream */
    void set_seed(uint64_t seed) { seed_ = seed; }
    /* the path capacity of walks whose extension functor declares no walk_length */
    void set_max_walk_length(step_t steps) { max_walk_length_ = steps; }

    /* random_walk (include/walk.hpp:423-436, :698-878): walks walker_conf's
     * walkers with the transition config's hooks, in epochs of the walk
     * config's rate; each epoch's paths go to the output file (prefix ".0",
     * "w" then "a", include/walk.hpp:826-842) and to the output consumer as
     * a PathSet it owns. */
    template <typename WC, typename TC>
    void random_walk(WC *walker_config, TC *transition_config, WalkConfig *walk_config_param = nullptr)
    {
        static_assert(std::is_same<typename WC::state_type, S>::value, "the walker state is the engine's");
        static_assert(std::is_same<typename TC::state_type, S>::value, "the walker state is the engine's");
        WalkConfig fallback;
        const WalkConfig &wcfg = walk_config_param ? *walk_config_param : fallback;
        kk_walk_opts o{};
        o.app = KK_APP_DEEPWALK; /* not read for user hooks */
        o.weighted = TC::has_static ? 1 : 0;
        o.seed = seed_;
        o.walker_num = walker_config->walker_num;
        o.walker_begin = 0;
        if constexpr (has_walk_length<decltype(transition_config->extension_comp)>::value)
            o.walk_length = transition_config->extension_comp.walk_length;
        else
            o.walk_length = max_walk_length_;
        o.rate = wcfg.rate;
        kk_paths *p = nullptr;
        check(kk::random_walk<S>(e_, *walker_config, *transition_config, o, &p));
        try
        {
            if (wcfg.output_file_flag)
                check(kk_paths_dump(p, (wcfg.output_path_prefix + ".0").c_str(), "w",
                                    wcfg.print_with_head_info ? 1 : 0, worker_num_));
            if (wcfg.output_consumer_flag)
            {
                const uint32_t per = p->epoch_walkers ? p->epoch_walkers : p->walker_num;
                for (uint32_t eb = 0; eb < p->walker_num; eb += per)
                {
                    const uint32_t en = p->walker_num - eb < per ? p->walker_num - eb : per;
                    wcfg.output_consumer_func(PathSet::from_epoch(p, eb, en, worker_num_));
                }
            }
        }
        catch (...)
        {
            kk_paths_free(p);
            throw;
        }
        kk_paths_free(p);
    }

    kk_engine *handle() { return e_; }

  private:
    void check(kk_status st)
    {
        if (st != KK_OK)
            fail(st, kk_last_error(e_));
    }

    kk_engine *e_ = nullptr;
    int worker_num_ = 1;
    uint64_t seed_ = 1;
    step_t max_walk_length_ = 80;
};

} // namespace kk
