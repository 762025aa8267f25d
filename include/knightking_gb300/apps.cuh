/*
 * Built-in apps: the reference's src/apps functors as __device__ functors.
 * Each functor restates one lambda of the reference, with its arithmetic.
 */
#pragma once

#include <type_traits>

#include "walk.cuh"

namespace kk
{
namespace apps
{

/* ---- shared ---------------------------------------------------------------- */

/* walker.step >= walk_length ? 0 : 1 (deepwalk.hpp:36-38, node2vec.hpp:145-148) */
template <typename S>
struct FixedLengthExt
{
    step_t walk_length;
    __device__ __forceinline__ real_t operator()(const Walker<S> &w, vertex_id_t) const
    {
        return w.step >= walk_length ? 0.0f : 1.0f;
    }
};

/* get_trivial_static_comp for weighted graphs: the edge weight (static_comp.hpp:36-42) */
struct WeightStatic
{
    const float *w;
    __device__ __forceinline__ real_t operator()(vertex_id_t, const AdjUnit &e) const { return w[e.index]; }
};

struct ConstBound
{
    real_t value;
    __device__ __forceinline__ real_t operator()(vertex_id_t, const AdjList &) const { return value; }
};

/* ---- PPR (ppr.hpp:30-64) -------------------------------------------------- */

/* extension = 1 - terminate_prob, computed in float (ppr.hpp:35) */
struct ConstantExt
{
    real_t ext;
    __device__ __forceinline__ real_t operator()(const Walker<EmptyData> &, vertex_id_t) const { return ext; }
};

/* ---- node2vec (node2vec.hpp:30-202) --------------------------------------- */

struct Node2vecState
{
    vertex_id_t previous_vertex;
};

/* std::lower_bound over a sorted adjacency; returns a local index (deg if none). */
__device__ __forceinline__ uint32_t lower_bound_adj(const uint32_t *nbr, edge_id_t b, uint32_t deg, vertex_id_t x)
{
    uint32_t lo = 0, hi = deg;
    while (lo < hi)
    {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (gather(nbr + b + mid) < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* update: previous_vertex = current (node2vec.hpp:129-136) */
struct Node2vecUpdate
{
    static constexpr bool reads_edge_index = false;
    __device__ __forceinline__ void operator()(Walker<Node2vecState> &w, vertex_id_t cur, const AdjUnit &) const
    {
        w.data.previous_vertex = cur;
    }
};

/* post_query: from step 1 on, ask the previous vertex about the candidate (node2vec.hpp:150-158) */
struct Node2vecPostQuery
{
    static constexpr bool reads_edge_index = false;
    /* min(1, 1/q) as floats: a dart at or below it is accepted whether the
     * candidate is a neighbour of the previous vertex (dynamic component 1)
     * or not (1/q) */
    real_t sure_below = 0.0f;
    __device__ __forceinline__ bool operator()(const Walker<Node2vecState> &w, vertex_id_t, const AdjUnit &cand,
                                               vertex_id_t &target, vertex_id_t &query) const
    {
        if (w.step == 0)
            return false;
        target = w.data.previous_vertex;
        query = cand.neighbour;
        return true;
    }
    /* Whether the answer can change the trial's outcome: not for the return
     * edge (its dynamic component is 1/p either way), nor for a dart at or
     * below sure_below.  The reference asks in both cases (node2vec.hpp:150-
     * 158); skipping the question leaves every decision, and so every path,
     * as it is. */
    __device__ __forceinline__ bool query_matters(const Walker<Node2vecState> &w, const AdjUnit &cand,
                                                  real_t dart) const
    {
        return !(w.data.previous_vertex == cand.neighbour || dart <= sure_below);
    }
};

/* respond_query: whether the candidate is in N(previous), the result of
 * node2vec.hpp:159-166's std::binary_search over the sorted adjacency; looked
 * up in the edge set when the engine has one (same answer, one sector). */
struct Node2vecRespond
{
    const uint32_t *nbr;
    EdgeSetView set;
    __device__ __forceinline__ bool needs_adjacency() const { return set.keys == nullptr; }
    __device__ __forceinline__ void operator()(vertex_id_t target, const vertex_id_t &query, const AdjList &adj,
                                               bool &resp) const
    {
        if (set.keys != nullptr)
        {
            resp = edge_set_slot(set, target, query) != ~0ull;
            return;
        }
        uint32_t deg = adj.degree();
        uint32_t i = lower_bound_adj(nbr, adj.begin, deg, query);
        resp = i < deg && gather(nbr + adj.begin + i) == query;
    }
};

/* dynamic_comp (node2vec.hpp:167-185): ub at step 0, 1/p back to the previous
 * vertex, 1 to a common neighbour, 1/q otherwise (float divisions of the
 * float parameters). */
struct Node2vecDyn
{
    static constexpr bool reads_edge_index = false;
    real_t upperbound, inv_p, inv_q;
    __device__ __forceinline__ real_t operator()(const Walker<Node2vecState> &w, const bool &resp, vertex_id_t,
                                                 const AdjUnit &e) const
    {
        if (w.step == 0)
            return upperbound;
        if (w.data.previous_vertex == e.neighbour)
            return inv_p;
        if (resp)
            return 1.0f;
        return inv_q;
    }
};

/* outlier_upperbound (node2vec.hpp:47-83): area overflow (unweighted) or
 * overflow * w(return edge) (weighted), one outlier.  Where the previous
 * vertex is not a neighbour (directed graphs) the reference reads past the
 * adjacency; here the area is empty. */
/* The return edge std::lower_bound(N(v), x) of node2vec.hpp:71-78 / :91-97:
 * its local index i (deg if none) and, when want_weight, its weight.  x = 0
 * (the value-initialised state of step 0) is at or below every neighbour, so
 * its position is 0 with no lookup; a neighbour x comes from the edge set,
 * index and weight in one access; anything else by binary search. */
__device__ __forceinline__ uint32_t n2v_return_edge(const uint32_t *nbr, const float *w, const EdgeSetView &set,
                                                    vertex_id_t v, const AdjList &adj, vertex_id_t x, bool want_weight,
                                                    float &weight, bool &is_x)
{
    const uint32_t deg = adj.degree();
    uint32_t i;
    is_x = false;
    if (x == 0)
    {
        i = 0;
    }
    else
    {
        if (set.keys != nullptr)
        {
            uint32_t pos;
            if (edge_set_find(set, v, x, pos, weight))
            {
                is_x = true; /* the edge at pos leads to x */
                return pos;
            }
        }
        i = lower_bound_adj(nbr, adj.begin, deg, x);
    }
    if (want_weight && i < deg)
        weight = gather(w + adj.begin + i);
    return i;
}

template <bool Weighted>
struct Node2vecOutlierUB
{
    const uint32_t *nbr;
    const float *w;
    real_t overflow;
    EdgeSetView set;
    __device__ __forceinline__ void operator()(const Walker<Node2vecState> &wk, vertex_id_t v, const AdjList &adj,
                                               real_t &area, vertex_id_t &num) const
    {
        num = 1;
        if constexpr (Weighted)
        {
            /* a non-positive overflow gives a non-positive area whatever the
             * return edge's weight: the appendix is skipped without the search */
            if (!(overflow > 0.0f))
            {
                area = overflow;
                return;
            }
            float rw = 0.0f;
            bool is_x;
            const uint32_t i = n2v_return_edge(nbr, w, set, v, adj, wk.data.previous_vertex, true, rw, is_x);
            area = i < adj.degree() ? fmul(rw, overflow) : 0.0f;
        }
        else
        {
            area = overflow;
        }
    }
};

/* outlier_search: the return edge, std::lower_bound(N(v), previous) (node2vec.hpp:85-102) */
struct Node2vecOutlierSearch
{
    const uint32_t *nbr;
    EdgeSetView set;
    __device__ __forceinline__ bool operator()(const Walker<Node2vecState> &wk, vertex_id_t v, const AdjList &adj,
                                               vertex_id_t, AdjUnit &out) const
    {
        float unused = 0.0f;
        bool is_x;
        const vertex_id_t x = wk.data.previous_vertex;
        const uint32_t i = n2v_return_edge(nbr, nullptr, set, v, adj, x, false, unused, is_x);
        if (i >= adj.degree())
            return false;
        out = AdjUnit{is_x ? x : gather(nbr + adj.begin + i), adj.begin + i};
        return true;
    }
};

/* Host-side constants, double then float as node2vec.hpp:126-139 computes them. */
struct Node2vecConstants
{
    float upperbound, lowerbound, overflow, inv_p, inv_q;
    bool outlier;
    static Node2vecConstants make(float p, float q)
    {
        Node2vecConstants c;
        double ip = 1.0 / (double)p, iq = 1.0 / (double)q;
        c.upperbound = (float)(iq > 1.0 ? iq : 1.0);
        double m = iq < 1.0 ? iq : 1.0;
        c.lowerbound = (float)(ip < m ? ip : m);
        c.overflow = (float)(ip - (double)c.upperbound);
        c.inv_p = 1.0f / p;
        c.inv_q = 1.0f / q;
        c.outlier = c.overflow > 0.0f;
        return c;
    }
};

/* ---- metapath (metapath.hpp:32-128, metascheme.hpp:36-54) ------------------ */

struct MetapathState
{
    int scheme_id;
    int state;
};

struct MetaSchemes
{
    uint8_t mask[16][16]; /* scheme x state -> allowed edge types (bit t) */
    uint8_t len[16];
    uint32_t n;
};

/* The hooks read their job's schemes from device memory (a batch gives each
 * job its own set). */

/* extension: 0 at the length or when no out-edge has an allowed type (metapath.hpp:102-105) */
struct MetapathExt
{
    const uint8_t *vertex_mask;
    step_t walk_length;
    const MetaSchemes *sc;
    __device__ __forceinline__ real_t operator()(const Walker<MetapathState> &w, vertex_id_t v) const
    {
        return (w.step >= walk_length || !(gather(vertex_mask + v) & sc->mask[w.data.scheme_id][w.data.state])) ? 0.0f
                                                                                                            : 1.0f;
    }
};

/* dynamic_comp: 1 if the edge's type is allowed in the current state, else 0 (metapath.hpp:107-116) */
struct MetapathDyn
{
    /* the type comes from the bucket's tag (index and neighbour buckets carry
     * it); the edge index is read only where no tag is held */
    static constexpr bool reads_edge_index = false;
    static constexpr bool needs_type_tag = true;
    const uint8_t *type;
    const MetaSchemes *sc;
    __device__ __forceinline__ real_t operator()(const Walker<MetapathState> &w, vertex_id_t, const AdjUnit &e) const
    {
        const uint32_t t = (e.type_tag & 0x100u) ? (e.type_tag & 0xffu) : gather(type + e.index);
        return ((sc->mask[w.data.scheme_id][w.data.state] >> t) & 1u) ? 1.0f : 0.0f;
    }
};

/* init_state: scheme = gen(#schemes) (metapath.hpp:91-95) or round robin; state 0 */
struct MetapathInitState
{
    const MetaSchemes *sc;
    int round_robin;
    __device__ __forceinline__ void operator()(Walker<MetapathState> &w, vertex_id_t, Sampler &rng) const
    {
        const uint32_t n = sc->n;
        w.data.scheme_id = round_robin ? (int)(w.id % n) : (int)rng.gen(n);
        w.data.state = 0;
    }
};

/* update: state = (state + 1) % len(scheme) (metapath.hpp:96-99) */
struct MetapathUpdate
{
    static constexpr bool reads_edge_index = false;
    const MetaSchemes *sc;
    __device__ __forceinline__ void operator()(Walker<MetapathState> &w, vertex_id_t, const AdjUnit &) const
    {
        w.data.state = (w.data.state + 1) % (int)sc->len[w.data.scheme_id];
    }
};

/* vertex_masks (metapath.hpp:77-88): OR of 1 << type over the out-edges */
static __global__ void metapath_vertex_mask_kernel(GraphView g, uint8_t *vmask)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x)
    {
        uint8_t m = 0;
        for (int64_t e = g.off[v]; e < g.off[v + 1]; e++)
            m |= (uint8_t)(1u << g.type[e]);
        vmask[v] = m;
    }
}

/* ---- batch builders: one job's hooks from its BatchJob row ---------------- */

template <bool Weighted>
struct DeepWalkBatch
{
    typedef EmptyData S;
    typedef WalkerConfig<EmptyData> WC;
    typedef TransitionConfig<EmptyData, FixedLengthExt<EmptyData>,
                             typename std::conditional<Weighted, WeightStatic, NoHook>::type>
        TC;
    const float *w;
    __device__ __forceinline__ void make(const BatchJob &j, WC &wc, TC &tc) const
    {
        wc.walker_num = j.walker_num;
        tc.extension_comp = FixedLengthExt<EmptyData>{j.walk_length};
        if constexpr (Weighted)
            tc.static_comp = WeightStatic{w};
    }
};

/* Every node2vec job uses the outlier-capable hooks: a job whose overflow
 * 1/p - max(1, 1/q) is not positive gets an outlier area <= 0, so the
 * area > 0 test skips the appendix and draws nothing, exactly as the
 * reference does without the outlier hooks (src/apps/node2vec.hpp:137-139). */
template <bool Weighted>
struct Node2vecBatch
{
    typedef Node2vecState S;
    typedef WalkerConfig<Node2vecState, NoHook, NoHook, Node2vecUpdate> WC;
    typedef SecondOrderTransitionConfig<Node2vecState, vertex_id_t, bool, FixedLengthExt<Node2vecState>,
                                        typename std::conditional<Weighted, WeightStatic, NoHook>::type,
                                        Node2vecPostQuery, Node2vecRespond, Node2vecDyn, ConstBound, ConstBound,
                                        Node2vecOutlierUB<Weighted>, Node2vecOutlierSearch>
        TC;
    const uint32_t *nbr;
    const float *w;
    EdgeSetView set;
    __device__ __forceinline__ void make(const BatchJob &j, WC &wc, TC &tc) const
    {
        wc.walker_num = j.walker_num;
        tc.extension_comp = FixedLengthExt<Node2vecState>{j.walk_length};
        if constexpr (Weighted)
            tc.static_comp = WeightStatic{w};
        tc.post_query = Node2vecPostQuery{j.c[4] < 1.0f ? j.c[4] : 1.0f};
        tc.respond_query = Node2vecRespond{nbr, set};
        tc.dynamic_comp = Node2vecDyn{j.c[0], j.c[3], j.c[4]};
        tc.dcomp_upperbound = ConstBound{j.c[0]};
        tc.dcomp_lowerbound = ConstBound{j.c[1]};
        tc.outlier_upperbound = Node2vecOutlierUB<Weighted>{nbr, w, j.c[2], set};
        tc.outlier_search = Node2vecOutlierSearch{nbr, set};
    }
};

template <bool Weighted>
struct MetapathBatch
{
    typedef MetapathState S;
    typedef WalkerConfig<MetapathState, NoHook, MetapathInitState, MetapathUpdate> WC;
    typedef TransitionConfig<MetapathState, MetapathExt,
                             typename std::conditional<Weighted, WeightStatic, NoHook>::type, MetapathDyn, ConstBound>
        TC;
    const uint8_t *vmask;
    const uint8_t *type;
    const float *w;
    __device__ __forceinline__ void make(const BatchJob &j, WC &wc, TC &tc) const
    {
        const MetaSchemes *sc = (const MetaSchemes *)j.param;
        wc.walker_num = j.walker_num;
        wc.walker_init_state = MetapathInitState{sc, j.flag};
        wc.walker_update_state = MetapathUpdate{sc};
        tc.extension_comp = MetapathExt{vmask, j.walk_length, sc};
        if constexpr (Weighted)
            tc.static_comp = WeightStatic{w};
        tc.dynamic_comp = MetapathDyn{type, sc};
        tc.dcomp_upperbound = ConstBound{1.0f};
    }
};

} // namespace apps
} // namespace kk
