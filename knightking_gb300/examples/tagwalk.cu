/*
 * Example of the plugin API: tag walks with user-defined hooks.
 *
 * The bound and outlier tag walks of the reference's tests
 * (src/tests/test_bound.cpp:105-193, src/tests/test_outlier.cpp:105-252),
 * written as __device__ functors for TransitionConfig /
 * SecondOrderTransitionConfig and run with kk::random_walk.  Every edge has a
 * tag (the graph's edge type) and every vertex a tag; a walker carries a tag
 * that advances by one per step.  The bound form uses a per-vertex lower and
 * upper bound of the dynamic component; the outlier form amplifies edges whose
 * tag equals the walker's and moves them into the outlier appendix (adjacency
 * grouped by edge tag).  Second order asks the previous vertex for its tag
 * through post_query / respond_query.
 *
 * Built into knightking_gb300/lib/libkk_example_tagwalk.so next to the engine.
 */
#include <stdlib.h>

#include <type_traits>
#include <vector>

#include "knightking_gb300/engine.cuh"

namespace
{
using namespace kk;

struct TagState
{
    int tag;
    vertex_id_t previous_vertex;
};

struct TagExt
{
    step_t walk_length;
    __device__ real_t operator()(const Walker<TagState> &w, vertex_id_t) const
    {
        return w.step >= walk_length ? 0.0f : 1.0f;
    }
};

/* bound form: ub = T + vtag * vtw, lb = vtag * vtw (test_bound.cpp:136-143) */
struct TagUB
{
    const int *vtag;
    int T;
    float vtw;
    __device__ real_t operator()(vertex_id_t v, const AdjList &) const
    {
        return fadd((float)T, fmul((float)vtag[v], vtw));
    }
};

struct TagLB
{
    const int *vtag;
    float vtw;
    __device__ real_t operator()(vertex_id_t v, const AdjList &) const { return fmul((float)vtag[v], vtw); }
};

struct TagConst
{
    real_t value;
    __device__ real_t operator()(vertex_id_t, const AdjList &) const { return value; }
};

/* 1 + (tag of the previous vertex + walker tag + edge tag) % T, then the
 * vertex-tag term (bound form) or the amplifier on matching tags (outlier) */
struct TagDynValue
{
    const uint8_t *etag;
    const int *vtag;
    int T;
    float vtw, amp;
    bool outlier;
    __device__ real_t value(const Walker<TagState> &w, int prev_tag, vertex_id_t v, const AdjUnit &e) const
    {
        if (w.step == 0)
            return (float)T;
        const int et = etag[e.index];
        float temp = fadd(1.0f, (float)((prev_tag + w.data.tag + et) % T));
        if (outlier)
        {
            if (w.data.tag == et)
                temp = fmul(temp, amp);
        }
        else
        {
            temp = fadd(temp, fmul((float)vtag[v], vtw));
        }
        return temp;
    }
};

struct TagDyn1 : TagDynValue
{
    __device__ real_t operator()(const Walker<TagState> &w, vertex_id_t v, const AdjUnit &e) const
    {
        return value(w, w.step == 0 ? 0 : vtag[w.data.previous_vertex], v, e);
    }
};

struct TagDyn2 : TagDynValue
{
    __device__ real_t operator()(const Walker<TagState> &w, const int &resp, vertex_id_t v, const AdjUnit &e) const
    {
        return value(w, w.step == 0 ? 0 : resp, v, e);
    }
};

struct TagPostQuery
{
    __device__ bool operator()(const Walker<TagState> &w, vertex_id_t, const AdjUnit &, vertex_id_t &target,
                               EmptyData &) const
    {
        if (w.step == 0)
            return false;
        target = w.data.previous_vertex;
        return true;
    }
};

struct TagRespond
{
    const int *vtag;
    __device__ void operator()(vertex_id_t target, const EmptyData &, const AdjList &, int &resp) const
    {
        resp = vtag[target];
    }
};

/* outlier form: the walker's tag range of the tag-grouped adjacency, area =
 * max of T * (amp - 1) * weight over it (test_outlier.cpp:151-170) */
struct TagOutlierUB
{
    const uint32_t *tb, *te;
    const float *w;
    int T;
    float amp;
    __device__ void operator()(const Walker<TagState> &wk, vertex_id_t v, const AdjList &adj, real_t &area,
                               vertex_id_t &num) const
    {
        if (wk.step == 0)
        {
            area = 0.0f;
            num = 0;
            return;
        }
        const uint32_t b = tb[(uint64_t)v * T + wk.data.tag], e = te[(uint64_t)v * T + wk.data.tag];
        float a = 0.0f;
        for (uint32_t i = b; i < e; i++)
        {
            const float wt = w ? w[adj.begin + i] : 1.0f;
            const float c = fmul(fmul((float)T, fsub(amp, 1.0f)), wt);
            if (a < c)
                a = c;
        }
        area = a;
        num = e - b;
    }
};

struct TagOutlierSearch
{
    const uint32_t *tb;
    const uint32_t *nbr;
    int T;
    __device__ bool operator()(const Walker<TagState> &wk, vertex_id_t v, const AdjList &adj, vertex_id_t idx,
                               AdjUnit &out) const
    {
        const uint32_t li = tb[(uint64_t)v * T + wk.data.tag] + idx;
        out = AdjUnit{nbr[adj.begin + li], adj.begin + li};
        return true;
    }
};

struct TagInit
{
    int T;
    __device__ void operator()(Walker<TagState> &w, vertex_id_t, Sampler &) const { w.data.tag = (int)(w.id % T); }
};

struct TagUpdate
{
    int T;
    __device__ void operator()(Walker<TagState> &w, vertex_id_t cur, const AdjUnit &) const
    {
        w.data.tag = (w.data.tag + 1) % T;
        w.data.previous_vertex = cur;
    }
};

struct Args
{
    const int *vtag;
    const uint32_t *tb, *te;
    int T;
    float vtw, amp;
};

template <int Order, bool Outlier, bool Weighted>
kk_status run(kk_engine *e, const kk_walk_opts &o, const Args &a, kk_paths **out)
{
    typedef typename std::conditional<Weighted, apps::WeightStatic, NoHook>::type StaticT;
    typedef typename std::conditional<Outlier, TagConst, TagUB>::type UBT;
    typedef typename std::conditional<Outlier, TagConst, TagLB>::type LBT;
    typedef typename std::conditional<Outlier, TagOutlierUB, NoHook>::type OutUBT;
    typedef typename std::conditional<Outlier, TagOutlierSearch, NoHook>::type OutSearchT;
    WalkerConfig<TagState, NoHook, TagInit, TagUpdate> wc;
    wc.walker_num = o.walker_num;
    wc.walker_init_state = TagInit{a.T};
    wc.walker_update_state = TagUpdate{a.T};
    TagDynValue dv{e->d_type, a.vtag, a.T, a.vtw, a.amp, Outlier};
    UBT ub;
    LBT lb;
    if constexpr (Outlier)
    {
        ub = TagConst{(float)a.T};
        lb = TagConst{1.0f};
    }
    else
    {
        ub = TagUB{a.vtag, a.T, a.vtw};
        lb = TagLB{a.vtag, a.vtw};
    }
    OutUBT oub{};
    OutSearchT osr{};
    if constexpr (Outlier)
    {
        oub = TagOutlierUB{a.tb, a.te, Weighted ? e->d_w : nullptr, a.T, a.amp};
        osr = TagOutlierSearch{a.tb, e->d_nbr, a.T};
    }
    StaticT st{};
    if constexpr (Weighted)
        st = apps::WeightStatic{e->d_w};
    if constexpr (Order == 1)
    {
        TransitionConfig<TagState, TagExt, StaticT, TagDyn1, UBT, LBT, OutUBT, OutSearchT> tc;
        tc.extension_comp = TagExt{o.walk_length};
        tc.static_comp = st;
        tc.dynamic_comp = TagDyn1{dv};
        tc.dcomp_upperbound = ub;
        tc.dcomp_lowerbound = lb;
        tc.outlier_upperbound = oub;
        tc.outlier_search = osr;
        return random_walk<TagState>(e, wc, tc, o, out);
    }
    else
    {
        SecondOrderTransitionConfig<TagState, EmptyData, int, TagExt, StaticT, TagPostQuery, TagRespond, TagDyn2,
                                    UBT, LBT, OutUBT, OutSearchT>
            tc;
        tc.extension_comp = TagExt{o.walk_length};
        tc.static_comp = st;
        tc.post_query = TagPostQuery{};
        tc.respond_query = TagRespond{a.vtag};
        tc.dynamic_comp = TagDyn2{dv};
        tc.dcomp_upperbound = ub;
        tc.dcomp_lowerbound = lb;
        tc.outlier_upperbound = oub;
        tc.outlier_search = osr;
        return random_walk<TagState>(e, wc, tc, o, out);
    }
}

} // namespace

/* Tag walk over the engine's graph: edge tags are its edge types (grouped by
 * tag within each adjacency for the outlier form), vertex_tag[V] is a host
 * array, order 1 or 2, outlier 0 (bound form) or 1, opts->weighted selects the
 * weight as static component. */
extern "C" kk_status kk_example_tagwalk(kk_engine *e, const kk_walk_opts *opts, const int32_t *vertex_tag,
                                        int tag_num, float vertex_tag_weight, float outlier_amplifier, int order,
                                        int outlier, kk_paths **out)
{
    if (!e || !opts || !vertex_tag || !out || tag_num < 1 || tag_num > 255 || (order != 1 && order != 2))
        return KK_ERR_INVALID_CONFIG;
    uint32_t V = 0;
    uint64_t E = 0;
    int hw = 0, ht = 0;
    kk_status s = kk_graph_info(e, &V, &E, &hw, &ht);
    if (s != KK_OK)
        return s;
    if (!ht || (opts->weighted && !hw))
        return KK_ERR_INVALID_CONFIG;
    std::vector<int64_t> off((size_t)V + 1);
    std::vector<uint8_t> type(E + 1);
    if ((s = kk_graph_download(e, off.data(), nullptr, nullptr, type.data())) != KK_OK)
        return s;
    std::vector<uint32_t> tb((size_t)V * tag_num, 0), te((size_t)V * tag_num, 0);
    for (uint32_t v = 0; v < V; v++)
        for (int64_t i = off[v]; i < off[v + 1]; i++)
        {
            if (type[i] >= tag_num)
                return KK_ERR_INVALID_CONFIG;
            const size_t k = (size_t)v * tag_num + type[i];
            const uint32_t li = (uint32_t)(i - off[v]);
            if (tb[k] == te[k])
                tb[k] = li;
            te[k] = li + 1;
        }
    int *d_vtag = nullptr;
    uint32_t *d_tb = nullptr, *d_te = nullptr;
    if (cudaMalloc(&d_vtag, (size_t)V * 4) != cudaSuccess || cudaMalloc(&d_tb, tb.size() * 4) != cudaSuccess ||
        cudaMalloc(&d_te, te.size() * 4) != cudaSuccess)
    {
        cudaFree(d_vtag);
        cudaFree(d_tb);
        return KK_ERR_OOM;
    }
    cudaMemcpy(d_vtag, vertex_tag, (size_t)V * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_tb, tb.data(), tb.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_te, te.data(), te.size() * 4, cudaMemcpyHostToDevice);
    Args a{d_vtag, d_tb, d_te, tag_num, vertex_tag_weight, outlier_amplifier};
    const int key = (order == 2 ? 4 : 0) + (outlier ? 2 : 0) + (opts->weighted ? 1 : 0);
    switch (key)
    {
    case 0: s = run<1, false, false>(e, *opts, a, out); break;
    case 1: s = run<1, false, true>(e, *opts, a, out); break;
    case 2: s = run<1, true, false>(e, *opts, a, out); break;
    case 3: s = run<1, true, true>(e, *opts, a, out); break;
    case 4: s = run<2, false, false>(e, *opts, a, out); break;
    case 5: s = run<2, false, true>(e, *opts, a, out); break;
    case 6: s = run<2, true, false>(e, *opts, a, out); break;
    default: s = run<2, true, true>(e, *opts, a, out); break;
    }
    cudaFree(d_vtag);
    cudaFree(d_tb);
    cudaFree(d_te);
    return s;
}
