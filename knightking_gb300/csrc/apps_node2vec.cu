/*
 * node2vec (src/apps/node2vec.hpp:108-202): second order, lower-bound
 * pre-accept, outlier appendix when 1/p > max(1, 1/q), unweighted or weighted.
 */
#include <type_traits>

#include "knightking_gb300/engine.cuh"

namespace kk
{
using namespace apps;

namespace
{

template <bool Weighted, bool Outlier>
void run_n2v(kk_engine *e, const kk_walk_opts &o, const Node2vecConstants &c, const RunSpec &rs, WalkResult &res,
             EdgeSetView set)
{
    typedef typename std::conditional<Weighted, WeightStatic, NoHook>::type StaticT;
    typedef typename std::conditional<Outlier, Node2vecOutlierUB<Weighted>, NoHook>::type OutUBT;
    typedef typename std::conditional<Outlier, Node2vecOutlierSearch, NoHook>::type OutSearchT;
    SecondOrderTransitionConfig<Node2vecState, vertex_id_t, bool, FixedLengthExt<Node2vecState>, StaticT,
                                Node2vecPostQuery, Node2vecRespond, Node2vecDyn, ConstBound, ConstBound, OutUBT,
                                OutSearchT>
        tc;
    tc.extension_comp = FixedLengthExt<Node2vecState>{o.walk_length};
    if constexpr (Weighted)
        tc.static_comp = WeightStatic{e->d_w};
    tc.post_query = Node2vecPostQuery{c.inv_q < 1.0f ? c.inv_q : 1.0f};
    tc.respond_query = Node2vecRespond{e->d_nbr, set};
    tc.dynamic_comp = Node2vecDyn{c.upperbound, c.inv_p, c.inv_q};
    tc.dcomp_upperbound = ConstBound{c.upperbound};
    tc.dcomp_lowerbound = ConstBound{c.lowerbound};
    if constexpr (Outlier)
    {
        tc.outlier_upperbound = Node2vecOutlierUB<Weighted>{e->d_nbr, e->d_w, c.overflow, set};
        tc.outlier_search = Node2vecOutlierSearch{e->d_nbr, set};
    }
    WalkerConfig<Node2vecState, NoHook, NoHook, Node2vecUpdate> wc;
    wc.walker_num = rs.walker_num;
    run_walk<Node2vecState>(e, wc, tc, rs, res);
}

} // namespace

void run_app_node2vec(kk_engine *e, const kk_walk_opts &o, const RunSpec &rs0, WalkResult &res)
{
    if (!(o.p > 0.0f) || !(o.q > 0.0f))
        fail(KK_ERR_INVALID_CONFIG, "node2vec needs p > 0 and q > 0");
    if (o.weighted && e->d_w == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "weighted node2vec needs edge weights");
    graph_sort_adjacency(e);
    RunSpec rs = rs0;
    rs.fixed_cap = true;
    rs.cap = o.walk_length + 1;
    rs.exact = true; /* ends only after walk_length steps or on an isolated start */
    Node2vecConstants c = Node2vecConstants::make(o.p, o.q);
    const EdgeSetView set = node2vec_edge_set(e);
    if (o.weighted)
    {
        if (c.outlier)
            run_n2v<true, true>(e, o, c, rs, res, set);
        else
            run_n2v<true, false>(e, o, c, rs, res, set);
    }
    else
    {
        if (c.outlier)
            run_n2v<false, true>(e, o, c, rs, res, set);
        else
            run_n2v<false, false>(e, o, c, rs, res, set);
    }
}

} // namespace kk
