/*
 * First-order built-in apps: DeepWalk (src/apps/deepwalk.hpp:30-47), PPR
 * (src/apps/ppr.hpp:30-64) and metapath (src/apps/metapath.hpp:70-128), each
 * unweighted (uniform pick) or weighted (alias tables of the edge weight).
 */
#include "knightking_gb300/engine.cuh"

namespace kk
{
using namespace apps;

namespace
{

template <typename TC>
void run_empty_state(kk_engine *e, const TC &tc, const RunSpec &rs, WalkResult &res)
{
    WalkerConfig<EmptyData> wc;
    wc.walker_num = rs.walker_num;
    run_walk<EmptyData>(e, wc, tc, rs, res);
}

void run_deepwalk(kk_engine *e, const kk_walk_opts &o, RunSpec rs, WalkResult &res)
{
    rs.fixed_cap = true;
    rs.cap = o.walk_length + 1;
    FixedLengthExt<EmptyData> ext{o.walk_length};
    if (o.weighted)
    {
        TransitionConfig<EmptyData, FixedLengthExt<EmptyData>, WeightStatic> tc;
        tc.extension_comp = ext;
        tc.static_comp = WeightStatic{e->d_w};
        run_empty_state(e, tc, rs, res);
    }
    else
    {
        TransitionConfig<EmptyData, FixedLengthExt<EmptyData>> tc;
        tc.extension_comp = ext;
        run_empty_state(e, tc, rs, res);
    }
}

void run_ppr(kk_engine *e, const kk_walk_opts &o, RunSpec rs, WalkResult &res)
{
    /* real_t extension_comp = 1 - terminate_prob (ppr.hpp:35), one float rounding */
    volatile float term = o.terminate_prob;
    float ext = 1.0f - term;
    if (!(ext < 1.0f) || !(ext >= 0.0f))
        fail(KK_ERR_INVALID_CONFIG, "PPR needs 0 < terminate_prob <= 1");
    rs.fixed_cap = false;
    rs.const_ext = ext;
    ConstantExt cext{ext};
    if (o.weighted)
    {
        TransitionConfig<EmptyData, ConstantExt, WeightStatic> tc;
        tc.extension_comp = cext;
        tc.static_comp = WeightStatic{e->d_w};
        run_empty_state(e, tc, rs, res);
    }
    else
    {
        TransitionConfig<EmptyData, ConstantExt> tc;
        tc.extension_comp = cext;
        run_empty_state(e, tc, rs, res);
    }
}

void run_metapath(kk_engine *e, const kk_walk_opts &o, RunSpec rs, WalkResult &res)
{
    if (e->d_type == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "metapath needs edge types");
    if (o.n_schemes < 1 || o.n_schemes > KK_MAX_SCHEMES)
        fail(KK_ERR_INVALID_CONFIG, "metapath needs 1..16 schemes");
    MetaSchemes sc;
    memset(&sc, 0, sizeof(sc));
    sc.n = (uint32_t)o.n_schemes;
    for (int s = 0; s < o.n_schemes; s++)
    {
        if (o.scheme_len[s] < 1 || o.scheme_len[s] > KK_MAX_SCHEME_LEN)
            fail(KK_ERR_INVALID_CONFIG, "metapath scheme length must be 1..16");
        sc.len[s] = (uint8_t)o.scheme_len[s];
        for (int j = 0; j < o.scheme_len[s]; j++)
            sc.mask[s][j] = o.scheme_mask[s][j];
    }
    GraphView g = e->view();
    uint8_t *vmask = e->vmask.as<uint8_t>(e->V);
    metapath_vertex_mask_kernel<<<grid_for(e, e->V, 256), 256, 0, e->stream>>>(g, vmask);
    KK_CUDA_CHECK(cudaGetLastError());
    rs.fixed_cap = true;
    rs.cap = o.walk_length + 1;
    WalkerConfig<MetapathState, NoHook, MetapathInitState, MetapathUpdate> wc;
    wc.walker_num = rs.walker_num;
    wc.walker_init_state = MetapathInitState{sc.n, o.scheme_round_robin};
    wc.walker_update_state = MetapathUpdate{sc};
    MetapathExt ext{vmask, o.walk_length, sc};
    MetapathDyn dyn{e->d_type, sc};
    if (o.weighted)
    {
        TransitionConfig<MetapathState, MetapathExt, WeightStatic, MetapathDyn, ConstBound> tc;
        tc.extension_comp = ext;
        tc.static_comp = WeightStatic{e->d_w};
        tc.dynamic_comp = dyn;
        tc.dcomp_upperbound = ConstBound{1.0f};
        run_walk<MetapathState>(e, wc, tc, rs, res);
    }
    else
    {
        TransitionConfig<MetapathState, MetapathExt, NoHook, MetapathDyn, ConstBound> tc;
        tc.extension_comp = ext;
        tc.dynamic_comp = dyn;
        tc.dcomp_upperbound = ConstBound{1.0f};
        run_walk<MetapathState>(e, wc, tc, rs, res);
    }
}

} // namespace

void run_app_first_order(kk_engine *e, const kk_walk_opts &o, const RunSpec &rs, WalkResult &res)
{
    switch (o.app)
    {
    case KK_APP_DEEPWALK:
        run_deepwalk(e, o, rs, res);
        break;
    case KK_APP_PPR:
        run_ppr(e, o, rs, res);
        break;
    case KK_APP_METAPATH:
        run_metapath(e, o, rs, res);
        break;
    default:
        fail(KK_ERR_INVALID_CONFIG, "unknown app");
    }
}

} // namespace kk
