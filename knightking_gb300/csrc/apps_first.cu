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
    rs.exact = true; /* ends only after walk_length steps or on an isolated start */
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
    rs.exact = true; /* ends only by the extension draw or on an isolated start */
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
    const MetaSchemes host_sc = make_schemes(o);
    MetaSchemes *sc = e->schemes.as<MetaSchemes>(1);
    KK_CUDA_CHECK(cudaMemcpyAsync(sc, &host_sc, sizeof(MetaSchemes), cudaMemcpyHostToDevice, e->stream));
    const uint8_t *vmask = metapath_vertex_masks(e);
    rs.fixed_cap = true;
    rs.cap = o.walk_length + 1;
    WalkerConfig<MetapathState, NoHook, MetapathInitState, MetapathUpdate> wc;
    wc.walker_num = rs.walker_num;
    wc.walker_init_state = MetapathInitState{sc, o.scheme_round_robin};
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
