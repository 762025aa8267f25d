/*
 * Batched walks: many walk jobs of one app in one launch.
 *
 * Jobs of uneven walker counts, lengths, node2vec (p, q) and metapath schemes
 * share one kernel (walk_batch_kernel): the alias tables of the graph are built
 * once for the batch, and small jobs fill the GPU alongside large ones instead
 * of each paying a launch with an idle tail.  Every job's paths equal those of
 * the same job run alone through kk_walk.
 */
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "knightking_gb300/engine.cuh"

namespace kk
{
using namespace apps;

BatchPlan plan_batch(kk_engine *e, const kk_walk_opts *jobs, int n, bool longest_first)
{
    require_graph(e);
    if (jobs == nullptr || n < 1 || (uint32_t)n > kMaxBatchJobs)
        fail(KK_ERR_INVALID_CONFIG, "a batch holds 1..1024 jobs");
    BatchPlan plan;
    plan.app = jobs[0].app;
    plan.weighted = jobs[0].weighted != 0;
    if (plan.app != KK_APP_DEEPWALK && plan.app != KK_APP_NODE2VEC && plan.app != KK_APP_METAPATH)
        fail(KK_ERR_INVALID_CONFIG, "batches take DeepWalk, node2vec or metapath jobs");
    if (plan.weighted && e->d_w == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "weighted batch on a graph without weights");
    if (plan.app == KK_APP_METAPATH && e->d_type == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "metapath needs edge types");
    uint64_t first = 0, base = 0;
    for (int j = 0; j < n; j++)
    {
        const kk_walk_opts &o = jobs[j];
        if (o.app != plan.app || (o.weighted != 0) != plan.weighted)
            fail(KK_ERR_INVALID_CONFIG, "all jobs of a batch have the same app and weighting");
        if (o.start != nullptr || (o.rate != 0.0 && o.rate != 1.0))
            fail(KK_ERR_INVALID_CONFIG, "batch jobs take no start list and no epochs");
        if ((uint64_t)o.walker_begin + o.walker_num > 0x100000000ULL || o.walk_length >= 0xfffffff0u)
            fail(KK_ERR_INVALID_CONFIG, "walker ids or walk length out of range");
        BatchJob b;
        memset(&b, 0, sizeof(b));
        b.seed = o.seed;
        b.walker_begin = o.walker_begin;
        b.walker_num = o.walker_num;
        b.first_task = (uint32_t)first;
        b.cap = o.walk_length + 1;
        b.path_base = base;
        b.walk_length = o.walk_length;
        b.flag = o.scheme_round_robin;
        if (plan.app == KK_APP_NODE2VEC)
        {
            if (!(o.p > 0.0f) || !(o.q > 0.0f))
                fail(KK_ERR_INVALID_CONFIG, "node2vec needs p > 0 and q > 0");
            const Node2vecConstants c = Node2vecConstants::make(o.p, o.q);
            b.c[0] = c.upperbound;
            b.c[1] = c.lowerbound;
            b.c[2] = c.overflow;
            b.c[3] = c.inv_p;
            b.c[4] = c.inv_q;
        }
        if (plan.app == KK_APP_METAPATH)
            plan.schemes.push_back(make_schemes(o));
        first += o.walker_num;
        base += (uint64_t)o.walker_num * b.cap;
        if (first > 0x80000000ULL)
            fail(KK_ERR_INVALID_CONFIG, "at most 2^31 walkers per batch");
        plan.jobs.push_back(b);
    }
    plan.total = (uint32_t)first;
    plan.total_cap = base;
    /* longest_first: the launch takes the jobs longest walk first (ties:
     * more walkers first), so the walkers that run longest start in the first
     * blocks and the batch's last blocks hold short walks, not a tail of long
     * ones (served S24 stream in batches of 1024: 87.3 -> 83.2 ms per pass).
     * Each job keeps its own first_task and path_base, so the results are laid
     * out in job order whatever the launch order. */
    std::vector<uint32_t> order(plan.jobs.size());
    for (size_t j = 0; j < order.size(); j++)
        order[j] = (uint32_t)j;
    if (longest_first)
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            const BatchJob &x = plan.jobs[a], &y = plan.jobs[b];
            return x.walk_length != y.walk_length ? x.walk_length > y.walk_length : x.walker_num > y.walker_num;
        });
    uint32_t at = 0;
    for (size_t k = 0; k < order.size(); k++)
    {
        plan.jobs[k].launch_first = at;
        plan.jobs[k].launch_job = order[k];
        at += plan.jobs[order[k]].walker_num;
    }
    return plan;
}

namespace
{

/* Launches the batch on the slot, reading alias tables in the Bucket layout
 * (built on the engine's stream first unless prepared). */
template <typename App, typename Bucket>
void launch_batch_with(kk_engine *e, const App &app, const BatchPlan &plan, BatchSlot &slot, const BatchJob *d_jobs,
                       uint32_t *length, uint32_t **path, unsigned long long *steps, int *status, bool want_paths,
                       bool prepared, const uint32_t *hdr)
{
    typedef typename App::TC TC;
    const Bucket *alias = nullptr;
    if constexpr (TC::has_static)
    {
        if (!prepared)
        {
            TransitionConfig<EmptyData, FixedLengthExt<EmptyData>, WeightStatic> stc;
            stc.static_comp = WeightStatic{e->d_w};
            build_alias<decltype(stc), Bucket>(e, stc);
        }
        alias = (const Bucket *)e->alias.p;
    }
    /* a captured launch (hdr != nullptr) serves every batch of the slot: the
     * buffers are the slot's full-size ones and the counts come from hdr */
    const uint64_t cap = hdr ? slot.max_cap : plan.total_cap;
    const uint32_t walkers = hdr ? slot.max_walkers : plan.total;
    *path = want_paths ? slot.path.as<uint32_t>(cap) : nullptr;
    if (!hdr)
        KK_CUDA_CHECK(cudaEventRecord(slot.ev[1], slot.stream));
    GraphView gv = e->view();
    if constexpr (!TC::has_static)
    {
        if (e->cursor_adjacency)
            gv.adjc = !prepared ? cursor_adjacency_of(e) : e->adjc_valid ? (const uint4 *)e->adjc.p : nullptr;
    }
    const unsigned bs = (unsigned)e->walk_block;
    const uint32_t nj = (uint32_t)plan.jobs.size();
    unsigned long long *st = e->walk_stats ? steps + 1 : nullptr;
    if (e->walk_schedule == 0)
    {
        unsigned grid = grid_for(e, walkers, bs);
        if (hdr && grid > 64u * (unsigned)e->sm_count)
            grid = 64u * (unsigned)e->sm_count; /* grid-stride over whatever the header holds */
        /* parking (first-order rejection walks) on the engine's own batch
         * slot only: serving slots replay captured launches and run side by
         * side, and the queues are the engine's */
        BatchPark bp;
        typedef ParkedWalker<typename App::S> PW;
        PW *q[2] = {nullptr, nullptr};
        uint32_t *cnt = nullptr;
        const bool park = parks<TC>() && e->walk_park > 0 && hdr == nullptr && &slot == &e->bslot && plan.total > 0;
        if (park)
        {
            q[0] = e->park[0].as<PW>(plan.total);
            q[1] = e->park[1].as<PW>(plan.total);
            cnt = e->park_count.as<uint32_t>(2);
            KK_CUDA_CHECK(cudaMemsetAsync(cnt, 0, 2 * sizeof(uint32_t), slot.stream));
            bp.out = q[0];
            bp.count = cnt;
            bp.below = (uint32_t)e->walk_park;
        }
        walk_batch_kernel<typename App::S, App, Bucket><<<grid, bs, 0, slot.stream>>>(
            gv, app, d_jobs, nj, plan.total, alias, (const float *)e->sum.p, *path, length, steps, status,
            e->trial_limit, st, hdr, bp, slot.notify);
        count_launch(e);
        if (park)
        {
            const unsigned rgrid = (unsigned)e->sm_count * (1024u / bs);
            for (int r = 0; r < kParkRounds; r++)
            {
                const int cur = r & 1, nxt = cur ^ 1;
                KK_CUDA_CHECK(cudaMemsetAsync(cnt + nxt, 0, sizeof(uint32_t), slot.stream));
                BatchPark br;
                if (r + 1 < kParkRounds)
                {
                    br.out = q[nxt];
                    br.count = cnt + nxt;
                    br.below = (uint32_t)e->walk_park;
                }
                walk_batch_resume_kernel<typename App::S, App, Bucket><<<rgrid, bs, 0, slot.stream>>>(
                    gv, app, d_jobs, nj, alias, (const float *)e->sum.p, *path, length, steps, status,
                    e->trial_limit, st, q[cur], cnt + cur, br);
                count_launch(e);
            }
        }
    }
    else
    {
        /* persistent walker pool: as many resident blocks as fit, on every SM */
        static int resident = 0;
        if (resident == 0)
            KK_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &resident, walk_batch_pool_kernel<typename App::S, App, Bucket>, (int)bs, 0));
        const uint64_t want = (uint64_t)e->sm_count * (resident > 0 ? resident : 1);
        const uint64_t need = ((uint64_t)walkers + bs - 1) / bs;
        const unsigned grid = (unsigned)(want < need ? want : (need ? need : 1));
        walk_batch_pool_kernel<typename App::S, App, Bucket><<<grid, bs, 0, slot.stream>>>(
            gv, app, d_jobs, nj, plan.total, alias, (const float *)e->sum.p, *path, length, steps, status,
            e->trial_limit, st, hdr, slot.notify);
        count_launch(e);
    }
    KK_CUDA_CHECK(cudaGetLastError());
}

/* The alias layout the engine's alias_layout option picks for the app:
 * where the app's hooks allow them, cursor (0) or 16 B neighbour (2)
 * buckets; else index buckets (1). */
template <typename App>
int app_layout(const kk_engine *e)
{
    if (e->alias_layout == 0 && use_cursor_buckets<typename App::WC, typename App::TC>())
        return 0;
    if (e->alias_layout == 2 && use_neighbour_buckets<typename App::WC, typename App::TC>())
        return 2;
    return 1;
}

template <typename App>
void launch_batch(kk_engine *e, const App &app, const BatchPlan &plan, BatchSlot &slot, const BatchJob *d_jobs,
                  uint32_t *length, uint32_t **path, unsigned long long *steps, int *status, bool want_paths,
                  bool prepared, const uint32_t *hdr = nullptr)
{
    if constexpr (use_cursor_buckets<typename App::WC, typename App::TC>())
    {
        if (app_layout<App>(e) == 0)
        {
            launch_batch_with<App, CursorBucket>(e, app, plan, slot, d_jobs, length, path, steps, status,
                                                 want_paths, prepared, hdr);
            return;
        }
    }
    if constexpr (use_neighbour_buckets<typename App::WC, typename App::TC>())
    {
        if (app_layout<App>(e) == 2)
        {
            launch_batch_with<App, NeighbourBucket>(e, app, plan, slot, d_jobs, length, path, steps, status,
                                                    want_paths, prepared, hdr);
            return;
        }
    }
    launch_batch_with<App, IndexBucket>(e, app, plan, slot, d_jobs, length, path, steps, status, want_paths,
                                        prepared, hdr);
}

/* The app's launch (the dispatch of run_batch), for a prepared engine. */
void launch_app_batch(kk_engine *e, const BatchPlan &plan, BatchSlot &slot, const BatchJob *d_jobs, uint32_t *length,
                      uint32_t **path, unsigned long long *d_steps, int *d_status, bool want_paths, bool p,
                      const uint32_t *hdr)
{
    const GraphView g = e->view();
    const uint8_t *vmask = (const uint8_t *)e->vmask.p;
    if (plan.app == KK_APP_DEEPWALK)
    {
        if (plan.weighted)
            launch_batch(e, DeepWalkBatch<true>{e->d_w}, plan, slot, d_jobs, length, path, d_steps, d_status,
                         want_paths, p, hdr);
        else
            launch_batch(e, DeepWalkBatch<false>{nullptr}, plan, slot, d_jobs, length, path, d_steps, d_status,
                         want_paths, p, hdr);
    }
    else if (plan.app == KK_APP_NODE2VEC)
    {
        const EdgeSetView set = p ? e->n2v_adjacency == 0
                                        ? EdgeSetView{(const uint64_t *)e->edge_set.p, e->edge_set_nb}
                                        : EdgeSetView{nullptr, 0}
                                  : node2vec_edge_set(e);
        if (plan.weighted)
            launch_batch(e, Node2vecBatch<true>{g.nbr, e->d_w, set}, plan, slot, d_jobs, length, path, d_steps,
                         d_status, want_paths, p, hdr);
        else
            launch_batch(e, Node2vecBatch<false>{g.nbr, nullptr, set}, plan, slot, d_jobs, length, path, d_steps,
                         d_status, want_paths, p, hdr);
    }
    else
    {
        if (!p)
            vmask = metapath_vertex_masks(e);
        if (plan.weighted)
            launch_batch(e, MetapathBatch<true>{vmask, e->d_type, e->d_w}, plan, slot, d_jobs, length, path,
                         d_steps, d_status, want_paths, p, hdr);
        else
            launch_batch(e, MetapathBatch<false>{vmask, e->d_type, nullptr}, plan, slot, d_jobs, length, path,
                         d_steps, d_status, want_paths, p, hdr);
    }
}

/* Builds the weight alias tables in the layout App's walk reads. */
template <typename App>
void prepare_tables(kk_engine *e)
{
    TransitionConfig<EmptyData, FixedLengthExt<EmptyData>, WeightStatic> stc;
    stc.static_comp = WeightStatic{e->d_w};
    const int layout = app_layout<App>(e);
    if (layout == 0)
        build_alias<decltype(stc), CursorBucket>(e, stc);
    else if (layout == 2)
        build_alias<decltype(stc), NeighbourBucket>(e, stc);
    else
        build_alias<decltype(stc), IndexBucket>(e, stc);
}

} // namespace

void batch_prepare(kk_engine *e, const BatchPlan &plan)
{
    if (plan.app == KK_APP_NODE2VEC)
    {
        graph_sort_adjacency(e);
        node2vec_edge_set(e);
    }
    if (plan.app == KK_APP_METAPATH)
        metapath_vertex_masks(e);
    if (!plan.weighted && e->cursor_adjacency)
        cursor_adjacency_of(e);
    if (plan.weighted)
    {
        if (plan.app == KK_APP_DEEPWALK)
            prepare_tables<DeepWalkBatch<true>>(e);
        else if (plan.app == KK_APP_NODE2VEC)
            prepare_tables<Node2vecBatch<true>>(e);
        else
            prepare_tables<MetapathBatch<true>>(e);
    }
}

/* Staging layout of a graph-mode slot (pinned): the job table, the metapath
 * schemes, the counts header, the status words. */
struct GraphStage
{
    BatchJob *jobs;
    MetaSchemes *schemes;
    uint32_t *hdr;
    int *status;
};

static GraphStage graph_stage(const BatchSlot &slot)
{
    GraphStage g;
    g.jobs = (BatchJob *)slot.h_stage;
    g.schemes = (MetaSchemes *)(g.jobs + kMaxBatchJobs);
    g.hdr = (uint32_t *)(g.schemes + kMaxBatchJobs);
    g.status = (int *)(g.hdr + 4);
    return g;
}

void batch_slot_graph_mode(kk_engine *e, BatchSlot &slot, uint32_t max_walkers, uint64_t max_cap)
{
    for (int i = 0; i < 3; i++)
        if (slot.ev[i] == nullptr)
            KK_CUDA_CHECK(cudaEventCreate(&slot.ev[i]));
    slot.max_walkers = max_walkers;
    slot.max_cap = max_cap;
    slot.jobs.as<BatchJob>(kMaxBatchJobs);
    slot.schemes.as<MetaSchemes>(kMaxBatchJobs);
    slot.small.ensure(128);
    slot.length.as<uint32_t>(max_walkers);
    slot.path.as<uint32_t>(max_cap);
    const size_t stage = kMaxBatchJobs * (sizeof(BatchJob) + sizeof(MetaSchemes)) + 16 + 64;
    KK_CUDA_CHECK(cudaHostAlloc((void **)&slot.h_stage, stage, cudaHostAllocDefault));
    memset(slot.h_stage, 0, stage);
    slot.graph_mode = true;
    (void)e;
}

void batch_slot_notify_mode(BatchSlot &slot)
{
    if (slot.notify.count != nullptr)
        return;
    uint32_t *d = slot.notify_dev.as<uint32_t>(2 * kMaxBatchJobs);
    KK_CUDA_CHECK(cudaHostAlloc((void **)&slot.h_flag, kMaxBatchJobs * sizeof(uint32_t), cudaHostAllocMapped));
    memset(slot.h_flag, 0, kMaxBatchJobs * sizeof(uint32_t));
    uint32_t *d_flag = nullptr;
    KK_CUDA_CHECK(cudaHostGetDevicePointer((void **)&d_flag, slot.h_flag, 0));
    KK_CUDA_CHECK(cudaStreamCreateWithFlags(&slot.copy, cudaStreamNonBlocking));
    slot.notify.count = d;
    slot.notify.status = (int *)(d + kMaxBatchJobs);
    slot.notify.flag = d_flag;
}

/* The per-request counters and status words start at zero for every batch. */
static void reset_notify(const BatchSlot &slot)
{
    if (slot.notify.count != nullptr)
        KK_CUDA_CHECK(cudaMemsetAsync(slot.notify.count, 0, 2 * kMaxBatchJobs * sizeof(uint32_t), slot.stream));
}

/* One graph-mode batch: stage the job table and counts, replay (capturing it
 * on first use) the slot's graph; the status read-back lands in the staging
 * block when the graph ends. */
static void launch_batch_graph(kk_engine *e, BatchPlan &plan, BatchSlot &slot)
{
    if (plan.total > slot.max_walkers || plan.total_cap > slot.max_cap)
        fail(KK_ERR_INVALID_CONFIG, "batch larger than the slot");
    const GraphStage h = graph_stage(slot);
    BatchJob *d_jobs = (BatchJob *)slot.jobs.p;
    MetaSchemes *d_sc = (MetaSchemes *)slot.schemes.p;
    int *d_status = (int *)slot.small.p;
    unsigned long long *d_steps = (unsigned long long *)((char *)d_status + 16);
    const uint32_t *d_hdr = (const uint32_t *)((char *)d_status + 64);
    const uint32_t nj = (uint32_t)plan.jobs.size();
    for (uint32_t j = 0; j < nj; j++)
        plan.jobs[j].param = d_sc + j;
    memcpy(h.jobs, plan.jobs.data(), nj * sizeof(BatchJob));
    if (!plan.schemes.empty())
        memcpy(h.schemes, plan.schemes.data(), plan.schemes.size() * sizeof(MetaSchemes));
    h.hdr[0] = nj;
    h.hdr[1] = plan.total;
    if (slot.exec == nullptr)
    {
        cudaGraph_t graph = nullptr;
        KK_CUDA_CHECK(cudaStreamBeginCapture(slot.stream, cudaStreamCaptureModeThreadLocal));
        try
        {
            KK_CUDA_CHECK(cudaMemcpyAsync(d_jobs, h.jobs, kMaxBatchJobs * sizeof(BatchJob), cudaMemcpyHostToDevice,
                                          slot.stream));
            if (plan.app == KK_APP_METAPATH)
                KK_CUDA_CHECK(cudaMemcpyAsync(d_sc, h.schemes, kMaxBatchJobs * sizeof(MetaSchemes),
                                              cudaMemcpyHostToDevice, slot.stream));
            KK_CUDA_CHECK(cudaMemcpyAsync((void *)d_hdr, h.hdr, 16, cudaMemcpyHostToDevice, slot.stream));
            KK_CUDA_CHECK(cudaMemsetAsync(d_status, 0, 64, slot.stream));
            reset_notify(slot);
            uint32_t *path = nullptr;
            launch_app_batch(e, plan, slot, d_jobs, (uint32_t *)slot.length.p, &path, d_steps, d_status, true, true,
                             d_hdr);
            /* with per-request completion each request's status comes with
             * its flag and its steps with its paths: no read-back, which
             * would wait on a copy engine behind the other slots' paths */
            if (slot.notify.count == nullptr)
                KK_CUDA_CHECK(cudaMemcpyAsync(h.status, d_status, 64, cudaMemcpyDeviceToHost, slot.stream));
        }
        catch (...)
        {
            cudaStreamEndCapture(slot.stream, &graph);
            if (graph)
                cudaGraphDestroy(graph);
            throw;
        }
        KK_CUDA_CHECK(cudaStreamEndCapture(slot.stream, &graph));
        const cudaError_t ie = cudaGraphInstantiate(&slot.exec, graph, 0);
        cudaGraphDestroy(graph);
        KK_CUDA_CHECK(ie);
    }
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[1], slot.stream));
    KK_CUDA_CHECK(cudaGraphLaunch(slot.exec, slot.stream));
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[2], slot.stream));
}

/* Waits for a graph-mode batch; its status and walker-steps from the staging
 * block (a slot with per-request completion reads neither: see
 * launch_batch_graph). */
static uint64_t finish_batch_graph(BatchSlot &slot)
{
    const GraphStage h = graph_stage(slot);
    KK_CUDA_CHECK(cudaStreamSynchronize(slot.stream));
    if (slot.notify.count != nullptr)
        fail(KK_ERR_INVALID_CONFIG, "a slot with per-request completion has no batch count");
    slot.alias_ms = 0.0f;
    KK_CUDA_CHECK(cudaEventElapsedTime(&slot.walk_ms, slot.ev[1], slot.ev[2]));
    if (h.status[0] & KK_STATUS_TRIAL_LIMIT)
        fail(KK_ERR_TRIAL_LIMIT, "a walker exceeded the rejection-trial limit");
    if (h.status[0] & KK_STATUS_PATH_CAPACITY)
        fail(KK_ERR_PATH_CAPACITY, "a walk exceeded its path capacity");
    unsigned long long steps;
    memcpy(&steps, (char *)h.status + 16, sizeof(steps));
    return steps;
}

static uint64_t run_batch_graph(kk_engine *e, BatchPlan &plan, BatchSlot &slot)
{
    launch_batch_graph(e, plan, slot);
    return finish_batch_graph(slot);
}

void batch_launch_async(kk_engine *e, BatchPlan &plan, BatchSlot &slot)
{
    if (slot.graph_mode)
    {
        launch_batch_graph(e, plan, slot);
        return;
    }
    for (int i = 0; i < 3; i++)
        if (slot.ev[i] == nullptr)
            KK_CUDA_CHECK(cudaEventCreate(&slot.ev[i]));
    if (plan.app == KK_APP_METAPATH)
    {
        MetaSchemes *d_sc = slot.schemes.as<MetaSchemes>(plan.schemes.size());
        KK_CUDA_CHECK(cudaMemcpyAsync(d_sc, plan.schemes.data(), plan.schemes.size() * sizeof(MetaSchemes),
                                      cudaMemcpyHostToDevice, slot.stream));
        for (size_t j = 0; j < plan.jobs.size(); j++)
            plan.jobs[j].param = d_sc + j;
    }
    BatchJob *d_jobs = slot.jobs.as<BatchJob>(plan.jobs.size());
    KK_CUDA_CHECK(cudaMemcpyAsync(d_jobs, plan.jobs.data(), plan.jobs.size() * sizeof(BatchJob),
                                  cudaMemcpyHostToDevice, slot.stream));
    int *d_status = (int *)slot.small.ensure(64);
    unsigned long long *d_steps = (unsigned long long *)((char *)d_status + 16);
    KK_CUDA_CHECK(cudaMemsetAsync(d_status, 0, 64, slot.stream));
    reset_notify(slot);
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[0], slot.stream));
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[1], slot.stream));
    uint32_t *length = slot.length.as<uint32_t>(plan.total);
    uint32_t *path = nullptr;
    launch_app_batch(e, plan, slot, d_jobs, length, &path, d_steps, d_status, true, true, nullptr);
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[2], slot.stream));
}

uint64_t batch_finish(kk_engine *e, BatchSlot &slot)
{
    (void)e;
    if (slot.graph_mode)
        return finish_batch_graph(slot);
    KK_CUDA_CHECK(cudaStreamSynchronize(slot.stream));
    int h_small[16];
    KK_CUDA_CHECK(cudaMemcpy(h_small, slot.small.p, sizeof(h_small), cudaMemcpyDeviceToHost));
    KK_CUDA_CHECK(cudaEventElapsedTime(&slot.alias_ms, slot.ev[0], slot.ev[1]));
    KK_CUDA_CHECK(cudaEventElapsedTime(&slot.walk_ms, slot.ev[1], slot.ev[2]));
    if (h_small[0] & KK_STATUS_TRIAL_LIMIT)
        fail(KK_ERR_TRIAL_LIMIT, "a walker exceeded the rejection-trial limit");
    if (h_small[0] & KK_STATUS_PATH_CAPACITY)
        fail(KK_ERR_PATH_CAPACITY, "a walk exceeded its path capacity");
    unsigned long long steps;
    memcpy(&steps, (char *)h_small + 16, sizeof(steps));
    return steps;
}

uint64_t run_batch(kk_engine *e, BatchPlan &plan, BatchSlot &slot, bool want_paths, bool prepared)
{
    if (slot.graph_mode)
        return run_batch_graph(e, plan, slot);
    for (int i = 0; i < 3; i++)
        if (slot.ev[i] == nullptr)
            KK_CUDA_CHECK(cudaEventCreate(&slot.ev[i]));
    if (!prepared && plan.app == KK_APP_NODE2VEC)
        graph_sort_adjacency(e);
    if (plan.app == KK_APP_METAPATH)
    {
        MetaSchemes *d_sc = slot.schemes.as<MetaSchemes>(plan.schemes.size());
        KK_CUDA_CHECK(cudaMemcpyAsync(d_sc, plan.schemes.data(), plan.schemes.size() * sizeof(MetaSchemes),
                                      cudaMemcpyHostToDevice, slot.stream));
        for (size_t j = 0; j < plan.jobs.size(); j++)
            plan.jobs[j].param = d_sc + j;
    }
    BatchJob *d_jobs = slot.jobs.as<BatchJob>(plan.jobs.size());
    KK_CUDA_CHECK(cudaMemcpyAsync(d_jobs, plan.jobs.data(), plan.jobs.size() * sizeof(BatchJob),
                                  cudaMemcpyHostToDevice, slot.stream));
    int *d_status = (int *)slot.small.ensure(64);
    unsigned long long *d_steps = (unsigned long long *)((char *)d_status + 16);
    KK_CUDA_CHECK(cudaMemsetAsync(d_status, 0, 64, slot.stream));
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[0], slot.stream));
    if (!prepared && slot.stream != e->stream)
    {
        /* tables are built on the engine's stream */
        KK_CUDA_CHECK(cudaEventRecord(e->ev_fork, slot.stream));
        KK_CUDA_CHECK(cudaStreamWaitEvent(e->stream, e->ev_fork, 0));
    }
    uint32_t *length = slot.length.as<uint32_t>(plan.total);
    uint32_t *path = nullptr;
    launch_app_batch(e, plan, slot, d_jobs, length, &path, d_steps, d_status, want_paths, prepared, nullptr);
    KK_CUDA_CHECK(cudaEventRecord(slot.ev[2], slot.stream));
    int h_small[16];
    KK_CUDA_CHECK(cudaMemcpyAsync(h_small, d_status, sizeof(h_small), cudaMemcpyDeviceToHost, slot.stream));
    KK_CUDA_CHECK(cudaStreamSynchronize(slot.stream));
    if (&slot == &e->bslot)
        memcpy(e->last_stats, (char *)h_small + 24, sizeof(e->last_stats));
    KK_CUDA_CHECK(cudaEventElapsedTime(&slot.alias_ms, slot.ev[0], slot.ev[1]));
    KK_CUDA_CHECK(cudaEventElapsedTime(&slot.walk_ms, slot.ev[1], slot.ev[2]));
    if (h_small[0] & KK_STATUS_TRIAL_LIMIT)
        fail(KK_ERR_TRIAL_LIMIT, "a walker exceeded the rejection-trial limit");
    if (h_small[0] & KK_STATUS_PATH_CAPACITY)
        fail(KK_ERR_PATH_CAPACITY, "a walk exceeded its path capacity");
    unsigned long long steps;
    memcpy(&steps, (char *)h_small + 16, sizeof(steps));
    return steps;
}

} // namespace kk


using namespace kk;

extern "C" {

kk_status kk_batch_walk_device(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, uint64_t *total_steps,
                               const uint32_t **d_length, const uint32_t **d_vertices)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        BatchPlan plan = plan_batch(e, jobs, n_jobs);
        BatchSlot &slot = e->bslot;
        slot.stream = e->stream;
        const bool want = d_vertices != nullptr;
        uint64_t steps = run_batch(e, plan, slot, want, false);
        e->alias_ms = slot.alias_ms;
        e->walk_ms = slot.walk_ms;
        if (total_steps)
            *total_steps = steps;
        if (d_length)
            *d_length = (const uint32_t *)slot.length.p;
        if (d_vertices)
            *d_vertices = (const uint32_t *)slot.path.p;
    });
}

} /* extern "C" */

namespace
{

/* A walked batch's paths out: all jobs packed in one pass, then every job's
 * lengths, offsets and vertices copied straight into a pooled pinned block,
 * one wait. */
void batch_paths_out(kk_engine *e, const BatchPlan &plan, BatchSlot &slot, kk_paths **out)
{
    const int n_jobs = (int)plan.jobs.size();
    {
        const uint32_t *len = (const uint32_t *)slot.length.p, *path = (const uint32_t *)slot.path.p;
        /* all jobs packed in one pass, then every job's lengths, offsets and
         * vertices copied straight into a pooled pinned block, one wait */
        std::vector<uint64_t> jb;
        const uint64_t *d_rel = nullptr;
        const uint32_t *d_verts = nullptr;
        pack_batch_paths(e, plan, (const BatchJob *)slot.jobs.p, len, path, &d_rel, &d_verts, jb);
        if (e->host_pool == nullptr)
        {
            e->host_pool = new HostPool();
            e->host_pool->limit = kBatchPoolCache;
        }
        for (int j = 0; j < n_jobs; j++)
        {
            const BatchJob &b = plan.jobs[j];
            const uint32_t n = b.walker_num;
            const uint64_t total = jb[j + 1] - jb[j];
            const size_t len_bytes = ((size_t)n * 4 + 15) & ~(size_t)15;
            const size_t off_bytes = ((size_t)n * 8 + 15) & ~(size_t)15;
            kk_paths *p = (kk_paths *)calloc(1, sizeof(kk_paths));
            PooledPaths *o = new (std::nothrow) PooledPaths();
            size_t cls = 0;
            char *blk = (p && o) ? (char *)e->host_pool->get(len_bytes + off_bytes + total * 4 + 16, &cls) : nullptr;
            if (!blk)
            {
                free(p);
                delete o;
                fail(KK_ERR_OOM, "host allocation failed");
            }
            o->pool = e->host_pool;
            o->block = blk;
            o->cls = cls;
            p->owner = o;
            out[j] = p;
            p->walker_num = n;
            p->walker_begin = b.walker_begin;
            p->epoch_walkers = n;
            p->total_steps = total - n;
            p->length = (uint32_t *)blk;
            p->offset = (uint64_t *)(blk + len_bytes);
            p->vertices = (uint32_t *)(blk + len_bytes + off_bytes);
            if (n == 0)
                continue;
            KK_CUDA_CHECK(cudaMemcpyAsync(p->length, len + b.first_task, (size_t)n * 4, cudaMemcpyDeviceToHost,
                                          e->stream));
            KK_CUDA_CHECK(cudaMemcpyAsync(p->offset, d_rel + b.first_task, (size_t)n * 8, cudaMemcpyDeviceToHost,
                                          e->stream));
            KK_CUDA_CHECK(cudaMemcpyAsync(p->vertices, d_verts + jb[j], total * 4, cudaMemcpyDeviceToHost,
                                          e->stream));
        }
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    }
}

void free_outs(kk_paths **out, int n)
{
    for (int j = 0; j < n; j++)
    {
        kk_paths_free(out[j]);
        out[j] = nullptr;
    }
}

} // namespace

/* A submitted batch: its plan, on the engine's batch slot. */
struct kk_batch
{
    kk_engine *e = nullptr;
    BatchPlan plan;
};

extern "C" {

kk_status kk_batch_walk(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, kk_paths **out)
{
    if (!e || !out)
        return KK_ERR_INVALID_CONFIG;
    for (int j = 0; j < n_jobs; j++)
        out[j] = nullptr;
    kk_status s = guard(e, [&] {
        BatchPlan plan = plan_batch(e, jobs, n_jobs);
        BatchSlot &slot = e->bslot;
        slot.stream = e->stream;
        run_batch(e, plan, slot, true, false);
        e->alias_ms = slot.alias_ms;
        e->walk_ms = slot.walk_ms;
        batch_paths_out(e, plan, slot, out);
    });
    if (s != KK_OK)
        free_outs(out, n_jobs);
    return s;
}

kk_status kk_batch_submit(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, kk_batch **out)
{
    if (!e || !out)
        return KK_ERR_INVALID_CONFIG;
    *out = nullptr;
    kk_batch *b = new (std::nothrow) kk_batch();
    if (!b)
        return KK_ERR_OOM;
    kk_status s = guard(e, [&] {
        b->e = e;
        b->plan = plan_batch(e, jobs, n_jobs);
        BatchSlot &slot = e->bslot;
        slot.stream = e->stream;
        batch_prepare(e, b->plan); /* the tables the walk reads, on the engine's stream */
        batch_launch_async(e, b->plan, slot);
    });
    if (s != KK_OK)
    {
        delete b;
        return s;
    }
    e->batch_out = true;
    *out = b;
    return KK_OK;
}

kk_status kk_batch_wait(kk_batch *b, kk_paths **out)
{
    if (!b || !out)
        return KK_ERR_INVALID_CONFIG;
    kk_engine *e = b->e;
    const int n_jobs = (int)b->plan.jobs.size();
    for (int j = 0; j < n_jobs; j++)
        out[j] = nullptr;
    e->batch_wait = true;
    kk_status s = guard(e, [&] {
        BatchSlot &slot = e->bslot;
        batch_finish(e, slot);
        e->alias_ms = slot.alias_ms;
        e->walk_ms = slot.walk_ms;
        batch_paths_out(e, b->plan, slot, out);
    });
    if (s != KK_OK)
        free_outs(out, n_jobs);
    e->batch_out = e->batch_wait = false;
    delete b;
    return s;
}

} /* extern "C" */
