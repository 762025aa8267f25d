/*
 * Engine internals shared by the C-ABI translation units.
 *
 * kk_engine owns the CSR in HBM (int64 off[V+1], uint32 nbr[E], float w[E],
 * uint8 type[E]) and grow-only work buffers (alias tables, path buffers), all
 * on one CUDA stream.  Errors inside are C++ exceptions (kk::Error) that the
 * C-ABI entry points turn into kk_status codes; none crosses the ABI.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string.h>

#include <atomic>
#include <functional>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "knightking_gb300.h"
#include "knightking_gb300/apps.cuh"

namespace kk
{

struct Error
{
    kk_status status;
    std::string msg;
};

[[noreturn]] inline void fail(kk_status s, const std::string &msg)
{
    throw Error{s, msg};
}

#define KK_CUDA_CHECK(call)                                                                                         \
    do                                                                                                              \
    {                                                                                                               \
        cudaError_t _e = (call);                                                                                    \
        if (_e != cudaSuccess)                                                                                      \
            ::kk::fail(_e == cudaErrorMemoryAllocation ? KK_ERR_OOM : KK_ERR_CUDA,                                  \
                       std::string(#call) + ": " + cudaGetErrorString(_e));                                         \
    } while (0)

/* Grow-only device buffer. */
struct DevBuf
{
    void *p = nullptr;
    size_t bytes = 0;
    void *ensure(size_t n)
    {
        if (n > bytes)
        {
            /* work in flight on any stream may still read the old buffer */
            if (p)
            {
                cudaDeviceSynchronize();
                cudaFree(p);
            }
            p = nullptr;
            bytes = 0;
            KK_CUDA_CHECK(cudaMalloc(&p, n));
            bytes = n;
        }
        return p;
    }
    template <typename T>
    T *as(size_t count)
    {
        return (T *)ensure(count * sizeof(T) > 0 ? count * sizeof(T) : 16);
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

/* Where one walk call's results are (device). */
struct WalkResult
{
    uint32_t walker_num = 0;
    uint32_t *length = nullptr;      /* walker_num */
    const uint64_t *path_off = nullptr; /* walker_num + 1, or nullptr with fixed cap */
    uint32_t cap = 0;
    uint32_t *path = nullptr;
    uint64_t total_steps = 0;
    bool packed = false; /* path_off holds the exact lengths: path is packed */
};

/* Stream, events and buffers one batch runs on: the engine's own (for the
 * synchronous batch calls) or a serving slot's, so that batches on different
 * slots run concurrently. */
struct BatchSlot
{
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    DevBuf jobs, small, length, path, schemes;
    float alias_ms = 0.0f, walk_ms = 0.0f;
    /* CUDA-graph mode (serving): buffers sized once for a full slot, the job
     * table and counts staged in pinned memory, the kernel reading the counts
     * from device memory, so one captured graph (uploads, status reset,
     * kernel, status read-back) is replayed for every batch */
    bool graph_mode = false;
    uint32_t max_walkers = 0;
    uint64_t max_cap = 0;
    cudaGraphExec_t exec = nullptr;
    char *h_stage = nullptr; /* pinned: jobs | schemes | header | status */
    /* per-request completion (serving): counters and status words on the
     * device, flags in mapped host memory (notify.count == nullptr: off); the
     * slot's requests are copied out on `copy`; job_ev holds the events the
     * slot's thread created (one per request in flight, reused) */
    BatchNotify notify;
    DevBuf notify_dev;        /* count[kMaxBatchJobs] | status[kMaxBatchJobs] */
    uint32_t *h_flag = nullptr;
    cudaStream_t copy = nullptr;
    std::vector<cudaEvent_t> job_ev;
    void release()
    {
        DevBuf *b[] = {&jobs, &small, &length, &path, &schemes, &notify_dev};
        for (DevBuf *x : b)
            x->release();
        if (copy)
        {
            cudaStreamSynchronize(copy);
            cudaStreamDestroy(copy);
        }
        copy = nullptr;
        for (cudaEvent_t ev_j : job_ev)
            cudaEventDestroy(ev_j);
        job_ev.clear();
        if (h_flag)
            cudaFreeHost(h_flag);
        h_flag = nullptr;
        notify = BatchNotify{};
        for (int i = 0; i < 3; i++)
            if (ev[i])
                cudaEventDestroy(ev[i]);
        ev[0] = ev[1] = ev[2] = nullptr;
        if (exec)
            cudaGraphExecDestroy(exec);
        exec = nullptr;
        if (h_stage)
            cudaFreeHost(h_stage);
        h_stage = nullptr;
    }
};

/* Pinned host blocks recycled by size class (powers of two from 64 KiB).
 * Reference-counted: the owner holds one reference and every block handed out
 * holds one, so blocks may be returned after the owner is gone. */
struct HostPool
{
    std::mutex m;
    std::vector<std::pair<size_t, void *>> free_blocks; /* (class bytes, block) */
    size_t cached = 0, limit = 0;
    int refs = 1;

    static size_t class_of(size_t bytes)
    {
        size_t c = 64 * 1024;
        while (c < bytes)
            c <<= 1;
        return c;
    }
    /* A block of at least `bytes`; its class in *cls. */
    void *get(size_t bytes, size_t *cls)
    {
        const size_t c = class_of(bytes);
        *cls = c;
        {
            std::lock_guard<std::mutex> lk(m);
            refs++;
            for (size_t i = 0; i < free_blocks.size(); i++)
                if (free_blocks[i].first == c)
                {
                    void *p = free_blocks[i].second;
                    free_blocks[i] = free_blocks.back();
                    free_blocks.pop_back();
                    cached -= c;
                    return p;
                }
        }
        void *p = nullptr;
        if (cudaHostAlloc(&p, c, cudaHostAllocDefault) != cudaSuccess)
        {
            cudaGetLastError();
            put(nullptr, 0);
            return nullptr;
        }
        return p;
    }
    /* Returns a block (nullptr: only the reference) and drops its reference. */
    void put(void *p, size_t cls)
    {
        bool last;
        {
            std::lock_guard<std::mutex> lk(m);
            if (p != nullptr)
            {
                if (cached + cls <= limit)
                {
                    free_blocks.push_back({cls, p});
                    cached += cls;
                    p = nullptr;
                }
            }
            last = --refs == 0;
        }
        if (p != nullptr)
            cudaFreeHost(p);
        if (last)
        {
            for (auto &b : free_blocks)
                cudaFreeHost(b.second);
            delete this;
        }
    }
    void release() { put(nullptr, 0); }
};

/* Pinned bytes the pool of kk_batch_walk's results keeps for reuse once the
 * caller has returned them (kk_paths_free). */
constexpr size_t kBatchPoolCache = (size_t)4 << 30;

/* Owner record of a kk_paths whose arrays live in one pooled block. */
struct PooledPaths
{
    HostPool *pool;
    void *block;
    size_t cls;
};

/* kk_walk_into's streamed copy-out of one walk whose path offsets are known
 * before it runs.  The walk counts finished walkers per segment of
 * 2^shift walkers (at most kMaxSegments segments); the host copies each
 * segment's lengths and paths out as soon as its flag is set, while the rest
 * of the walk goes on, instead of splitting the walk into launches (each of
 * which pays its own tail). */
constexpr uint32_t kMaxSegments = 256;
constexpr size_t kStatusBytes = 8192;  /* the mapped status block */
constexpr size_t kSegFlagAt = 1024;    /* segment flags: kMaxSegments words */
constexpr size_t kSegBoundAt = 2048;   /* segment path offsets: kMaxSegments + 1 */
struct SegmentSink
{
    /* the walk's path offsets d_off (n + 1, total vertices total) are final;
     * the walk is not launched yet */
    std::function<void(const uint64_t *d_off, uint32_t n, uint64_t total)> before;
    /* the walk is launched (event walked after it): copies every segment out
     * as it finishes, and whatever is left once walked has completed;
     * bound[k] = the path offset of segment k's first walker */
    std::function<void(const uint32_t *d_len, const uint32_t *d_path, uint32_t n, uint32_t shift, uint32_t nseg,
                       const volatile uint32_t *flag, const volatile uint64_t *bound, cudaEvent_t walked)>
        during;
    bool used = false;
};

struct RunSpec
{
    uint64_t seed = 1;
    walker_id_t walker_begin = 0;
    uint32_t walker_num = 0;
    const uint32_t *d_start = nullptr;
    uint32_t n_start = 0;
    bool fixed_cap = true;
    uint32_t cap = 1;        /* vertices per walker, fixed_cap */
    float const_ext = 0.0f;  /* !fixed_cap: constant extension probability */
    bool want_paths = true;
    /* the walk ends only by its extension or on an isolated start vertex
     * (built-in DeepWalk, PPR, node2vec): on a graph where no walker can
     * reach a dead end, every path length is known before the walk, and
     * the walk writes its paths packed */
    bool exact = false;
    bool packed_out = false; /* the caller packs the paths (or wants them packed) */
};

} // namespace kk

struct kk_engine
{
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;     /* where work is issued */
    cudaStream_t own_stream = nullptr; /* created with the engine */
    std::string err;

    /* graph */
    bool has_graph = false;
    /* the last file load: the whole call and its device part, host clocks
     * in ms */
    double load_total_ms = 0.0, load_device_ms = 0.0;
    /* the binary loader's readers: per reader two pinned blocks, a stream
     * and two events, made on the first untyped file load and kept */
    static constexpr int kReaders = 16;
    static constexpr size_t kReadBlock = (size_t)4 << 20;
    unsigned char *read_pinned = nullptr; /* kReaders x 2 x kReadBlock */
    cudaStream_t read_st[kReaders] = {};
    cudaEvent_t read_ev[kReaders][2] = {};
    uint32_t V = 0;
    uint64_t E = 0;
    int64_t *d_off = nullptr;
    uint32_t *d_nbr = nullptr;
    float *d_w = nullptr;
    uint8_t *d_type = nullptr;
    int sorted = -1; /* -1 unknown, 0 no, 1 adjacency sorted by neighbour */

    /* work buffers */
    kk::DevBuf alias, sum, ave, ra, scratch, vmask, path, length, path_off, caps, start, small, cub_tmp, packed, packed_off;

    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaStream_t side = nullptr; /* hub alias builds run here, joined by events */
    cudaStream_t hub = nullptr;  /* alias_streams 4: the hubs alone on this stream */
    cudaEvent_t ev_hub_join = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    /* vertices by degree, descending (cached per graph), and the alias-build
     * classes: tier[k] = number of vertices of degree > kAliasClassMax[k]
     * (k < 8) and tier[8] = number of degree > 0, so [0, n_hub) are the hubs,
     * [tier[c - 1], tier[c]) class c, [n_nz, V) isolated */
    kk::DevBuf order, rows; /* rows: RowDesc of each position of the order */
    uint32_t tier[kk::kTierBounds] = {};
    uint32_t n_hub = 0, n_nz = 0;
    kk::DevBuf alias_next; /* the classes' work counters */
    /* kk_walk_into in walker chunks (option into_chunks): chunk c + 1 walks
     * into the other output set (walk_set) while chunk c is packed and copied
     * to the caller's buffers on copy_stream */
    int walk_set = 0;
    int into_chunks = 6;
    kk::DevBuf path_x[2], length_x[2], path_off_x[2], caps_x[2]; /* output sets 1 and 2 */
    kk::DevBuf into_lens[3], into_off[3], into_offb[3], into_lenb[3], into_verts[3], into_cub[3];
    cudaStream_t copy_stream = nullptr;
    void *h_status = nullptr;      /* mapped pinned words for the walks' status and capacity reads */
    void *d_status_host = nullptr; /* the device address of h_status */
    /* streamed copy-out of the running walk (kk_walk_into; nullptr: none) and
     * its per-segment walker counters */
    kk::SegmentSink *seg_sink = nullptr;
    int into_stream = 1; /* option into_stream: 0 keeps the walker chunks */
    kk::DevBuf seg_count;
    /* kk_batch_walk: the jobs' packed offsets and first vertices, and the
     * pooled pinned blocks its results are handed out in (created on first
     * use; kk_paths_free returns a block) */
    kk::DevBuf batch_small, batch_rel;
    kk::HostPool *host_pool = nullptr;
    cudaEvent_t ev_walked[3] = {nullptr, nullptr, nullptr}, ev_copied[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_seg_copy = nullptr; /* after the last streamed segment copy issued */
    /* no walker can reach a vertex without out-edges except by starting on
     * one (every edge's target has out-edges); cached per graph */
    bool no_dead_ends = false, dead_ends_valid = false;
    /* kernels this library has launched on the engine's streams (CUDA-graph
     * replays not counted; kk_engine_launch_count) */
    std::atomic<uint64_t> launches{0};
    bool order_valid = false;
    kk::DevBuf vcur; /* vertex cursors (begin | degree << 40), cached per graph */
    bool vcur_valid = false;
    /* cursor_adjacency (option): uniform picks read a per-graph copy of the
     * adjacency holding each neighbour's cursor (16 B/edge), one dependent
     * random read per step instead of the offsets then the neighbour */
    int cursor_adjacency = 0;
    kk::DevBuf adjc;
    bool adjc_valid = false;
    float adjc_ms = 0.0f; /* time of its last build */
    /* node2vec adjacency test: 0 edge set (built once per graph), 1 binary
     * search of the sorted adjacency (option node2vec_adjacency) */
    int n2v_adjacency = 0;
    kk::DevBuf edge_set;
    uint64_t edge_set_nb = 0;
    bool edge_set_valid = false;
    kk::DevBuf schemes;    /* metapath schemes of the running job */
    kk::BatchSlot bslot;   /* where the synchronous batch calls run */
    bool vmask_valid = false;
    float alias_ms = 0.0f, walk_ms = 0.0f;
    /* Rejection trials allowed per walker step before the walk fails with
     * KK_ERR_TRIAL_LIMIT (bounds every device loop; a valid configuration with
     * acceptance probability 1e-5 exceeds it with probability ~e^-167). */
    uint32_t trial_limit = 1u << 24;
    /* walk scheduling (kk_engine_set_option): 0 one walker per thread
     * (measured faster on every workload), 1 persistent walker pool; pool
     * blocks per SM (0 = as many as fit) */
    int walk_schedule = 0;
    int walk_blocks_per_sm = 0;
    /* threads per block of the one-walker-per-thread and batch walk kernels
     * (option walk_block: 32..256, a multiple of 32) */
    int walk_block = 256;
    /* walkers per thread of the always-accepting first-order walks (option
     * walk_multi: 1, 2 or 4) */
    int walk_multi = 1;
    /* walk_park (option): first-order walks with rejection trials park the
     * walkers of a warp with fewer than this many lanes still walking and
     * resume them in kParkRounds later launches (0: no parking; default 20:
     * metapath S22 walk 19.3 -> 13.6 ms) */
    int walk_park = 20;
    kk::DevBuf park[2], park_count;
    /* regroup_interval (option): 0 off; k > 0 runs the walks of walk_static
     * scheduling that do not park in phases of k steps, each phase's walkers
     * sorted by the vertex they stand on (walk_regroup_kernel): records,
     * sort keys in and out, sort values, the sorted order, the counts */
    int regroup = 0;
    kk::DevBuf regroup_rec[2], regroup_key[2], regroup_val, regroup_perm, regroup_count;
    /* walk_stats (option): count trials, queries and binary-search probes of
     * the walks (kk_last_walk_stats) */
    int walk_stats = 0;
    /* kk_batch_submit: a batch is on the engine's batch slot until
     * kk_batch_wait (batch_wait: the wait itself is running) */
    bool batch_out = false, batch_wait = false;
    uint64_t last_stats[3] = {0, 0, 0};
    /* alias-table layout: 0 cursor buckets where the hooks allow them, 1 index
     * buckets always, 2 (default) 16 B neighbour buckets where the hooks allow
     * them (DeepWalk S22: build 2.50 -> 2.25 ms, walk 5.71 -> 5.06 ms) */
    int alias_layout = 2;
    /* alias_cache (option): keep the edge-weight alias tables of the built-in
     * apps across calls instead of rebuilding them per call as the reference
     * does (same tables either way).  alias_cached: layout the tables in
     * e->alias hold (0 cursor, 1 index), -1 none. */
    int alias_cache = 0;
    int alias_cached = -1;
    /* alias_hub_grid (option): blocks of the hub alias kernel (0: one per two
     * SMs); fewer leave more of the SMs to the classes on the main stream */
    int alias_hub_grid = 0;
    /* alias_streams (option): 1 every class but the hubs on the main stream,
     * 2 the classes of degree <= 128 after the hubs on the side stream, 3 the
     * classes of degree <= 512 (S22 lognormal build 2.69 -> 2.50 ms); 4 the
     * hubs alone on a third stream, the classes of degree <= 512 on the side
     * stream from the start (a hub row's pairing is a long chain of rounds
     * that the small classes need not wait for) */
    int alias_streams = 3;
    /* alias_small_lanes (option): 0 lane groups of 4 (degree 17..32) and 2
     * (1..16) per row; 1 groups of 2 and 1 */
    int alias_small_lanes = 0;
    /* l2_fetch_bytes (option): the context's cudaLimitMaxL2FetchGranularity
     * hint while the engine lives (0: left as found); the value found is put
     * back when the option returns to 0 and when the engine is destroyed. */
    int l2_fetch = 0;
    size_t l2_fetch_saved = 0;

    kk::GraphView view() const { return kk::GraphView{V, E, d_off, d_nbr, d_w, d_type}; }
    void free_graph();
};

namespace kk
{

/* One more kernel launched on the engine's streams (any host thread). */
inline void count_launch(kk_engine *e) { e->launches.fetch_add(1, std::memory_order_relaxed); }

/* n 32-bit words from src to the engine's mapped host words at word `at`,
 * written by a kernel on the engine's stream (no copy engine involved). */
void words_to_host(kk_engine *e, const uint32_t *src, int at, int n);
/* Resume launches after a parking walk; the last one parks nothing. */
constexpr int kParkRounds = 6;

/* The path offsets of segments 0..nseg (walker k << shift, the last one n)
 * into the mapped status block at kSegBoundAt, on the engine's stream. */
void segment_bounds_to_host(kk_engine *e, const uint64_t *off, uint32_t n, uint32_t shift, uint32_t nseg);

/* Runs f, turning the exceptions inside the engine into a status and the
 * engine's last-error message (no exception crosses the C-ABI). */
template <typename F>
kk_status guard(kk_engine *e, F f)
{
    try
    {
        if (e)
        {
            e->err.clear();
            if (e->batch_out && !e->batch_wait)
                fail(KK_ERR_INVALID_CONFIG, "a submitted batch is outstanding (kk_batch_wait first)");
        }
        f();
        return KK_OK;
    }
    catch (const Error &x)
    {
        if (e)
            e->err = x.msg;
        return x.status;
    }
    catch (const std::bad_alloc &)
    {
        if (e)
            e->err = "host allocation failed";
        return KK_ERR_OOM;
    }
    catch (const std::exception &x)
    {
        if (e)
            e->err = x.what();
        return KK_ERR_CUDA;
    }
}

/* Packs a walk's paths on the device: per-walker offsets and vertices
 * (engine.cu); returns the number of vertices. */
uint64_t pack_walk_paths(kk_engine *e, const WalkResult &r, uint64_t **d_off, uint32_t **d_verts);

inline void require_graph(const kk_engine *e)
{
    if (!e->has_graph)
        fail(KK_ERR_NO_GRAPH, "no graph loaded");
}

inline unsigned grid_for(const kk_engine *e, uint64_t n, unsigned block)
{
    uint64_t g = (n + block - 1) / block;
    if (g == 0)
        g = 1;
    if (g > 0x7fffffffULL)
        g = 0x7fffffffULL;
    return (unsigned)g;
}

/* Exclusive scan of n+1 uint64 values in place-ish: out[i] = sum(in[0..i)). */
void exclusive_scan_u64(kk_engine *e, const uint64_t *in, uint64_t *out, uint64_t n);
/* The same on stream st with temporary storage tmp. */
void exclusive_scan_u64(kk_engine *e, const uint64_t *in, uint64_t *out, uint64_t n, cudaStream_t st,
                        kk::DevBuf &tmp);

/* Sorts n (key, value) pairs by the low `bits` bits of the key (stable), on
 * the engine's stream: the regrouped walk's records by vertex. */
void sort_pairs_u32(kk_engine *e, const uint32_t *keys_in, uint32_t *keys_out, const uint32_t *vals_in,
                    uint32_t *vals_out, uint32_t n, int bits);

/* Vertices sorted by degree, descending, with the alias tiers (cached per graph). */
const uint32_t *vertex_order(kk_engine *e);

/* Vertex cursors, cached per graph. */
const uint64_t *vertex_cursors(kk_engine *e);
/* The cursor adjacency of the loaded graph (built once per graph). */
const uint4 *cursor_adjacency_of(kk_engine *e);
/* Whether no edge leads to a vertex without out-edges (cached per graph). */
bool graph_no_dead_ends(kk_engine *e);

/* The edge set the node2vec adjacency test reads (cached per graph), or an
 * empty view when the engine's node2vec_adjacency option asks for binary
 * search. */
EdgeSetView node2vec_edge_set(kk_engine *e);

/* Per-vertex OR of 1 << edge type (metapath.hpp:77-88), cached per graph. */
const uint8_t *metapath_vertex_masks(kk_engine *e);

/* A batch of walk jobs (batch.cu): the job table, the metapath schemes and
 * the batch's walker and path-slot totals. */
struct BatchPlan
{
    std::vector<BatchJob> jobs;
    std::vector<apps::MetaSchemes> schemes;
    uint32_t total = 0;
    uint64_t total_cap = 0;
    int app = 0;
    bool weighted = false;
};

/* Checks the jobs and lays out the batch (fails on mixed apps or weighting).
 * longest_first: the launch takes the jobs longest walk first (the shortest
 * makespan for a batch whose results are used together); else in job order
 * (served requests, each handed out as it ends). */
BatchPlan plan_batch(kk_engine *e, const kk_walk_opts *jobs, int n, bool longest_first = true);

/* Packs a finished batch's paths (job j's walker i at path[path_base_j + i *
 * cap_j], its length at length[first_task_j + i]; d_jobs the job table on the
 * device) into one buffer in job order, on the engine's stream (engine.cu):
 * *d_verts the packed vertices, *d_rel each walker's offset counted from its
 * job's first vertex, job_begin (host, one entry per job and one past the
 * last) the position of each job's first vertex in *d_verts. */
void pack_batch_paths(kk_engine *e, const BatchPlan &plan, const BatchJob *d_jobs, const uint32_t *length,
                      const uint32_t *path, const uint64_t **d_rel, const uint32_t **d_verts,
                      std::vector<uint64_t> &job_begin);

/* Everything a batch of the plan's app reads besides the graph, on the
 * engine's stream: the sorted adjacency (node2vec), the vertex type masks
 * (metapath), the alias tables in the layout the walk uses (weighted). */
void batch_prepare(kk_engine *e, const BatchPlan &plan);

/* Runs the batch on a slot, paths in HBM in the batch layout: job j's walker i
 * at path[path_base_j + i * cap_j], its length at length[first_task_j + i].
 * prepared: batch_prepare already ran for this app (the slot then only reads
 * the shared tables).  Returns the walker-steps; fails on a walk error. */
uint64_t run_batch(kk_engine *e, BatchPlan &plan, BatchSlot &slot, bool want_paths, bool prepared);

/* Puts a slot in CUDA-graph mode for batches of up to max_walkers walkers and
 * max_cap path vertices (batch_prepare must have run: the graph reads the
 * shared tables). */
void batch_slot_graph_mode(kk_engine *e, BatchSlot &slot, uint32_t max_walkers, uint64_t max_cap);

/* Gives a slot per-request completion (BatchNotify): each job of its batches
 * raises its own flag, with its own status, as its last walker ends.  Call
 * before the slot's first batch (a graph-mode slot captures the counters'
 * reset with its launch). */
void batch_slot_notify_mode(BatchSlot &slot);

/* run_batch in two halves for a prepared engine: batch_launch_async queues
 * the batch on the slot's stream (its end recorded in slot.ev[2]);
 * batch_finish waits for it and returns the walker-steps.  With per-request
 * completion, a failed walk is reported per job in its flag, not here. */
void batch_launch_async(kk_engine *e, BatchPlan &plan, BatchSlot &slot);
uint64_t batch_finish(kk_engine *e, BatchSlot &slot);

/* Metapath schemes of one job as per-state type masks, checked. */
inline apps::MetaSchemes make_schemes(const kk_walk_opts &o)
{
    if (o.n_schemes < 1 || o.n_schemes > KK_MAX_SCHEMES)
        fail(KK_ERR_INVALID_CONFIG, "metapath needs 1..16 schemes");
    apps::MetaSchemes sc;
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
    return sc;
}

/* One thread tier: blocks of NT vertices, a few resident per SM. */
/* Launches one alias class [lo, hi) with kernel `kern` of nt threads and
 * smem bytes of dynamic shared memory per block, as many blocks as fit on
 * every SM (at most one per `per_block` vertices). */
template <typename K>
void launch_alias_class(kk_engine *e, K kern, unsigned nt, size_t smem, uint32_t per_block, uint32_t lo, uint32_t hi,
                        int &resident, const std::function<void(unsigned)> &launch, int cap_per_sm = 0)
{
    if (hi <= lo)
        return;
    if (resident == 0)
    {
        /* the opt-in limit counts dynamic bytes only; static shared memory comes on top */
        KK_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        KK_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, (int)nt, smem));
        if (resident < 1)
            resident = 1;
    }
    const int per_sm = cap_per_sm > 0 && cap_per_sm < resident ? cap_per_sm : resident;
    const uint64_t want = (uint64_t)per_sm * (uint64_t)e->sm_count;
    const uint64_t need = ((uint64_t)(hi - lo) + per_block - 1) / per_block;
    launch((unsigned)(need < want ? need : want));
    KK_CUDA_CHECK(cudaGetLastError());
}

/* Builds alias tables in the Bucket layout into e->alias/e->sum for a
 * static functor: hubs on the side stream, the other classes in turn on the
 * main stream or (alias_streams) the small-row classes after the hubs on the
 * side stream, every class largest vertex first from its own counter. */
template <typename TC, typename Bucket = IndexBucket>
void build_alias(kk_engine *e, const TC &tc)
{
    constexpr bool weight_tables = std::is_same<typename TC::static_type, apps::WeightStatic>::value;
    const int layout = Bucket::cursor ? 0 : (Bucket::compact ? 2 : 1);
    if constexpr (weight_tables)
    {
        if (e->alias_cache && e->alias_cached == layout && tc.static_comp.w == e->d_w)
            return;
    }
    e->alias_cached = -1;
    GraphView g = e->view();
    Bucket *alias = e->alias.as<Bucket>(e->E);
    float *sum = e->sum.as<float>(e->V);
    const uint32_t *order = vertex_order(e);
    const RowDesc *rows = (const RowDesc *)e->rows.p;
    const uint64_t *vcur = Bucket::cursor ? vertex_cursors(e) : nullptr;
    uint2 *scratch = e->scratch.as<uint2>(2 * e->E);
    uint32_t *next = e->alias_next.as<uint32_t>(16);
    KK_CUDA_CHECK(cudaMemsetAsync(next, 0, 16 * sizeof(uint32_t), e->stream));
    const uint32_t *t = e->tier;
    cudaStream_t st = e->stream;
    const bool hub_alone = e->alias_streams == 4 && e->n_hub;
    cudaStream_t hub_st = hub_alone ? e->hub : e->side;
    KK_CUDA_CHECK(cudaEventRecord(e->ev_fork, e->stream));
    if (e->n_hub)
    {
        /* hubs first, largest first, on their own stream so they start at once */
        KK_CUDA_CHECK(cudaStreamWaitEvent(hub_st, e->ev_fork, 0));
        /* half the SMs by default: the hubs' serial sums and short batches use
         * few lanes, and the classes on the main stream get the other half */
        const uint32_t cap =
            e->alias_hub_grid > 0 ? (uint32_t)e->alias_hub_grid : (uint32_t)(e->sm_count > 1 ? e->sm_count / 2 : 1);
        const unsigned grid = e->n_hub < cap ? e->n_hub : cap;
        alias_build_hub_kernel<TC, Bucket><<<grid, 1024, 0, hub_st>>>(g, tc, alias, vcur, sum, scratch, order, 0,
                                                                      e->n_hub, next);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
    }
    /* 4097..16384: the hub kernel in 256-thread blocks */
    {
        static int res = 0;
        launch_alias_class(e, alias_build_hub_kernel<TC, Bucket>, 256, 0, 1, t[0], t[1], res, [&](unsigned grid) {
            alias_build_hub_kernel<TC, Bucket><<<grid, 256, 0, st>>>(g, tc, alias, vcur, sum, scratch, order, t[0],
                                                                     t[1], next + 1);
            count_launch(e);
        });
    }
    /* 2049..4096: a block per vertex, the row in shared memory */
    {
        static int res = 0;
        constexpr size_t smem = alias_block_row_smem<4096>();
        launch_alias_class(e, alias_block_row_kernel<TC, Bucket, 256, 4096>, 256, smem, 1, t[1], t[2], res,
                           [&](unsigned grid) {
                               alias_block_row_kernel<TC, Bucket, 256, 4096>
                                   <<<grid, 256, smem, st>>>(g, tc, alias, vcur, sum, order, t[1], t[2], next + 2);
                               count_launch(e);
                           });
    }
    /* 1..2048: lane groups, 32/G vertices per warp */
    auto group = [&](auto kern, uint32_t G, size_t smem_warp, int c, int &res, cudaStream_t s) {
        constexpr unsigned W = kAliasGroupWarps;
        const size_t smem = smem_warp * W;
        launch_alias_class(e, kern, 32 * W, smem, W * (32 / G), t[c - 1], t[c], res, [&](unsigned grid) {
            kern<<<grid, 32 * W, smem, s>>>(g, tc, alias, vcur, sum, rows, t[c - 1], t[c], next + c);
            count_launch(e);
        });
    };
    /* alias_streams 2: the classes of degree <= 128 (2.5 to 5 KB of shared
     * memory per warp) follow the hubs on the side stream and share the SMs
     * with the classes of large rows (10 to 48 KB per warp or block); 3: the
     * class 129..512 with them */
    const bool split = e->alias_streams >= 2;
    cudaStream_t light = st;
    if (split)
    {
        if (!e->n_hub || hub_alone)
            KK_CUDA_CHECK(cudaStreamWaitEvent(e->side, e->ev_fork, 0));
        light = e->side;
    }
    static int r3 = 0, r4 = 0, r5 = 0, r6 = 0, r7 = 0, r8 = 0;
    group(alias_group_kernel<TC, Bucket, 32, 2048>, 32, alias_group_smem_per_warp<32, 2048>(), 3, r3, st);
    group(alias_group_kernel<TC, Bucket, 32, 1024>, 32, alias_group_smem_per_warp<32, 1024>(), 4, r4, st);
    group(alias_group_kernel<TC, Bucket, 16, 512>, 16, alias_group_smem_per_warp<16, 512>(), 5, r5,
          e->alias_streams >= 3 ? light : st);
    group(alias_group_kernel<TC, Bucket, 8, 128>, 8, alias_group_smem_per_warp<8, 128>(), 6, r6, light);
    if (e->alias_small_lanes == 0)
    {
        group(alias_group_kernel<TC, Bucket, 4, 32>, 4, alias_group_smem_per_warp<4, 32>(), 7, r7, light);
        group(alias_group_kernel<TC, Bucket, 2, 16>, 2, alias_group_smem_per_warp<2, 16>(), 8, r8, light);
    }
    else
    {
        /* half the lanes per row: more rows per warp, each row's sum on its own lane */
        static int r7h = 0, r8h = 0;
        group(alias_group_kernel<TC, Bucket, 2, 32>, 2, alias_group_smem_per_warp<2, 32>(), 7, r7h, light);
        group(alias_group_kernel<TC, Bucket, 1, 16>, 1, alias_group_smem_per_warp<1, 16>(), 8, r8h, light);
    }
    if (e->n_hub || split)
    {
        KK_CUDA_CHECK(cudaEventRecord(e->ev_join, e->side));
        KK_CUDA_CHECK(cudaStreamWaitEvent(e->stream, e->ev_join, 0));
    }
    if (hub_alone)
    {
        KK_CUDA_CHECK(cudaEventRecord(e->ev_hub_join, e->hub));
        KK_CUDA_CHECK(cudaStreamWaitEvent(e->stream, e->ev_hub_join, 0));
    }
    if constexpr (weight_tables)
    {
        if (tc.static_comp.w == e->d_w)
            e->alias_cached = layout;
    }
}

/* A regrouped walk (option regroup_interval = k): phases of k steps, each
 * phase's walkers in the order of the vertices they stand on
 * (walk_regroup_kernel).  After each phase the host reads how many walkers
 * are still walking (through the mapped status words, no copy engine) and
 * sorts exactly those records by vertex.  Every phase moves each walker it
 * holds by at least k steps or ends it, and a walk ends within its path
 * capacity or its trial limit, so the phases are bounded. */
template <typename S, typename WC, typename TC, typename Bucket>
void walk_regrouped(kk_engine *e, const GraphView &g, const WC &wc, const TC &tc, const Bucket *alias,
                    const float *ra, const WalkLaunch &L)
{
    typedef ParkedWalker<S> PW;
    const uint32_t n = L.walker_num;
    PW *rec[2] = {e->regroup_rec[0].as<PW>(n), e->regroup_rec[1].as<PW>(n)};
    uint32_t *key = e->regroup_key[0].as<uint32_t>(n), *key_sorted = e->regroup_key[1].as<uint32_t>(n);
    uint32_t *val = e->regroup_val.as<uint32_t>(n), *perm = e->regroup_perm.as<uint32_t>(n);
    uint32_t *cnt = e->regroup_count.as<uint32_t>(2);
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)g.V)
        bits++;
    const unsigned bs = (unsigned)e->walk_block;
    const uint32_t k = (uint32_t)e->regroup;
    const PW *in = nullptr;
    uint32_t left = n;
    for (int ph = 0; left > 0; ph++)
    {
        const int o = ph & 1;
        KK_CUDA_CHECK(cudaMemsetAsync(cnt + o, 0, sizeof(uint32_t), e->stream));
        walk_regroup_kernel<S, WC, TC, Bucket><<<grid_for(e, left, bs), bs, 0, e->stream>>>(
            g, wc, tc, alias, ra, L, in, perm, cnt + (o ^ 1), rec[o], key, val, cnt + o, k);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        words_to_host(e, cnt + o, 44, 1);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        left = ((volatile uint32_t *)e->h_status)[44];
        if (left > 0)
            sort_pairs_u32(e, key, key_sorted, val, perm, left, bits);
        in = rec[o];
    }
}

/* One walk over walkers [rs.walker_begin, + rs.walker_num): alias tables,
 * regular area, path capacity, the walk kernel.  Events: ev0 before the alias
 * build, ev1 before the walk, ev2 after. */
template <typename S, typename WC, typename TC, typename Bucket>
void run_walk_with(kk_engine *e, const WC &wc, const TC &tc, const RunSpec &rs, WalkResult &res)
{
    GraphView g = e->view();
    if constexpr (!TC::has_static)
    {
        if (e->cursor_adjacency)
            g.adjc = cursor_adjacency_of(e);
    }
    uint32_t n = rs.walker_num;
    int *d_status = (int *)e->small.ensure(64);
    unsigned long long *d_steps = (unsigned long long *)((char *)d_status + 16);
    KK_CUDA_CHECK(cudaMemsetAsync(d_status, 0, 64, e->stream));
    KK_CUDA_CHECK(cudaEventRecord(e->ev[0], e->stream));
    const Bucket *alias = nullptr;
    const float *ra = nullptr;
    if constexpr (TC::has_static)
    {
        build_alias<TC, Bucket>(e, tc);
        alias = (const Bucket *)e->alias.p;
    }
    if constexpr (TC::has_outlier)
    {
        float *rap = e->ra.as<float>(e->V);
        regular_area_kernel<TC><<<grid_for(e, g.V, 256), 256, 0, e->stream>>>(g, tc, (const float *)e->sum.p, rap);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        ra = rap;
    }
    WalkLaunch L;
    L.seed = rs.seed;
    L.walker_begin = rs.walker_begin;
    L.walker_num = n;
    L.start = rs.d_start;
    L.n_start = rs.n_start;
    L.total_steps = d_steps;
    L.alias_sum = (const float *)e->sum.p;
    L.status = d_status;
    L.trial_limit = e->trial_limit;
    L.stats = e->walk_stats ? (unsigned long long *)((char *)d_status + 24) : nullptr;
    /* the walk's output set (two sets let a chunked kk_walk_into walk one
     * chunk while the previous one is packed and copied out) */
    const int ws = e->walk_set;
    kk::DevBuf &b_length = ws ? e->length_x[ws - 1] : e->length, &b_caps = ws ? e->caps_x[ws - 1] : e->caps;
    kk::DevBuf &b_off = ws ? e->path_off_x[ws - 1] : e->path_off, &b_path = ws ? e->path_x[ws - 1] : e->path;
    L.length = b_length.as<uint32_t>(n);
    uint64_t total_cap;
    const bool exact = rs.exact && rs.packed_out && rs.want_paths && graph_no_dead_ends(e);
    uint32_t seg_shift = 0, nseg = 0, *seg_count = nullptr;
    if (rs.fixed_cap && !exact)
    {
        L.path_off = nullptr;
        L.cap = rs.cap;
        total_cap = (uint64_t)n * rs.cap;
    }
    else
    {
        uint64_t *caps = b_caps.as<uint64_t>((uint64_t)n + 1);
        uint64_t *off = b_off.as<uint64_t>((uint64_t)n + 1);
        KK_CUDA_CHECK(cudaMemsetAsync(caps + n, 0, sizeof(uint64_t), e->stream));
        if (!rs.fixed_cap)
        {
            /* the extension bound; a walker on an isolated start gets its one
             * vertex here, with no draws (its walk ends there at once: a bound
             * that is exact, packed paths or not) */
            constant_extension_bound_kernel<<<grid_for(e, n, 256), 256, 0, e->stream>>>(
                g, true, rs.d_start, rs.n_start, rs.seed, rs.walker_begin, n, rs.const_ext, 1u << 24, caps,
                d_status);
            count_launch(e);
            KK_CUDA_CHECK(cudaGetLastError());
        }
        if (exact && rs.fixed_cap)
        {
            /* the full capacity, and one vertex for a walker on an isolated
             * start */
            exact_caps_kernel<<<grid_for(e, n, 256), 256, 0, e->stream>>>(g, rs.d_start, rs.n_start, rs.walker_begin,
                                                                          n, rs.cap, caps);
            count_launch(e);
            KK_CUDA_CHECK(cudaGetLastError());
        }
        exclusive_scan_u64(e, caps, off, (uint64_t)n + 1);
        words_to_host(e, (const uint32_t *)(off + n), 32, 2); /* host words 32, 33 of the 64 */
        if (exact && e->seg_sink != nullptr && n > 0)
        {
            /* streamed copy-out: segments of 2^shift >= 4096 walkers, at most
             * kMaxSegments of them; flags cleared before the walk can set any */
            seg_shift = 12;
            while ((((uint64_t)n + (1ull << seg_shift) - 1) >> seg_shift) > kMaxSegments)
                seg_shift++;
            nseg = (uint32_t)(((uint64_t)n + (1ull << seg_shift) - 1) >> seg_shift);
            memset((char *)e->h_status + kSegFlagAt, 0, (size_t)nseg * 4);
            seg_count = e->seg_count.as<uint32_t>(kMaxSegments);
            KK_CUDA_CHECK(cudaMemsetAsync(seg_count, 0, (size_t)nseg * 4, e->stream));
            segment_bounds_to_host(e, off, n, seg_shift, nseg);
        }
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        total_cap = ((volatile uint64_t *)e->h_status)[16];
        L.path_off = off;
        L.cap = 0;
        if (nseg > 0)
        {
            e->seg_sink->before(off, n, total_cap);
            L.seg_count = seg_count;
            L.seg_flag = (volatile uint32_t *)((char *)e->d_status_host + kSegFlagAt);
            L.seg_shift = seg_shift;
        }
    }
    L.path = rs.want_paths ? b_path.as<uint32_t>(total_cap) : nullptr;
    KK_CUDA_CHECK(cudaEventRecord(e->ev[1], e->stream));
    if constexpr (TC::order == 1 && !TC::has_dynamic)
    {
        if (e->walk_schedule == 0 && e->walk_multi > 1 && e->regroup == 0)
        {
            /* W walkers per thread, gathers of all W in flight together */
            const unsigned bs = (unsigned)e->walk_block;
            const uint64_t threads = ((uint64_t)n + e->walk_multi - 1) / e->walk_multi;
            if (e->walk_multi == 2)
                walk_multi_kernel<S, WC, TC, Bucket, 2><<<grid_for(e, threads, bs), bs, 0, e->stream>>>(g, wc, tc,
                                                                                                       alias, L);
            else
                walk_multi_kernel<S, WC, TC, Bucket, 4><<<grid_for(e, threads, bs), bs, 0, e->stream>>>(g, wc, tc,
                                                                                                       alias, L);
            count_launch(e);
            goto launched;
        }
    }
    if (e->walk_schedule == 0 && e->regroup > 0 && !(parks<TC>() && e->walk_park > 0) && n > 0)
    {
        walk_regrouped<S, WC, TC, Bucket>(e, g, wc, tc, alias, ra, L);
        goto launched;
    }
    if (e->walk_schedule == 0)
    {
        const unsigned bs = (unsigned)e->walk_block;
        if constexpr (parks<TC>())
        {
            if (e->walk_park > 0 && n > 0)
            {
                /* the first launch parks the stragglers of thinned-out warps
                 * into queue 0; each resume round runs one queue 32 walkers
                 * to a warp and parks into the other, the last round parks
                 * nothing */
                typedef ParkedWalker<S> PW;
                PW *q[2] = {e->park[0].as<PW>(n), e->park[1].as<PW>(n)};
                uint32_t *cnt = e->park_count.as<uint32_t>(2);
                KK_CUDA_CHECK(cudaMemsetAsync(cnt, 0, 2 * sizeof(uint32_t), e->stream));
                WalkLaunch Lp = L;
                Lp.park = q[0];
                Lp.park_count = cnt;
                Lp.park_below = (uint32_t)e->walk_park;
                walk_static_kernel<S, WC, TC, Bucket><<<grid_for(e, n, bs), bs, 0, e->stream>>>(g, wc, tc, alias, ra,
                                                                                               Lp);
                count_launch(e);
                const unsigned rgrid = (unsigned)e->sm_count * (1024u / bs);
                for (int r = 0; r < kParkRounds; r++)
                {
                    const int cur = r & 1, nxt = cur ^ 1;
                    KK_CUDA_CHECK(cudaMemsetAsync(cnt + nxt, 0, sizeof(uint32_t), e->stream));
                    WalkLaunch Lr = L;
                    if (r + 1 < kParkRounds)
                    {
                        Lr.park = q[nxt];
                        Lr.park_count = cnt + nxt;
                        Lr.park_below = (uint32_t)e->walk_park;
                    }
                    walk_resume_kernel<S, WC, TC, Bucket><<<rgrid, bs, 0, e->stream>>>(g, wc, tc, alias, ra, Lr,
                                                                                      q[cur], cnt + cur);
                    count_launch(e);
                }
                goto launched;
            }
        }
        walk_static_kernel<S, WC, TC, Bucket><<<grid_for(e, n, bs), bs, 0, e->stream>>>(g, wc, tc, alias, ra, L);
        count_launch(e);
    }
    else
    {
        /* persistent walker pool: blocks_per_sm resident blocks on every SM */
        static int resident = 0;
        if (resident == 0)
            KK_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, walk_pool_kernel<S, WC, TC, Bucket>, 256, 0));
        int per_sm = e->walk_blocks_per_sm > 0 && e->walk_blocks_per_sm < resident ? e->walk_blocks_per_sm : resident;
        uint64_t want = (uint64_t)e->sm_count * (per_sm > 0 ? per_sm : 1);
        uint64_t need = ((uint64_t)n + 255) / 256;
        unsigned grid = (unsigned)(want < need ? want : (need ? need : 1));
        walk_pool_kernel<S, WC, TC, Bucket><<<grid, 256, 0, e->stream>>>(g, wc, tc, alias, ra, L);
        count_launch(e);
    }
launched:
    KK_CUDA_CHECK(cudaGetLastError());
    KK_CUDA_CHECK(cudaEventRecord(e->ev[2], e->stream));
    if (nseg > 0)
    {
        e->seg_sink->used = true;
        e->seg_sink->during(L.length, L.path, n, seg_shift, nseg,
                            (const volatile uint32_t *)((const char *)e->h_status + kSegFlagAt),
                            (const volatile uint64_t *)((const char *)e->h_status + kSegBoundAt), e->ev[2]);
    }
    words_to_host(e, (const uint32_t *)d_status, 0, 16);
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    int h_small[16];
    memcpy(h_small, e->h_status, sizeof(h_small));
    memcpy(e->last_stats, (char *)h_small + 24, sizeof(e->last_stats));
    KK_CUDA_CHECK(cudaEventElapsedTime(&e->alias_ms, e->ev[0], e->ev[1]));
    KK_CUDA_CHECK(cudaEventElapsedTime(&e->walk_ms, e->ev[1], e->ev[2]));
    if (h_small[0] & KK_STATUS_BAD_START) /* first: it can cause the others */
        fail(KK_ERR_INVALID_CONFIG, "start vertex >= v_num");
    if (h_small[0] & KK_STATUS_TRIAL_LIMIT)
        fail(KK_ERR_TRIAL_LIMIT, "a walker exceeded the rejection-trial limit");
    if (h_small[0] & KK_STATUS_PATH_CAPACITY)
        fail(KK_ERR_PATH_CAPACITY, "a walk exceeded its path capacity");
    unsigned long long steps;
    memcpy(&steps, (char *)h_small + 16, sizeof(steps));
    res.walker_num = n;
    res.packed = exact;
    res.length = L.length;
    res.path_off = L.path_off;
    res.cap = L.cap;
    res.path = L.path;
    res.total_steps = steps;
}

/* Runs a walk with the alias-table layout the engine's alias_layout option
 * picks: where no hook reads the taken edge's index, cursor buckets (0) or
 * 16 B neighbour buckets (2); else index buckets. */
template <typename S, typename WC, typename TC>
void run_walk(kk_engine *e, const WC &wc, const TC &tc, const RunSpec &rs, WalkResult &res)
{
    if constexpr (use_cursor_buckets<WC, TC>())
    {
        if (e->alias_layout == 0)
        {
            run_walk_with<S, WC, TC, CursorBucket>(e, wc, tc, rs, res);
            return;
        }
    }
    if constexpr (use_neighbour_buckets<WC, TC>())
    {
        if (e->alias_layout == 2)
        {
            run_walk_with<S, WC, TC, NeighbourBucket>(e, wc, tc, rs, res);
            return;
        }
    }
    run_walk_with<S, WC, TC, IndexBucket>(e, wc, tc, rs, res);
}

/* The built-in apps (apps_*.cu). */
void run_app_first_order(kk_engine *e, const kk_walk_opts &o, const RunSpec &rs, WalkResult &res);
void run_app_node2vec(kk_engine *e, const kk_walk_opts &o, const RunSpec &rs, WalkResult &res);

/* Graph helpers (graph.cu). */
void graph_check_sorted(kk_engine *e);
void graph_sort_adjacency(kk_engine *e);

/* Runs one epoch of a walk: fills the WalkResult for rs's walkers. */
typedef std::function<void(const RunSpec &, WalkResult &)> EpochRunner;

/* kk_walk's epoch loop, path packing and copy-out, with `custom` (non-null)
 * running a user's hooks instead of a built-in app (engine.cu). */
kk_status walk_to_host(kk_engine *e, const kk_walk_opts *opts, kk_paths **out, const EpochRunner *custom);

/* random_walk() with user-defined hooks (include/walk.hpp:423-436): the
 * reference's WalkEngine::random_walk(WalkerConfig*, TransitionConfig*,
 * WalkConfig*) for a graph already in the engine.  opts supplies the walker
 * range, seed, start list and epoch rate; opts->walk_length bounds every walk
 * (path capacity walk_length + 1 vertices; a longer walk fails with
 * KK_ERR_PATH_CAPACITY).  Returns the paths like kk_walk. */
template <typename S, typename WC, typename TC>
kk_status random_walk(kk_engine *e, const WC &wc, const TC &tc, const kk_walk_opts &opts, kk_paths **out)
{
    EpochRunner run = [&](const RunSpec &rs, WalkResult &res) { run_walk<S>(e, wc, tc, rs, res); };
    return walk_to_host(e, &opts, out, &run);
}

} // namespace kk
