/*
 * knightking_gb300: C-ABI of the GB300 walker-step engine.
 *
 * Drop-in replacement, on one GPU, for KnightKing's WalkEngine::random_walk()
 * path (include/walk.hpp:423-436 of the reference) and the graph/path plumbing
 * around it.  Plain C types only; every call returns a kk_status and never
 * throws.  Paths are bit-identical to the reference's sampler fed the same
 * counter-based Philox stream (see KK_RNG_* below).
 *
 * Threading: one engine is driven by one host thread at a time.
 */
#ifndef KNIGHTKING_GB300_H
#define KNIGHTKING_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference asserts or exits instead) ------------- */
typedef int kk_status;
#define KK_OK 0
#define KK_ERR_INVALID_CONFIG 1 /* include/walk.hpp:251-261 asserts, bad sizes */
#define KK_ERR_OOM 2
#define KK_ERR_IO 3           /* include/storage.hpp:39 assert, include/graph.hpp:427 exit */
#define KK_ERR_TRIAL_LIMIT 4  /* a walker exceeded the rejection-trial cap */
#define KK_ERR_TIMEOUT 5
#define KK_ERR_CUDA 6
#define KK_ERR_NO_GRAPH 7
#define KK_ERR_PATH_CAPACITY 8

/* ---- edge kinds of the binary edge-list file (include/type.hpp:43-85) --- */
#define KK_EDGE_UNWEIGHTED 0   /* Edge<EmptyData>:          {u32 src, u32 dst}           8 B */
#define KK_EDGE_F32 1          /* Edge<real_t>:             {u32 src, u32 dst, f32 w}   12 B */
#define KK_EDGE_META 2         /* Edge<UnweightedMetaData>: {u32 src, u32 dst, i32 type} 12 B */
#define KK_EDGE_META_F32 3     /* Edge<WeightedMetaData>:   {src, dst, f32 w, i32 type}  16 B */

/* ---- built-in apps (the reference's src/apps functors) ------------------ */
#define KK_APP_DEEPWALK 0  /* src/apps/deepwalk.hpp:30-47 */
#define KK_APP_PPR 1       /* src/apps/ppr.hpp:30-64 */
#define KK_APP_NODE2VEC 2  /* src/apps/node2vec.hpp:108-202 */
#define KK_APP_METAPATH 3  /* src/apps/metapath.hpp:70-128 */

#define KK_MAX_SCHEMES 16
#define KK_MAX_SCHEME_LEN 16

/* Random stream: Philox4x32-10, key = seed, counter = (walker id, step,
 * draw >> 2, stream), word draw & 3.  Streams: */
#define KK_RNG_STREAM_WALK 0
#define KK_RNG_STREAM_INIT_STATE 1
#define KK_RNG_STREAM_INIT_DIST 2

typedef struct kk_engine kk_engine;

/* Options of one random_walk() call: the union of WalkConfig
 * (include/walk.hpp:105-145), WalkerConfig (:147-193) and the apps' confs. */
typedef struct
{
    int app;          /* KK_APP_* */
    int weighted;     /* static component = edge weight (alias sampling) */
    uint64_t seed;    /* Philox key */
    uint32_t walker_num;
    uint32_t walker_begin;   /* first walker id (ids are walker_begin + i) */
    uint32_t walk_length;    /* DeepWalk / node2vec / metapath */
    float terminate_prob;    /* PPR (extension = 1 - terminate_prob) */
    float p, q;              /* node2vec */
    int n_schemes;           /* metapath: schemes as per-state edge-type masks */
    int scheme_len[KK_MAX_SCHEMES];
    uint8_t scheme_mask[KK_MAX_SCHEMES][KK_MAX_SCHEME_LEN];
    int scheme_round_robin;  /* 0: scheme = gen(n_schemes) on stream 1 (metapath.hpp:91-95); 1: id % n */
    const uint32_t *start;   /* optional host start-vertex list (ppr.hpp:37-51); NULL: id % V */
    uint32_t n_start;
    double rate;             /* WalkConfig::set_walk_rate (-r), epochs of walker_num*rate walkers; 0 = 1 */
} kk_walk_opts;

/* Paths of one call, host memory, in walker-id order.  Walker i (id
 * walker_begin + i) has length[i] vertices at vertices[offset[i]...]. */
typedef struct
{
    uint32_t walker_num;
    uint32_t walker_begin;
    uint32_t epoch_walkers;  /* walkers per epoch of the call (walker_num when rate = 1) */
    uint64_t total_steps;    /* sum(length) - walker_num: walker-steps taken */
    uint32_t *length;
    uint64_t *offset;
    uint32_t *vertices;
    void *owner; /* library-internal: who holds the three arrays (NULL: malloc) */
} kk_paths;

/* ---- engine ------------------------------------------------------------- */

/* WalkEngine() (include/walk.hpp:378-381): binds CUDA device `device`. */
kk_status kk_engine_create(kk_engine **out, int device);
void kk_engine_destroy(kk_engine *e);
/* Runs the engine's work on `stream` (a cudaStream_t; NULL restores the
 * engine's own stream), so a caller can order and time it with its events. */
kk_status kk_engine_set_stream(kk_engine *e, void *stream);
/* Tuning knobs (results never change, only speed).  No counterpart in the
 * reference, whose CPU scheduling constants are compile-time macros
 * (include/constants.hpp:27-46):
 *   "walk_schedule"      0 one walker per thread (default), 1 persistent walker pool
 *   "walk_blocks_per_sm" pool blocks per SM, 0 = as many as fit (default)
 *   "walk_block"         threads per block of the walk kernels, 32..256 step 32 (default 256)
 *   "trial_limit"        rejection trials per step before KK_ERR_TRIAL_LIMIT (default 2^24)
 *   "alias_layout"       0 cursor buckets where no hook reads the taken edge's index
 *                        (a step reads one 32 B bucket), 1 index buckets always, 2 (default) 16 B
 *                        neighbour buckets where no hook reads the edge index (half the bytes to build)
 *   "alias_cache"        1 keeps the built-in apps' edge-weight alias tables across calls
 *                        (the reference rebuilds them per call; the tables are the same)
 *   "node2vec_adjacency" 0 edge-set lookup (built once per graph), 1 binary search of the
 *                        sorted adjacency, as node2vec.hpp:159-166
 *   "l2_fetch_bytes"     the context's cudaLimitMaxL2FetchGranularity while the engine
 *                        lives: 32, 64, 128, or 0 for the value found (restored on destroy)
 *   "walk_stats"         1 counts trials, queries and probes (kk_last_walk_stats)
 *   "walk_multi"         walkers per thread (1, 2, 4) of first-order walks without a dynamic component
 *   "walk_park"          first-order walks with a dynamic component (rejection trials), one walker per
 *                        thread: once fewer than this many lanes of a warp are walking, its walkers stop
 *                        at their next step boundary and later launches resume them 32 to a warp
 *                        (0 off, 1..32; default 20)
 *   "alias_hub_grid"     blocks of the hub alias kernel (0: one per two SMs)
 *   "alias_streams"      1 the alias classes of degree <= 16384 in turn on the engine's stream,
 *                        2 those of degree <= 128 after the hubs on a second stream, beside the rest,
 *                        3 (default) those of degree <= 512, 4 those of degree <= 512 on the second
 *                        stream from the start and the hubs alone on a third
 *   "alias_small_lanes"  0 (default) lane groups of 4 and 2 per row for the alias rows of degree
 *                        17..32 and 1..16; 1 groups of 2 and 1
 *   "into_stream"        1 (default): kk_walk_into walks whose path lengths are known before they
 *                        run (DeepWalk, PPR, node2vec on graphs without reachable dead ends) in one
 *                        launch per epoch and copies each segment of walkers out as soon as its
 *                        last walker finishes; 0: walker chunks for every walk (into_chunks)
 *   "into_chunks"        kk_walk_into walks that are not streamed (metapath excepted: one chunk) run in
 *                        up to this many walker chunks (>= 2^18 walkers each), copying each chunk's
 *                        paths out while the next chunk walks (default 6; 1 = whole)
 *   "cursor_adjacency"   1 uniform picks read a per-graph adjacency copy holding each neighbour's
 *                        position (16 B/edge, built on first use): one dependent read per step
 *   "regroup_interval"   0 (default) off; k > 0: single-job walks of the one-walker-per-thread schedule
 *                        that do not park run in phases of k steps, and each phase takes its walkers
 *                        sorted by the vertex they stand on (0..4096) */
kk_status kk_engine_set_option(kk_engine *e, const char *name, int64_t value);
/* Message of the last failed call on this engine ("" if none). */
const char *kk_last_error(const kk_engine *e);
/* Message for a status code. */
const char *kk_status_string(kk_status s);

/* ---- graph (GraphEngine::load_graph, include/graph.hpp:408-530) --------- */

/* Reads the reference's binary edge-list file (include/storage.hpp:35-55),
 * optionally mirrors every edge (--make-undirected, include/graph.hpp:430-443),
 * and builds the CSR in HBM with file order kept per source
 * (include/graph.hpp:309-330).  Untyped files are streamed to the device by
 * up to 16 host threads; the engine's first such load allocates 128 MiB of
 * pinned host memory for them (two 4 MiB buffers per thread), kept until
 * kk_engine_destroy.  A refused file (an endpoint >= v_num, a type outside
 * [0, 8)) leaves the engine's graph as it was. */
kk_status kk_graph_load_binary(kk_engine *e, uint32_t v_num, const char *path, int edge_kind, int make_undirected);

/* Reads a text edge list (read_edge_txt, include/storage.hpp:107-115): one
 * "src dst" (weighted = 0) or "src dst weight" (weighted = 1) per line, '#' or
 * '%' lines are comments, any other malformed line fails with KK_ERR_IO; then
 * as kk_graph_load_binary. */
kk_status kk_graph_load_text(kk_engine *e, uint32_t v_num, const char *path, int weighted, int make_undirected);
/* Timing of the engine's last kk_graph_load_binary / kk_graph_load_text call
 * (host clocks, ms): the whole call, and its device part.  For untyped binary
 * files the records are read and copied to the device in overlapped blocks,
 * and the device part runs from the records in HBM to the CSR (split and
 * mirror, stable sort by source, offsets, unpack); for text and typed files
 * the host splits the edges into columns, and the device part runs from their
 * copy to the device to the CSR.  No counterpart in the reference. */
kk_status kk_graph_load_timing(const kk_engine *e, double *total_ms, double *device_ms);

/* gconverter (src/tools/gconverter.cpp:69-100): a text edge list to the
 * binary Edge<T> file; *edges (nullable) gets the edge count.  Host only. */
kk_status kk_text_to_binary(const char *text_path, const char *binary_path, int weighted, uint64_t *edges);

/* read_metapath_schemes (src/apps/metascheme.hpp:69-98): a scheme file
 * ("schemes types", then per scheme its length and length x types 0/1 flags)
 * into opts' n_schemes / scheme_len / scheme_mask.  Host only. */
kk_status kk_read_metapath_schemes(const char *path, kk_walk_opts *opts);

/* Uploads a host CSR: off[V+1] int64, nbr[E], w[E] (nullable), type[E] (nullable). */
kk_status kk_graph_load_arrays(kk_engine *e, uint32_t v_num, uint64_t e_num, const int64_t *off,
                               const uint32_t *nbr, const float *w, const uint8_t *type);

/* Seeded R-MAT graph generated in HBM: edge_factor*2^scale draws with quadrant
 * probabilities a, b, c; self-loops dropped, pairs deduplicated and mirrored,
 * adjacency sorted.  weights: 0 none, 1 uniform [1,5), 2 lognormal(0,1);
 * types: number of edge types (0 = none). */
kk_status kk_graph_generate_rmat(kk_engine *e, uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                                 uint64_t seed, int weights, int types);

kk_status kk_graph_info(const kk_engine *e, uint32_t *v_num, uint64_t *e_num, int *has_weights, int *has_types);

/* Copies the device CSR to host arrays (any pointer may be NULL). */
kk_status kk_graph_download(kk_engine *e, int64_t *off, uint32_t *nbr, float *w, uint8_t *type);

/* node2vec needs each adjacency sorted by neighbour (src/apps/node2vec.hpp:122-125);
 * kk_walk sorts on demand, this does it eagerly.  In place, on the device. */
kk_status kk_graph_sort_adjacency(kk_engine *e);

/* ---- alias tables (init_alias_tables, include/walk.hpp:538-652) --------- */

/* Builds the alias tables of the static component w on the GPU and copies
 * them out: bucket j of vertex v at off[v]+j holds (p, p_idx, q_idx) with
 * indices local to v's adjacency (q_idx = 0xffffffff: no alias), and sum[v]
 * the sequential float sum of v's weights.  Outputs are host arrays. */
kk_status kk_alias_build(kk_engine *e, float *p, uint32_t *p_idx, uint32_t *q_idx, float *sum);

/* Alias tables built with no device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc (for example a serving process whose device memory belongs to
 * its own pool, or a latency-critical path where allocation and the device
 * synchronisation of cudaFree are not allowed).  The caller passes its own
 * device arrays: off[v_num+1] and w[E] in, p/p_idx/q_idx[E] and sum[v_num]
 * (sum may be NULL) out, in the layout of kk_alias_build, with the same
 * values bit for bit.  Its queue scratch is a fixed 32 MiB device array inside
 * the library that every GPU which loads the library keeps until the process
 * exits; a vertex degree above 16384 is rejected with KK_ERR_INVALID_CONFIG.
 * The first call on a device looks up that array's address; the work is
 * queued on `stream` (a cudaStream_t, NULL = default stream) after a short
 * degree check that synchronises the stream, so no call can be made while its
 * stream is being captured into a CUDA graph.
 * Calls share the scratch: calls that overlap on the GPU race. */
kk_status kk_alias_build_noalloc(uint32_t v_num, const int64_t *d_off, const float *d_w, float *d_p,
                                 uint32_t *d_p_idx, uint32_t *d_q_idx, float *d_sum, void *stream);

/* ---- walks (WalkEngine::random_walk, include/walk.hpp:423-436) ---------- */

/* Runs one walk job and returns its paths in host memory (free with
 * kk_paths_free).  Epochs (opts->rate < 1) run one after the other.  The
 * paths come in a pinned block from the engine's pool (one epoch, or epochs of
 * walks bounded by walk_length + 1 vertices), copied straight from the device;
 * kk_paths_free returns the block. */
kk_status kk_walk(kk_engine *e, const kk_walk_opts *opts, kk_paths **out);

/* The apps' entry points: set opts->app and call kk_walk. */
kk_status kk_walk_deepwalk(kk_engine *e, const kk_walk_opts *opts, kk_paths **out); /* deepwalk.hpp:30-47 */
kk_status kk_walk_ppr(kk_engine *e, const kk_walk_opts *opts, kk_paths **out);      /* ppr.hpp:30-64 */
kk_status kk_walk_node2vec(kk_engine *e, const kk_walk_opts *opts, kk_paths **out); /* node2vec.hpp:108-202 */
kk_status kk_walk_metapath(kk_engine *e, const kk_walk_opts *opts, kk_paths **out); /* metapath.hpp:70-128 */

/* Same walk into caller-owned host buffers (pinned memory gives full copy
 * bandwidth): h_length[walker_num], h_offset[walker_num], and h_vertices with
 * room for vertices_capacity vertices (KK_ERR_PATH_CAPACITY if too small).
 * The output is PathSet-equivalent (include/path.hpp:46-84) in walker-id order.
 * The copies to the caller's buffers overlap the walk (options into_stream,
 * into_chunks); the call returns when every path is in host memory. */
kk_status kk_walk_into(kk_engine *e, const kk_walk_opts *opts, uint32_t *h_length, uint64_t *h_offset,
                       uint32_t *h_vertices, uint64_t vertices_capacity, uint64_t *total_steps);

/* Same walk with paths left in HBM (no host copy): for callers that consume
 * paths on the GPU.  The buffers stay valid until the next walk call on this
 * engine.  *d_length / *d_offset / *d_vertices are device pointers.  With
 * d_offset NULL and d_vertices non-NULL the paths are returned as the walk
 * wrote them, unpacked: walker i's slot starts at i * (walk_length + 1)
 * (DeepWalk, node2vec, metapath) or at its PPR capacity offset.  With both
 * NULL no path is stored. */
kk_status kk_walk_device(kk_engine *e, const kk_walk_opts *opts, uint64_t *total_steps, const uint32_t **d_length,
                         const uint64_t **d_offset, const uint32_t **d_vertices);

/* ---- batches: many jobs in one launch (no counterpart in the reference,
 * which runs one random_walk() call at a time) ---------------------------- */

/* Runs n_jobs (1..1024) DeepWalk, node2vec or metapath jobs of one app and
 * weighting in one launch; each job has its own seed, walkers, length, (p, q)
 * or schemes, and its paths equal those of the job run alone.  Jobs take no
 * start list and no epochs.  out[j] receives job j's paths (kk_paths_free each). */
kk_status kk_batch_walk(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, kk_paths **out);

/* The same batch without waiting: kk_batch_submit checks the jobs, builds
 * what the walk reads and queues the batch on the engine's stream, then
 * returns; kk_batch_wait waits for it and hands out out[j] for job j (as
 * kk_batch_walk does) and frees the handle.  The calling thread is free
 * meanwhile.  Until the wait, the engine takes no other call
 * (KK_ERR_INVALID_CONFIG); destroy the engine only after the wait.  No
 * counterpart in the reference, whose random_walk() call blocks. */
typedef struct kk_batch kk_batch;
kk_status kk_batch_submit(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, kk_batch **out);
kk_status kk_batch_wait(kk_batch *b, kk_paths **out);

/* Same with paths left in HBM in the batch layout (job after job, walker i of a
 * job at i * (walk_length + 1)); valid until the next walk call. */
kk_status kk_batch_walk_device(kk_engine *e, const kk_walk_opts *jobs, int n_jobs, uint64_t *total_steps,
                               const uint32_t **d_length, const uint32_t **d_vertices);

/* ---- serving: continuous batching of walk requests (no counterpart in the
 * reference) ---------------------------------------------------------------
 * A server owns the engine while it runs (no other engine call until
 * kk_serve_stop).  It keeps the graph, the sorted adjacency and the alias
 * tables resident and runs `slots` batches at once, each on its own stream:
 * a slot that finishes takes the requests that arrived meanwhile (first come
 * first served, as many as fit its job count and memory), so new requests are
 * admitted while earlier ones are still on the GPU and their kernels overlap.
 * Every request's paths equal those of the same request run alone through
 * kk_walk.  Submit and poll are thread-safe. */
typedef struct kk_server kk_server;

typedef struct
{
    int app;                /* KK_APP_DEEPWALK, KK_APP_NODE2VEC or KK_APP_METAPATH */
    int weighted;
    int slots;              /* batches in flight, 1..8 (0: 2) */
    uint32_t max_jobs;      /* requests per batch, 1..1024 (0: 256) */
    uint64_t slot_bytes;    /* admission: device bytes of walker paths and state per slot
                               (walkers * ((walk_length + 1) * 4 + 4) per request; 0: 1 GiB) */
    int launch_mode;        /* 0: each slot replays one captured CUDA graph per batch (job table
                               upload, status reset, walk kernel, status read-back); 1: stream launches */
} kk_serve_opts;

typedef struct
{
    kk_status status;       /* the request's outcome */
    kk_paths *paths;        /* its paths (caller frees with kk_paths_free); offsets have
                               walk_length + 1 slots per walker */
    double queue_ms;        /* submit to launch */
    double latency_ms;      /* submit to paths on the host */
    uint32_t batch_jobs;    /* requests in the batch it ran in */
} kk_serve_result;

typedef struct
{
    uint64_t completed, failed, batches;
    uint64_t walker_steps;          /* of the completed requests */
    double p50_ms, p99_ms, mean_ms; /* latency of the completed requests */
    double mean_batch_jobs;
    double walk_ms, copy_ms, host_ms; /* summed over batches: launch to the batch's walk seen
                                         ended (0 when its last copies were issued first), from
                                         there to its last request's copies issued (the slot
                                         then takes its next batch), then the slot's own
                                         hand-out of failed requests */
} kk_serve_stats;

kk_status kk_serve_start(kk_engine *e, const kk_serve_opts *opts, kk_server **out);
/* Queues one request (a kk_walk_opts of the server's app and weighting, no
 * start list, no epochs); ticket identifies it.  KK_ERR_INVALID_CONFIG for a
 * request the server cannot run, larger than a slot included. */
kk_status kk_serve_submit(kk_server *s, const kk_walk_opts *req, uint64_t *ticket);
/* Waits up to timeout_ms (-1: no limit) for the request; KK_ERR_TIMEOUT if it
 * is not done yet.  A result is handed out once. */
kk_status kk_serve_poll(kk_server *s, uint64_t ticket, int timeout_ms, kk_serve_result *out);
kk_status kk_serve_stats_get(kk_server *s, kk_serve_stats *out);
/* Starts the statistics afresh (e.g. after a warm-up). */
kk_status kk_serve_stats_reset(kk_server *s);
/* Finishes the queued requests, stops the slots and frees the server (results
 * not yet polled are freed). */
kk_status kk_serve_stop(kk_server *s);
/* Open-loop client for measuring a server: submits reqs[i] through
 * kk_serve_submit at arrival_s[i] seconds (non-decreasing) after the call
 * starts, from the calling thread, while a second host thread polls every
 * request in order and frees its paths.  latency_ms[i] (may be NULL) receives
 * request i's submit-to-host latency, *total_steps the walker-steps of all
 * requests and *elapsed_s the time from the call's start to the last result.
 * A client driven from an interpreter adds its own per-call overhead to the
 * arrivals; this one keeps the schedule.  Returns the first failed submit's or
 * request's status (the requests submitted before it still finish). */
kk_status kk_serve_replay(kk_server *s, const kk_walk_opts *reqs, const double *arrival_s, uint32_t n,
                          double *latency_ms, uint64_t *total_steps, double *elapsed_s);

/* Access counts of the last walk call's last epoch when the walk_stats option
 * is on (zeros otherwise): rejection trials, second-order queries, and the
 * probes a binary search of each query target's sorted adjacency takes
 * (ceil(log2(degree + 1)); counted only with node2vec_adjacency = 1). */
kk_status kk_last_walk_stats(const kk_engine *e, uint64_t *trials, uint64_t *queries, uint64_t *probes);

/* Milliseconds of the alias build and of the walk kernels of the last walk
 * call, from CUDA events on the engine's stream. */
kk_status kk_last_walk_timing(const kk_engine *e, float *alias_ms, float *walk_ms);

/* The GPU's rate of dependent random 32-byte reads over a buffer of `bytes`
 * (>= 64 MiB; above the L2 size it measures HBM): every thread follows
 * chains of reads whose next address depends on the value read, as a walk
 * step does.  The random-gather ceiling the walk kernels are compared with;
 * allocates and frees `bytes` of device memory. */
kk_status kk_gather_ceiling(kk_engine *e, uint64_t bytes, double *reads_per_s);

/* n blocks of the walk's generator, Philox4x32-10, computed by a device
 * kernel on the current device: host arrays ctr[4n] in and out[4n] out, key =
 * seed (low 32 bits k0, high 32 bits k1).  For known-answer checks of the
 * random stream that replaces StdRandNumGenerator (include/util.hpp:45-70);
 * allocates and frees 32n bytes of device memory and synchronises. */
kk_status kk_philox_blocks(uint64_t seed, uint32_t n, const uint32_t *ctr, uint32_t *out);

/* Kernels this library has launched on the engine's streams since the engine
 * was created (alias builds, walks, batches, graph loading; the replays of a
 * serving slot's captured CUDA graph are not counted). */
kk_status kk_engine_launch_count(const kk_engine *e, uint64_t *count);

void kk_paths_free(kk_paths *p);

/* PathSet::dump text format (include/path.hpp:85-109): one line per walker,
 * "id length" when with_head, then " v" per vertex.  Epoch by epoch
 * (include/walk.hpp:804-844), walkers are written in the reference's segment
 * order for seg_num worker threads: segment t of an epoch starting at walker b
 * holds walkers b + t, b + t + seg_num, ... (include/path.hpp:383-441);
 * seg_num = 1 writes walker-id order.  mode is "w" or "a". */
kk_status kk_paths_dump(const kk_paths *p, const char *path, const char *mode, int with_head, int seg_num);

#ifdef __cplusplus
}
#endif

#endif
