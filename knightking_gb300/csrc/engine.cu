/*
 * C-ABI of the walker-step engine (include/knightking_gb300.h).
 *
 * random_walk() (include/walk.hpp:698-878) on one GPU: per epoch of
 * walker_num*rate walkers (:804-844) the app's kernels run on the engine's
 * stream and the epoch's paths are compacted on the device and copied out;
 * the reference's footprint shuffle and assembly (include/path.hpp:164-477)
 * reduce to that compaction because each walker writes its own path slot.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <cub/cub.cuh>
#include <string>
#include <vector>

#include "knightking_gb300/engine.cuh"

void kk_engine::free_graph()
{
    if (d_off)
        cudaFree(d_off);
    if (d_nbr)
        cudaFree(d_nbr);
    if (d_w)
        cudaFree(d_w);
    if (d_type)
        cudaFree(d_type);
    d_off = nullptr;
    d_nbr = nullptr;
    d_w = nullptr;
    d_type = nullptr;
    has_graph = false;
    V = 0;
    E = 0;
    sorted = -1;
    order_valid = false;
    vcur_valid = false;
    edge_set_valid = false;
    adjc_valid = false;
    dead_ends_valid = false;
    alias_cached = -1;
    n_hub = n_nz = 0;
    memset(tier, 0, sizeof(tier));
    vmask_valid = false;
}

namespace kk
{
void graph_upload(kk_engine *e, uint32_t V, uint64_t E, const int64_t *off, const uint32_t *nbr, const float *w,
                  const uint8_t *type);
void graph_load_arrays(kk_engine *e, uint32_t V, uint64_t E, const int64_t *off, const uint32_t *nbr, const float *w,
                       const uint8_t *type);
void graph_load_binary(kk_engine *e, uint32_t V, const char *path, int kind, int undirected);
void graph_load_text(kk_engine *e, uint32_t V, const char *path, int weighted, int undirected);
void parse_text_edges(const char *path, bool weighted, uint32_t V, std::vector<uint32_t> &src,
                      std::vector<uint32_t> &dst, std::vector<float> &w);
void graph_generate_rmat(kk_engine *e, uint32_t scale, uint32_t ef, double a, double b, double c, uint64_t seed,
                         int weights, int types);

namespace
{

/* One warp per walker copies its path into the packed output. */
__global__ void compact_paths_kernel(uint32_t n, const uint32_t *length, const uint64_t *src_off, uint32_t cap,
                                     const uint32_t *path, const uint64_t *dst_off, uint32_t *out)
{
    uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < n; i += nwarps)
    {
        uint64_t s = src_off ? src_off[i] : (uint64_t)i * cap;
        uint64_t d = dst_off[i];
        uint32_t len = length[i];
        for (uint32_t k = lane; k < len; k += 32)
            out[d + k] = path[s + k];
    }
}

__global__ void length_to_u64_kernel(const uint32_t *len, uint64_t *out, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x)
        out[i] = i < n ? len[i] : 0;
}

__global__ void words_to_host_kernel(const uint32_t *src, volatile uint32_t *dst, int n)
{
    if (threadIdx.x < (unsigned)n)
        dst[threadIdx.x] = src[threadIdx.x];
}

/* Position of each batch job's first vertex in the packed output:
 * out[j] = off[first_task_j], out[nj] = off[total]. */
__global__ void job_begin_kernel(const BatchJob *jobs, uint32_t nj, uint32_t total, const uint64_t *off,
                                 uint64_t *out)
{
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j <= nj; j += gridDim.x * blockDim.x)
        out[j] = off[j < nj ? jobs[j].first_task : total];
}

/* One warp per walker of a batch: finds the walker's job (binary search over
 * the jobs' first positions), copies its path from the batch layout (job
 * base + i * cap) to its packed offset, and writes the offset counted from
 * the job's first vertex. */
__global__ void pack_batch_kernel(const BatchJob *jobs, uint32_t nj, uint32_t total, const uint32_t *length,
                                  const uint32_t *path, const uint64_t *off, uint32_t *out, uint64_t *rel)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < total; t += nwarps)
    {
        uint32_t lo = 0, hi = nj;
        while (hi - lo > 1)
        {
            const uint32_t mid = (lo + hi) >> 1;
            if (jobs[mid].first_task <= t)
                lo = mid;
            else
                hi = mid;
        }
        const BatchJob &b = jobs[lo];
        const uint64_t s = b.path_base + (uint64_t)(t - b.first_task) * b.cap;
        const uint64_t d = off[t];
        const uint32_t len = length[t];
        for (uint32_t k = lane; k < len; k += 32)
            out[d + k] = path[s + k];
        if (lane == 0)
            rel[t] = d - off[b.first_task];
    }
}

/* Path offsets of the streamed segments: bound[k] = off[min(k << shift, n)]
 * for k = 0..nseg, written to mapped host memory. */
__global__ void segment_bounds_kernel(const uint64_t *off, uint32_t n, uint32_t shift, uint32_t nseg,
                                      volatile uint64_t *bound)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k <= nseg)
    {
        const uint64_t w = (uint64_t)k << shift;
        bound[k] = off[w < n ? w : n];
    }
}

/* Host-side path offsets of a chunk: its packed offsets plus the chunk's base
 * in the caller's vertex buffer, or i * cap + base when no packing was needed. */
__global__ void offsets_plus_base_kernel(const uint64_t *off, uint32_t cap, uint64_t base, uint32_t n, uint64_t *out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (off ? off[i] : (uint64_t)i * cap) + base;
}

/* A streamed walk's host-side offsets (packed offsets plus the chunk's base)
 * and path lengths, from its exact path offsets: walker i's length is
 * off[i + 1] - off[i], the capacity the walk fills exactly. */
__global__ void offsets_lengths_kernel(const uint64_t *off, uint64_t base, uint32_t n, uint64_t *out_off,
                                       uint32_t *out_len)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint64_t a = off[i];
        out_off[i] = a + base;
        out_len[i] = (uint32_t)(off[i + 1] - a);
    }
}

/* Gather-ceiling probe: every thread follows two dependent chains of random
 * 32 B-aligned reads over n sectors (the access a walk step makes: the next
 * address depends on the value read). */
__device__ __forceinline__ uint64_t probe_mix(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

__global__ void gather_probe_kernel(const uint4 *buf, uint64_t n, int iters, uint32_t *out)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t a = probe_mix(2 * tid) % n, b = probe_mix(2 * tid + 1) % n;
    uint32_t acc = 0;
    for (int it = 0; it < iters; it++)
    {
        const uint4 x = __ldg(buf + 2 * a), y = __ldg(buf + 2 * b);
        acc ^= x.x ^ y.x;
        a = probe_mix(a ^ x.x ^ (uint64_t)it) % n;
        b = probe_mix(b ^ y.x ^ (uint64_t)it) % n;
    }
    out[tid] = acc;
}

__global__ void cast_alias_kernel(const AliasBucket *b, uint64_t n, float *p, uint32_t *pi, uint32_t *qi)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        AliasBucket x = b[i];
        p[i] = x.p;
        pi[i] = x.p_idx;
        qi[i] = x.q_idx;
    }
}

void validate_opts(kk_engine *e, const kk_walk_opts *o, bool builtin)
{
    if (o == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "opts is NULL");
    require_graph(e);
    if (builtin && (o->app < KK_APP_DEEPWALK || o->app > KK_APP_METAPATH))
        fail(KK_ERR_INVALID_CONFIG, "unknown app");
    if (o->weighted && e->d_w == nullptr)
        fail(KK_ERR_INVALID_CONFIG, "weighted walk on a graph without weights");
    if (o->rate < 0.0 || o->rate > 1.0)
        fail(KK_ERR_INVALID_CONFIG, "rate must be in (0, 1]");
    if (o->start != nullptr && o->n_start == 0)
        fail(KK_ERR_INVALID_CONFIG, "start list with n_start == 0");
    if ((uint64_t)o->walker_begin + o->walker_num > 0x100000000ULL)
        fail(KK_ERR_INVALID_CONFIG, "walker ids exceed 32 bits");
    if (o->walker_num > 0x80000000u)
        fail(KK_ERR_INVALID_CONFIG, "at most 2^31 walkers per call");
    if (o->walk_length >= 0xfffffff0u)
        fail(KK_ERR_INVALID_CONFIG, "walk_length too large");
}

/* The context's L2 fetch-granularity hint: v bytes, or the value found (0). */
void set_l2_fetch(kk_engine *e, int v)
{
    if (v == e->l2_fetch)
        return;
    if (e->l2_fetch == 0)
        KK_CUDA_CHECK(cudaDeviceGetLimit(&e->l2_fetch_saved, cudaLimitMaxL2FetchGranularity));
    KK_CUDA_CHECK(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, v == 0 ? e->l2_fetch_saved : (size_t)v));
    e->l2_fetch = v;
}

/* Walkers per epoch: walker_num * rate, at least 1 (include/walk.hpp:706-709). */
uint32_t epoch_walkers(const kk_walk_opts *o)
{
    if (o->walker_num == 0)
        return 0;
    double rate = o->rate == 0.0 ? 1.0 : o->rate;
    uint32_t per = (uint32_t)((double)o->walker_num * rate);
    if (per == 0)
        per = 1;
    if (per > o->walker_num)
        per = o->walker_num;
    return per;
}

const uint32_t *upload_start(kk_engine *e, const kk_walk_opts *o)
{
    if (o->start == nullptr)
        return nullptr;
    /* the walk kernels check the vertices (KK_STATUS_BAD_START) */
    uint32_t *d = e->start.as<uint32_t>(o->n_start);
    KK_CUDA_CHECK(cudaMemcpyAsync(d, o->start, (size_t)o->n_start * 4, cudaMemcpyHostToDevice, e->stream));
    return d;
}

void run_epoch(kk_engine *e, const kk_walk_opts *o, const uint32_t *d_start, uint32_t begin, uint32_t num,
               bool want_paths, WalkResult &res, bool packed_out = true)
{
    RunSpec rs;
    rs.seed = o->seed;
    rs.walker_begin = begin;
    rs.walker_num = num;
    rs.d_start = d_start;
    rs.n_start = o->n_start;
    rs.want_paths = want_paths;
    rs.packed_out = packed_out;
    if (o->app == KK_APP_NODE2VEC)
        run_app_node2vec(e, *o, rs, res);
    else
        run_app_first_order(e, *o, rs, res);
}

/* Compacts an epoch's paths on the device: packed vertices + per-walker offsets. */
uint64_t pack_paths(kk_engine *e, const WalkResult &r, uint64_t **d_off_out, uint32_t **d_verts_out)
{
    uint32_t n = r.walker_num;
    if (r.packed)
    {
        /* the walk wrote its paths at their packed offsets */
        *d_off_out = const_cast<uint64_t *>(r.path_off);
        *d_verts_out = r.path;
        return r.total_steps + n;
    }
    uint64_t *lens64 = e->caps.as<uint64_t>((uint64_t)n + 1);
    uint64_t *off = e->packed_off.as<uint64_t>((uint64_t)n + 1);
    length_to_u64_kernel<<<grid_for(e, (uint64_t)n + 1, 256), 256, 0, e->stream>>>(r.length, lens64, n);
    count_launch(e);
    exclusive_scan_u64(e, lens64, off, (uint64_t)n + 1);
    uint64_t total = r.total_steps + n;
    uint32_t *verts = e->packed.as<uint32_t>(total);
    compact_paths_kernel<<<grid_for(e, (uint64_t)n * 32, 256), 256, 0, e->stream>>>(n, r.length, r.path_off, r.cap,
                                                                                   r.path, off, verts);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    *d_off_out = off;
    *d_verts_out = verts;
    return total;
}

/* Packs a walk's paths on stream st into output set s for the host copy:
 * *verts the packed vertices, *offb the per-walker offsets plus base.  A
 * fixed-capacity walk whose walkers all used their whole capacity is already
 * packed and is copied from where the walk wrote it. */
uint64_t pack_paths_on(kk_engine *e, const WalkResult &r, cudaStream_t st, int s, uint64_t base,
                       const uint64_t **offb, const uint32_t **verts)
{
    const uint32_t n = r.walker_num;
    const uint64_t total = r.total_steps + n;
    uint64_t *ob = e->into_offb[s].as<uint64_t>((uint64_t)n + 1);
    if (r.packed)
    {
        offsets_plus_base_kernel<<<grid_for(e, n, 256), 256, 0, st>>>(r.path_off, 0, base, n, ob);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        *offb = ob;
        *verts = r.path;
        return total;
    }
    if (r.path_off == nullptr && total == (uint64_t)n * r.cap)
    {
        offsets_plus_base_kernel<<<grid_for(e, n, 256), 256, 0, st>>>(nullptr, r.cap, base, n, ob);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        *offb = ob;
        *verts = r.path;
        return total;
    }
    uint64_t *lens64 = e->into_lens[s].as<uint64_t>((uint64_t)n + 1);
    uint64_t *off = e->into_off[s].as<uint64_t>((uint64_t)n + 1);
    length_to_u64_kernel<<<grid_for(e, (uint64_t)n + 1, 256), 256, 0, st>>>(r.length, lens64, n);
    count_launch(e);
    exclusive_scan_u64(e, lens64, off, (uint64_t)n + 1, st, e->into_cub[s]);
    uint32_t *vv = e->into_verts[s].as<uint32_t>(total);
    compact_paths_kernel<<<grid_for(e, (uint64_t)n * 32, 256), 256, 0, st>>>(n, r.length, r.path_off, r.cap, r.path,
                                                                            off, vv);
    count_launch(e);
    offsets_plus_base_kernel<<<grid_for(e, n, 256), 256, 0, st>>>(off, 0, base, n, ob);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    *offb = ob;
    *verts = vv;
    return total;
}

/* kk_walk_into for the built-in apps: the walkers of each epoch in chunks
 * (the into_chunks option; about kIntoMinChunk walkers at least).  Chunks
 * rotate over three output sets: chunk c + 1 walks while chunk c's lengths,
 * packed offsets and vertices go to the caller's buffers on the copy stream,
 * and chunk c + 3 waits only for chunk c's copies.  The
 * alias tables are built once per call, by the first chunk (the same tables
 * every chunk would build), unless the alias_cache option keeps them across
 * calls anyway. */
constexpr uint32_t kIntoMinChunk = 1u << 18;
constexpr uint32_t kIntoMinRun = 4; /* streamed segments per copy while the walk runs */

uint64_t walk_into_chunked(kk_engine *e, const kk_walk_opts *o, uint32_t *h_length, uint64_t *h_offset,
                           uint32_t *h_vertices, uint64_t capacity)
{
    validate_opts(e, o, true);
    const uint32_t *d_start = upload_start(e, o);
    if (e->copy_stream == nullptr)
    {
        /* the highest priority: a chunk's packing kernels start as soon as its
         * walk ends, not after the next chunk's walk blocks are all issued */
        int lo = 0, hi = 0;
        KK_CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        KK_CUDA_CHECK(cudaStreamCreateWithPriority(&e->copy_stream, cudaStreamNonBlocking, hi));
        for (int i = 0; i < 3; i++)
        {
            KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_walked[i], cudaEventDisableTiming));
            KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_copied[i], cudaEventDisableTiming));
        }
        KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_seg_copy, cudaEventDisableTiming));
    }
    const int user_cache = e->alias_cache;
    struct Restore
    {
        kk_engine *e;
        int cache;
        ~Restore()
        {
            e->alias_cache = cache;
            e->walk_set = 0;
            e->seg_sink = nullptr;
            cudaStreamSynchronize(e->copy_stream);
        }
    } restore{e, user_cache};
    /* a walk whose path lengths are known before it runs streams its
     * segments out as they finish: one launch per epoch, no chunk tails */
    const bool streamed = e->into_stream && o->app != KK_APP_METAPATH && graph_no_dead_ends(e);
    if (!user_cache)
        e->alias_cached = -1; /* this call builds its own tables */
    const uint32_t per = epoch_walkers(o);
    uint64_t base = 0, steps = 0;
    uint32_t done = 0, chunk = 0;
    while (done < o->walker_num)
    {
        const uint32_t epoch_n = o->walker_num - done < per ? o->walker_num - done : per;
        /* metapath walks end at random steps, so each chunk's walk pays a
         * tail of stragglers while its paths are short to copy: one chunk
         * (S22: 18.4 ms per call against 27.6 ms in six chunks) */
        uint32_t nch = e->into_chunks > 1 && !streamed && o->app != KK_APP_METAPATH ? (uint32_t)e->into_chunks : 1u;
        if (nch > epoch_n / kIntoMinChunk)
            nch = epoch_n / kIntoMinChunk > 1 ? epoch_n / kIntoMinChunk : 1u;
        /* chunk k holds a share 0.8^k of the epoch: each chunk's copy (~0.8 of
         * its walk time on GB300) hides under the next, smaller chunk's walk,
         * and the last copy, which nothing hides, is the smallest */
        double wsum = 0.0, wk = 1.0;
        for (uint32_t k = 0; k < nch; k++, wk *= 0.8)
            wsum += wk;
        double acc = 0.0;
        wk = 1.0;
        for (uint32_t k = 0; k < nch; k++, chunk++, wk *= 0.8)
        {
            const uint32_t cb = done + (uint32_t)((double)epoch_n * (acc / wsum));
            acc += wk;
            const uint32_t ce = k + 1 == nch ? done + epoch_n : done + (uint32_t)((double)epoch_n * (acc / wsum));
            if (ce <= cb)
                continue;
            const uint32_t num = ce - cb;
            const int s = (int)(chunk % 3u);
            /* the set's previous chunk must be out before this walk overwrites it */
            KK_CUDA_CHECK(cudaStreamWaitEvent(e->stream, e->ev_copied[s], 0));
            e->walk_set = s;
            cudaStream_t cs = e->copy_stream;
            SegmentSink sink;
            if (streamed)
            {
                sink.before = [&](const uint64_t *d_off, uint32_t n, uint64_t total) {
                    if (base + total > capacity)
                        fail(KK_ERR_PATH_CAPACITY, "vertices buffer too small");
                    /* the offsets are final (the engine's stream has been
                     * synchronised), and so are the lengths, which the walk
                     * fills exactly: both out at once, while the walk's first
                     * segments are still walking */
                    uint64_t *ob = e->into_offb[s].as<uint64_t>((uint64_t)n + 1);
                    uint32_t *lb = e->into_lenb[s].as<uint32_t>((uint64_t)n + 1);
                    offsets_lengths_kernel<<<grid_for(e, n, 256), 256, 0, cs>>>(d_off, base, n, ob, lb);
                    count_launch(e);
                    KK_CUDA_CHECK(cudaGetLastError());
                    KK_CUDA_CHECK(cudaMemcpyAsync(h_offset + cb, ob, (size_t)n * 8, cudaMemcpyDeviceToHost, cs));
                    KK_CUDA_CHECK(cudaMemcpyAsync(h_length + cb, lb, (size_t)n * 4, cudaMemcpyDeviceToHost, cs));
                };
                sink.during = [&](const uint32_t *d_len, const uint32_t *d_path, uint32_t n, uint32_t shift,
                                  uint32_t nseg, const volatile uint32_t *flag, const volatile uint64_t *bound,
                                  cudaEvent_t walked) {
                    std::vector<char> out(nseg, 0);
                    uint32_t left = nseg;
                    bool all = false, issued_any = false;
                    while (left > 0)
                    {
                        if (!all)
                        {
                            /* once the walk has ended every segment is final,
                             * whether or not its flag has arrived */
                            const cudaError_t q = cudaEventQuery(walked);
                            if (q == cudaSuccess)
                                all = true;
                            else if (q != cudaErrorNotReady)
                                KK_CUDA_CHECK(q);
                        }
                        for (uint32_t a = 0; a < nseg;)
                        {
                            if (out[a] || !(all || flag[a]))
                            {
                                a++;
                                continue;
                            }
                            uint32_t b = a;
                            while (b < nseg && !out[b] && (all || flag[b]))
                                b++;
                            /* while the copy engine has work queued, finished
                             * segments wait to go out in runs of at least
                             * kIntoMinRun (it moves fewer, larger copies
                             * faster); an idle engine takes whatever is ready */
                            if (!all && b - a < kIntoMinRun && b < nseg && issued_any)
                            {
                                const cudaError_t q = cudaEventQuery(e->ev_seg_copy);
                                if (q == cudaErrorNotReady)
                                {
                                    a = b;
                                    continue;
                                }
                                if (q != cudaSuccess)
                                    KK_CUDA_CHECK(q);
                            }
                            for (uint32_t k = a; k < b; k++)
                                out[k] = 1;
                            const uint64_t va = bound[a], vb = bound[b];
                            if (vb > va)
                                KK_CUDA_CHECK(cudaMemcpyAsync(h_vertices + base + va, d_path + va,
                                                              (size_t)(vb - va) * 4, cudaMemcpyDeviceToHost, cs));
                            KK_CUDA_CHECK(cudaEventRecord(e->ev_seg_copy, cs));
                            issued_any = true;
                            left -= b - a;
                            a = b;
                        }
                        /* no yield: the thread keeps its core, so a finished
                         * segment waits microseconds, not a time slice */
                    }
                };
                e->seg_sink = &sink;
            }
            WalkResult r;
            run_epoch(e, o, d_start, o->walker_begin + cb, num, true, r);
            e->seg_sink = nullptr;
            e->alias_cache = 1;
            steps += r.total_steps;
            const uint64_t total = r.total_steps + num;
            if (base + total > capacity)
                fail(KK_ERR_PATH_CAPACITY, "vertices buffer too small");
            if (sink.used)
            {
                /* every segment's copies are queued on the copy stream */
                KK_CUDA_CHECK(cudaEventRecord(e->ev_copied[s], cs));
                base += total;
                continue;
            }
            KK_CUDA_CHECK(cudaEventRecord(e->ev_walked[s], e->stream));
            KK_CUDA_CHECK(cudaStreamWaitEvent(cs, e->ev_walked[s], 0));
            const uint64_t *offb;
            const uint32_t *verts;
            pack_paths_on(e, r, cs, s, base, &offb, &verts);
            KK_CUDA_CHECK(cudaMemcpyAsync(h_length + cb, r.length, (size_t)num * 4, cudaMemcpyDeviceToHost, cs));
            KK_CUDA_CHECK(cudaMemcpyAsync(h_offset + cb, offb, (size_t)num * 8, cudaMemcpyDeviceToHost, cs));
            KK_CUDA_CHECK(cudaMemcpyAsync(h_vertices + base, verts, total * 4, cudaMemcpyDeviceToHost, cs));
            KK_CUDA_CHECK(cudaEventRecord(e->ev_copied[s], cs));
            base += total;
        }
        done += epoch_n;
    }
    KK_CUDA_CHECK(cudaStreamSynchronize(e->copy_stream));
    return steps;
}

/* Runs all epochs; sink(epoch_begin, n, d_len, d_off, d_verts, total_vertices)
 * per epoch.  `custom` runs a user's hooks instead of a built-in app. */
template <typename Sink>
uint64_t walk_epochs(kk_engine *e, const kk_walk_opts *o, const EpochRunner *custom, Sink sink)
{
    validate_opts(e, o, custom == nullptr);
    const uint32_t *d_start = upload_start(e, o);
    uint32_t per = epoch_walkers(o);
    uint64_t steps = 0;
    uint32_t done = 0;
    while (done < o->walker_num)
    {
        uint32_t num = o->walker_num - done < per ? o->walker_num - done : per;
        WalkResult r;
        if (custom == nullptr)
        {
            run_epoch(e, o, d_start, o->walker_begin + done, num, true, r);
        }
        else
        {
            RunSpec rs;
            rs.seed = o->seed;
            rs.walker_begin = o->walker_begin + done;
            rs.walker_num = num;
            rs.d_start = d_start;
            rs.n_start = o->n_start;
            rs.fixed_cap = true;
            rs.cap = o->walk_length + 1;
            (*custom)(rs, r);
        }
        uint64_t *d_off;
        uint32_t *d_verts;
        uint64_t total = pack_paths(e, r, &d_off, &d_verts);
        sink(done, num, r.length, d_off, d_verts, total);
        steps += r.total_steps;
        done += num;
    }
    return steps;
}

} // namespace

void segment_bounds_to_host(kk_engine *e, const uint64_t *off, uint32_t n, uint32_t shift, uint32_t nseg)
{
    segment_bounds_kernel<<<(nseg + 256) / 256, 256, 0, e->stream>>>(
        off, n, shift, nseg, (volatile uint64_t *)((char *)e->d_status_host + kSegBoundAt));
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
}

void words_to_host(kk_engine *e, const uint32_t *src, int at, int n)
{
    words_to_host_kernel<<<1, 32, 0, e->stream>>>(src, (volatile uint32_t *)e->d_status_host + at, n);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
}

void pack_batch_paths(kk_engine *e, const BatchPlan &plan, const BatchJob *d_jobs, const uint32_t *length,
                      const uint32_t *path, const uint64_t **d_rel, const uint32_t **d_verts,
                      std::vector<uint64_t> &job_begin)
{
    const uint32_t n = plan.total;
    const uint32_t nj = (uint32_t)plan.jobs.size();
    uint64_t *lens64 = e->caps.as<uint64_t>((uint64_t)n + 1);
    uint64_t *off = e->packed_off.as<uint64_t>((uint64_t)n + 1);
    length_to_u64_kernel<<<grid_for(e, (uint64_t)n + 1, 256), 256, 0, e->stream>>>(length, lens64, n);
    count_launch(e);
    exclusive_scan_u64(e, lens64, off, (uint64_t)n + 1);
    uint64_t *jb = e->batch_small.as<uint64_t>((uint64_t)nj + 1);
    job_begin_kernel<<<1, 256, 0, e->stream>>>(d_jobs, nj, n, off, jb);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    job_begin.assign((size_t)nj + 1, 0);
    KK_CUDA_CHECK(cudaMemcpyAsync(job_begin.data(), jb, ((size_t)nj + 1) * 8, cudaMemcpyDeviceToHost, e->stream));
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    uint32_t *verts = e->packed.as<uint32_t>(job_begin[nj]);
    uint64_t *rel = e->batch_rel.as<uint64_t>(n);
    if (n > 0)
    {
        pack_batch_kernel<<<grid_for(e, (uint64_t)n * 32, 256), 256, 0, e->stream>>>(d_jobs, nj, n, length, path, off,
                                                                                    verts, rel);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
    }
    *d_rel = rel;
    *d_verts = verts;
}

uint64_t pack_walk_paths(kk_engine *e, const WalkResult &r, uint64_t **d_off, uint32_t **d_verts)
{
    return pack_paths(e, r, d_off, d_verts);
}

} // namespace kk

using namespace kk;

extern "C" {

const char *kk_status_string(kk_status s)
{
    switch (s)
    {
    case KK_OK:
        return "ok";
    case KK_ERR_INVALID_CONFIG:
        return "invalid configuration";
    case KK_ERR_OOM:
        return "out of memory";
    case KK_ERR_IO:
        return "I/O error";
    case KK_ERR_TRIAL_LIMIT:
        return "rejection-trial limit exceeded";
    case KK_ERR_TIMEOUT:
        return "timeout";
    case KK_ERR_CUDA:
        return "CUDA error";
    case KK_ERR_NO_GRAPH:
        return "no graph loaded";
    case KK_ERR_PATH_CAPACITY:
        return "path capacity exceeded";
    default:
        return "unknown status";
    }
}

kk_status kk_engine_create(kk_engine **out, int device)
{
    if (out == nullptr)
        return KK_ERR_INVALID_CONFIG;
    *out = nullptr;
    kk_engine *e = new (std::nothrow) kk_engine();
    if (e == nullptr)
        return KK_ERR_OOM;
    kk_status s = guard(e, [&] {
        e->device = device;
        KK_CUDA_CHECK(cudaSetDevice(device));
        KK_CUDA_CHECK(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device));
        KK_CUDA_CHECK(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
        e->stream = e->own_stream;
        KK_CUDA_CHECK(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
        KK_CUDA_CHECK(cudaStreamCreateWithFlags(&e->hub, cudaStreamNonBlocking));
        for (int i = 0; i < 3; i++)
            KK_CUDA_CHECK(cudaEventCreate(&e->ev[i]));
        KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
        KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
        KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->ev_hub_join, cudaEventDisableTiming));
        /* mapped pinned words the walks' status and capacity reads land in:
         * a kernel writes them (kk::words_to_host), so the host read waits on
         * the engine's stream only, never on copies queued on other streams */
        KK_CUDA_CHECK(cudaHostAlloc(&e->h_status, kk::kStatusBytes, cudaHostAllocMapped));
        KK_CUDA_CHECK(cudaHostGetDevicePointer(&e->d_status_host, e->h_status, 0));
    });
    if (s != KK_OK)
    {
        if (e->h_status)
            cudaFreeHost(e->h_status);
        delete e;
        return s;
    }
    *out = e;
    return KK_OK;
}

void kk_engine_destroy(kk_engine *e)
{
    if (e == nullptr)
        return;
    cudaSetDevice(e->device);
    if (e->l2_fetch != 0)
        cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, e->l2_fetch_saved);
    if (e->stream)
        cudaStreamSynchronize(e->stream);
    e->free_graph();
    kk::DevBuf *bufs[] = {&e->alias, &e->sum, &e->ave, &e->ra, &e->scratch, &e->vmask,  &e->path,      &e->length,
                          &e->path_off, &e->caps, &e->start, &e->small, &e->cub_tmp, &e->packed, &e->packed_off,
                          &e->schemes};
    for (kk::DevBuf *b : bufs)
        b->release();
    for (int i = 0; i < 3; i++)
        if (e->ev[i])
            cudaEventDestroy(e->ev[i]);
    if (e->ev_fork)
        cudaEventDestroy(e->ev_fork);
    if (e->ev_join)
        cudaEventDestroy(e->ev_join);
    if (e->ev_hub_join)
        cudaEventDestroy(e->ev_hub_join);
    e->order.release();
    e->rows.release();
    e->adjc.release();
    if (e->h_status)
        cudaFreeHost(e->h_status);
    for (int r = 0; r < kk_engine::kReaders; r++)
    {
        if (e->read_st[r])
        {
            cudaStreamSynchronize(e->read_st[r]);
            cudaStreamDestroy(e->read_st[r]);
        }
        for (int b = 0; b < 2; b++)
            if (e->read_ev[r][b])
                cudaEventDestroy(e->read_ev[r][b]);
    }
    if (e->read_pinned)
        cudaFreeHost(e->read_pinned);
    if (e->copy_stream)
    {
        cudaStreamSynchronize(e->copy_stream);
        cudaStreamDestroy(e->copy_stream);
        for (int i = 0; i < 3; i++)
        {
            cudaEventDestroy(e->ev_walked[i]);
            cudaEventDestroy(e->ev_copied[i]);
        }
        if (e->ev_seg_copy)
            cudaEventDestroy(e->ev_seg_copy);
    }
    for (int i = 0; i < 2; i++)
    {
        e->path_x[i].release();
        e->length_x[i].release();
        e->path_off_x[i].release();
        e->caps_x[i].release();
    }
    for (int i = 0; i < 3; i++)
    {
        e->into_lens[i].release();
        e->into_off[i].release();
        e->into_offb[i].release();
        e->into_lenb[i].release();
        e->into_verts[i].release();
        e->into_cub[i].release();
    }
    e->alias_next.release();
    e->seg_count.release();
    e->batch_small.release();
    e->batch_rel.release();
    e->park[0].release();
    e->park[1].release();
    e->park_count.release();
    for (int i = 0; i < 2; i++)
    {
        e->regroup_rec[i].release();
        e->regroup_key[i].release();
    }
    e->regroup_val.release();
    e->regroup_perm.release();
    e->regroup_count.release();
    if (e->host_pool)
        e->host_pool->release();
    e->vcur.release();
    e->edge_set.release();
    e->bslot.release();
    if (e->hub)
    {
        cudaStreamSynchronize(e->hub);
        cudaStreamDestroy(e->hub);
    }
    if (e->side)
    {
        cudaStreamSynchronize(e->side);
        cudaStreamDestroy(e->side);
    }
    if (e->own_stream)
        cudaStreamDestroy(e->own_stream);
    delete e;
}

kk_status kk_engine_set_stream(kk_engine *e, void *stream)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        e->stream = stream ? (cudaStream_t)stream : e->own_stream;
    });
}

kk_status kk_engine_set_option(kk_engine *e, const char *name, int64_t value)
{
    if (!e || !name)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        std::string n(name);
        if (n == "walk_schedule" && (value == 0 || value == 1))
            e->walk_schedule = (int)value;
        else if (n == "walk_blocks_per_sm" && value >= 0 && value <= 64)
            e->walk_blocks_per_sm = (int)value;
        else if (n == "trial_limit" && value >= 1 && value <= 0xffffffffLL)
            e->trial_limit = (uint32_t)value;
        else if (n == "alias_layout" && value >= 0 && value <= 2)
            e->alias_layout = (int)value;
        else if (n == "alias_cache" && (value == 0 || value == 1))
            e->alias_cache = (int)value;
        else if (n == "l2_fetch_bytes" && (value == 0 || value == 32 || value == 64 || value == 128))
            set_l2_fetch(e, (int)value);
        else if (n == "node2vec_adjacency" && (value == 0 || value == 1))
            e->n2v_adjacency = (int)value;
        else if (n == "walk_block" && value >= 32 && value <= 256 && value % 32 == 0)
            e->walk_block = (int)value;
        else if (n == "walk_stats" && (value == 0 || value == 1))
            e->walk_stats = (int)value;
        else if (n == "into_chunks" && value >= 1 && value <= 64)
            e->into_chunks = (int)value;
        else if (n == "into_stream" && (value == 0 || value == 1))
            e->into_stream = (int)value;
        else if (n == "cursor_adjacency" && (value == 0 || value == 1))
            e->cursor_adjacency = (int)value;
        else if (n == "alias_hub_grid" && value >= 0 && value <= 4096)
            e->alias_hub_grid = (int)value;
        else if (n == "walk_park" && value >= 0 && value <= 32)
            e->walk_park = (int)value;
        else if (n == "alias_streams" && value >= 1 && value <= 4)
            e->alias_streams = (int)value;
        else if (n == "alias_small_lanes" && (value == 0 || value == 1))
            e->alias_small_lanes = (int)value;
        else if (n == "walk_multi" && (value == 1 || value == 2 || value == 4))
            e->walk_multi = (int)value;
        else if (n == "regroup_interval" && value >= 0 && value <= 4096)
            e->regroup = (int)value;
        else
            fail(KK_ERR_INVALID_CONFIG, "unknown option or value out of range: " + n);
    });
}

const char *kk_last_error(const kk_engine *e)
{
    return e ? e->err.c_str() : "engine is NULL";
}

kk_status kk_graph_load_binary(kk_engine *e, uint32_t v_num, const char *path, int edge_kind, int make_undirected)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        if (path == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "path is NULL");
        const auto t0 = std::chrono::steady_clock::now();
        graph_load_binary(e, v_num, path, edge_kind, make_undirected);
        e->load_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

kk_status kk_graph_load_text(kk_engine *e, uint32_t v_num, const char *path, int weighted, int make_undirected)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        if (path == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "path is NULL");
        const auto t0 = std::chrono::steady_clock::now();
        graph_load_text(e, v_num, path, weighted, make_undirected);
        e->load_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

kk_status kk_graph_load_timing(const kk_engine *e, double *total_ms, double *device_ms)
{
    if (!e || !total_ms || !device_ms)
        return KK_ERR_INVALID_CONFIG;
    *total_ms = e->load_total_ms;
    *device_ms = e->load_device_ms;
    return KK_OK;
}

kk_status kk_text_to_binary(const char *text_path, const char *binary_path, int weighted, uint64_t *edges)
{
    if (!text_path || !binary_path)
        return KK_ERR_INVALID_CONFIG;
    return guard(nullptr, [&] {
        std::vector<uint32_t> src, dst;
        std::vector<float> w;
        parse_text_edges(text_path, weighted != 0, 0xffffffffu, src, dst, w);
        FILE *f = fopen(binary_path, "wb");
        if (!f)
            fail(KK_ERR_IO, std::string("cannot create ") + binary_path);
        const size_t rec = weighted ? 12 : 8;
        std::vector<unsigned char> out(src.size() * rec);
        for (size_t i = 0; i < src.size(); i++)
        {
            memcpy(out.data() + i * rec, &src[i], 4);
            memcpy(out.data() + i * rec + 4, &dst[i], 4);
            if (weighted)
                memcpy(out.data() + i * rec + 8, &w[i], 4);
        }
        const size_t put = out.empty() ? 0 : fwrite(out.data(), 1, out.size(), f);
        const bool ok = put == out.size() && fclose(f) == 0;
        if (!ok)
            fail(KK_ERR_IO, std::string("write failed: ") + binary_path);
        if (edges)
            *edges = src.size();
    });
}

kk_status kk_read_metapath_schemes(const char *path, kk_walk_opts *opts)
{
    if (!path || !opts)
        return KK_ERR_INVALID_CONFIG;
    return guard(nullptr, [&] {
        FILE *f = fopen(path, "r");
        if (!f)
            fail(KK_ERR_IO, std::string("cannot open ") + path);
        int n = 0, states = 0;
        bool ok = fscanf(f, "%d %d", &n, &states) == 2 && n >= 1 && n <= KK_MAX_SCHEMES && states >= 1 && states <= 8;
        int len[KK_MAX_SCHEMES] = {0};
        uint8_t mask[KK_MAX_SCHEMES][KK_MAX_SCHEME_LEN];
        memset(mask, 0, sizeof(mask));
        for (int s = 0; ok && s < n; s++)
        {
            ok = fscanf(f, "%d", &len[s]) == 1 && len[s] >= 1 && len[s] <= KK_MAX_SCHEME_LEN;
            for (int l = 0; ok && l < len[s]; l++)
                for (int t = 0; ok && t < states; t++)
                {
                    int x = 0;
                    ok = fscanf(f, "%d", &x) == 1;
                    if (ok && x != 0)
                        mask[s][l] |= (uint8_t)(1u << t);
                }
        }
        fclose(f);
        if (!ok)
            fail(KK_ERR_IO, std::string("malformed metapath scheme file (1..16 schemes of length 1..16 over 1..8 "
                                        "types): ") + path);
        opts->n_schemes = n;
        for (int s = 0; s < KK_MAX_SCHEMES; s++)
        {
            opts->scheme_len[s] = s < n ? len[s] : 0;
            for (int l = 0; l < KK_MAX_SCHEME_LEN; l++)
                opts->scheme_mask[s][l] = s < n ? mask[s][l] : 0;
        }
    });
}

kk_status kk_graph_load_arrays(kk_engine *e, uint32_t v_num, uint64_t e_num, const int64_t *off, const uint32_t *nbr,
                               const float *w, const uint8_t *type)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] { graph_load_arrays(e, v_num, e_num, off, nbr, w, type); });
}

kk_status kk_graph_generate_rmat(kk_engine *e, uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                                 uint64_t seed, int weights, int types)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] { graph_generate_rmat(e, scale, edge_factor, a, b, c, seed, weights, types); });
}

kk_status kk_graph_info(const kk_engine *e, uint32_t *v_num, uint64_t *e_num, int *has_weights, int *has_types)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    if (!e->has_graph)
        return KK_ERR_NO_GRAPH;
    if (v_num)
        *v_num = e->V;
    if (e_num)
        *e_num = e->E;
    if (has_weights)
        *has_weights = e->d_w != nullptr;
    if (has_types)
        *has_types = e->d_type != nullptr;
    return KK_OK;
}

kk_status kk_graph_download(kk_engine *e, int64_t *off, uint32_t *nbr, float *w, uint8_t *type)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        require_graph(e);
        if (off)
            KK_CUDA_CHECK(cudaMemcpy(off, e->d_off, ((size_t)e->V + 1) * 8, cudaMemcpyDeviceToHost));
        if (nbr)
            KK_CUDA_CHECK(cudaMemcpy(nbr, e->d_nbr, e->E * 4, cudaMemcpyDeviceToHost));
        if (w && e->d_w)
            KK_CUDA_CHECK(cudaMemcpy(w, e->d_w, e->E * 4, cudaMemcpyDeviceToHost));
        if (type && e->d_type)
            KK_CUDA_CHECK(cudaMemcpy(type, e->d_type, e->E, cudaMemcpyDeviceToHost));
    });
}

kk_status kk_graph_sort_adjacency(kk_engine *e)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] { graph_sort_adjacency(e); });
}

kk_status kk_alias_build(kk_engine *e, float *p, uint32_t *p_idx, uint32_t *q_idx, float *sum)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        require_graph(e);
        if (e->d_w == nullptr)
            fail(KK_ERR_INVALID_CONFIG, "alias tables need edge weights");
        apps::WeightStatic ws{e->d_w};
        TransitionConfig<EmptyData, apps::FixedLengthExt<EmptyData>, apps::WeightStatic> tc;
        tc.static_comp = ws;
        float *d_sum = e->sum.as<float>(e->V);
        KK_CUDA_CHECK(cudaMemsetAsync(d_sum, 0, (size_t)e->V * 4, e->stream));
        build_alias(e, tc);
        uint64_t E = e->E;
        float *dp = nullptr;
        uint32_t *dpi = nullptr, *dqi = nullptr;
        KK_CUDA_CHECK(cudaMalloc(&dp, E * 4 + 4));
        KK_CUDA_CHECK(cudaMalloc(&dpi, E * 4 + 4));
        KK_CUDA_CHECK(cudaMalloc(&dqi, E * 4 + 4));
        cast_alias_kernel<<<grid_for(e, E, 256), 256, 0, e->stream>>>((const AliasBucket *)e->alias.p, E, dp, dpi,
                                                                      dqi);
        count_launch(e);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        if (p)
            KK_CUDA_CHECK(cudaMemcpy(p, dp, E * 4, cudaMemcpyDeviceToHost));
        if (p_idx)
            KK_CUDA_CHECK(cudaMemcpy(p_idx, dpi, E * 4, cudaMemcpyDeviceToHost));
        if (q_idx)
            KK_CUDA_CHECK(cudaMemcpy(q_idx, dqi, E * 4, cudaMemcpyDeviceToHost));
        if (sum)
            KK_CUDA_CHECK(cudaMemcpy(sum, d_sum, (size_t)e->V * 4, cudaMemcpyDeviceToHost));
        cudaFree(dp);
        cudaFree(dpi);
        cudaFree(dqi);
    });
}

} /* extern "C" */

namespace kk
{
kk_status walk_to_host(kk_engine *e, const kk_walk_opts *opts, kk_paths **out, const EpochRunner *custom)
{
    if (!e || !out)
        return KK_ERR_INVALID_CONFIG;
    *out = nullptr;
    kk_paths *p = (kk_paths *)calloc(1, sizeof(kk_paths));
    if (!p)
        return KK_ERR_OOM;
    kk_status s = guard(e, [&] {
        validate_opts(e, opts, custom == nullptr);
        uint32_t n = opts->walker_num;
        p->walker_num = n;
        p->walker_begin = opts->walker_begin;
        p->epoch_walkers = epoch_walkers(opts);
        /* one epoch, or epochs of walks no longer than walk_length + 1 vertices
         * (DeepWalk, node2vec, user hooks): lengths, offsets and vertices
         * straight from the device into one pooled pinned block (kk_paths_free
         * returns it), sized by the epoch's total or by that bound */
        const bool one_epoch = n > 0 && p->epoch_walkers >= n;
        const bool bounded = n > 0 && (custom != nullptr || opts->app == KK_APP_DEEPWALK ||
                                       opts->app == KK_APP_NODE2VEC);
        if (one_epoch || bounded)
        {
            uint64_t base = 0, vcap = 0;
            p->total_steps = walk_epochs(e, opts, custom, [&](uint32_t done, uint32_t num, const uint32_t *d_len,
                                                              const uint64_t *d_off, const uint32_t *d_verts,
                                                              uint64_t total) {
                const size_t len_bytes = ((size_t)n * 4 + 15) & ~(size_t)15;
                const size_t off_bytes = ((size_t)n * 8 + 15) & ~(size_t)15;
                if (p->owner == nullptr)
                {
                    if (e->host_pool == nullptr)
                    {
                        e->host_pool = new HostPool();
                        e->host_pool->limit = kBatchPoolCache;
                    }
                    vcap = one_epoch ? total : (uint64_t)n * ((uint64_t)opts->walk_length + 1);
                    PooledPaths *o = new (std::nothrow) PooledPaths();
                    size_t cls = 0;
                    char *blk = o ? (char *)e->host_pool->get(len_bytes + off_bytes + vcap * 4 + 16, &cls) : nullptr;
                    if (!blk)
                    {
                        delete o;
                        fail(KK_ERR_OOM, "host allocation failed");
                    }
                    o->pool = e->host_pool;
                    o->block = blk;
                    o->cls = cls;
                    p->owner = o;
                    p->length = (uint32_t *)blk;
                    p->offset = (uint64_t *)(blk + len_bytes);
                    p->vertices = (uint32_t *)(blk + len_bytes + off_bytes);
                }
                if (base + total > vcap)
                    fail(KK_ERR_PATH_CAPACITY, "a walk exceeded its path capacity");
                const uint64_t *src_off = d_off;
                if (base != 0)
                {
                    /* the epoch's offsets count from the caller's first vertex */
                    uint64_t *ob = e->into_offb[0].as<uint64_t>((uint64_t)num + 1);
                    offsets_plus_base_kernel<<<grid_for(e, num, 256), 256, 0, e->stream>>>(d_off, 0, base, num, ob);
                    count_launch(e);
                    KK_CUDA_CHECK(cudaGetLastError());
                    src_off = ob;
                }
                KK_CUDA_CHECK(cudaMemcpyAsync(p->length + done, d_len, (size_t)num * 4, cudaMemcpyDeviceToHost,
                                              e->stream));
                KK_CUDA_CHECK(cudaMemcpyAsync(p->offset + done, src_off, (size_t)num * 8, cudaMemcpyDeviceToHost,
                                              e->stream));
                KK_CUDA_CHECK(cudaMemcpyAsync(p->vertices + base, d_verts, total * 4, cudaMemcpyDeviceToHost,
                                              e->stream));
                /* the next epoch reuses the device buffers */
                KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
                base += total;
            });
            return;
        }
        p->length = (uint32_t *)malloc((size_t)n * 4 + 4);
        p->offset = (uint64_t *)malloc((size_t)n * 8 + 8);
        if (!p->length || !p->offset)
            fail(KK_ERR_OOM, "host allocation failed");
        std::vector<uint32_t *> chunks;
        std::vector<uint64_t> chunk_len;
        uint64_t base = 0;
        p->total_steps = walk_epochs(e, opts, custom, [&](uint32_t done, uint32_t num, const uint32_t *d_len,
                                                          const uint64_t *d_off, const uint32_t *d_verts,
                                                          uint64_t total) {
            KK_CUDA_CHECK(cudaMemcpyAsync(p->length + done, d_len, (size_t)num * 4, cudaMemcpyDeviceToHost, e->stream));
            KK_CUDA_CHECK(cudaMemcpyAsync(p->offset + done, d_off, (size_t)num * 8, cudaMemcpyDeviceToHost, e->stream));
            uint32_t *h = (uint32_t *)malloc(total * 4 + 4);
            if (!h)
                fail(KK_ERR_OOM, "host allocation failed");
            chunks.push_back(h);
            chunk_len.push_back(total);
            KK_CUDA_CHECK(cudaMemcpyAsync(h, d_verts, total * 4, cudaMemcpyDeviceToHost, e->stream));
            KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
            for (uint32_t i = 0; i < num; i++)
                p->offset[done + i] += base;
            base += total;
        });
        p->vertices = (uint32_t *)malloc(base * 4 + 4);
        if (!p->vertices)
            fail(KK_ERR_OOM, "host allocation failed");
        uint64_t at = 0;
        for (size_t c = 0; c < chunks.size(); c++)
        {
            memcpy(p->vertices + at, chunks[c], chunk_len[c] * 4);
            at += chunk_len[c];
            free(chunks[c]);
        }
    });
    if (s != KK_OK)
    {
        kk_paths_free(p);
        return s;
    }
    *out = p;
    return KK_OK;
}
} // namespace kk

extern "C" {

kk_status kk_walk(kk_engine *e, const kk_walk_opts *opts, kk_paths **out)
{
    return kk::walk_to_host(e, opts, out, nullptr);
}

static kk_status walk_app(kk_engine *e, const kk_walk_opts *opts, kk_paths **out, int app)
{
    if (!opts)
        return KK_ERR_INVALID_CONFIG;
    kk_walk_opts o = *opts;
    o.app = app;
    return kk_walk(e, &o, out);
}

kk_status kk_walk_deepwalk(kk_engine *e, const kk_walk_opts *o, kk_paths **out)
{
    return walk_app(e, o, out, KK_APP_DEEPWALK);
}
kk_status kk_walk_ppr(kk_engine *e, const kk_walk_opts *o, kk_paths **out)
{
    return walk_app(e, o, out, KK_APP_PPR);
}
kk_status kk_walk_node2vec(kk_engine *e, const kk_walk_opts *o, kk_paths **out)
{
    return walk_app(e, o, out, KK_APP_NODE2VEC);
}
kk_status kk_walk_metapath(kk_engine *e, const kk_walk_opts *o, kk_paths **out)
{
    return walk_app(e, o, out, KK_APP_METAPATH);
}

kk_status kk_walk_into(kk_engine *e, const kk_walk_opts *opts, uint32_t *h_length, uint64_t *h_offset,
                       uint32_t *h_vertices, uint64_t vertices_capacity, uint64_t *total_steps)
{
    if (!e || !h_length || !h_offset || !h_vertices)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        const uint64_t steps = walk_into_chunked(e, opts, h_length, h_offset, h_vertices, vertices_capacity);
        if (total_steps)
            *total_steps = steps;
    });
}

kk_status kk_walk_device(kk_engine *e, const kk_walk_opts *opts, uint64_t *total_steps, const uint32_t **d_length,
                         const uint64_t **d_offset, const uint32_t **d_vertices)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    return guard(e, [&] {
        validate_opts(e, opts, true);
        const uint32_t *d_start = upload_start(e, opts);
        WalkResult r;
        run_epoch(e, opts, d_start, opts->walker_begin, opts->walker_num, d_vertices != nullptr, r,
                  d_offset != nullptr);
        if (total_steps)
            *total_steps = r.total_steps;
        if (d_length)
            *d_length = r.length;
        if (d_vertices && d_offset)
        {
            uint64_t *d_off;
            uint32_t *d_verts;
            pack_paths(e, r, &d_off, &d_verts);
            KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
            *d_offset = d_off;
            *d_vertices = d_verts;
        }
        else if (d_vertices)
        {
            *d_vertices = r.path; /* unpacked: walker i's slot as the walk wrote it */
        }
    });
}

kk_status kk_last_walk_stats(const kk_engine *e, uint64_t *trials, uint64_t *queries, uint64_t *probes)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    if (trials)
        *trials = e->last_stats[0];
    if (queries)
        *queries = e->last_stats[1];
    if (probes)
        *probes = e->last_stats[2];
    return KK_OK;
}

kk_status kk_gather_ceiling(kk_engine *e, uint64_t bytes, double *reads_per_s)
{
    if (!e || !reads_per_s || bytes < (64ull << 20))
        return KK_ERR_INVALID_CONFIG;
    return kk::guard(e, [&] {
        KK_CUDA_CHECK(cudaSetDevice(e->device));
        const uint64_t n = bytes / 32;
        const unsigned threads = 256, blocks = 4u * (unsigned)e->sm_count;
        const int iters = 64;
        uint4 *buf = nullptr;
        uint32_t *out = nullptr;
        KK_CUDA_CHECK(cudaMalloc(&buf, n * 32));
        KK_CUDA_CHECK(cudaMalloc(&out, (size_t)blocks * threads * 4));
        KK_CUDA_CHECK(cudaMemsetAsync(buf, 0x5a, n * 32, e->stream));
        float best = 1e30f;
        for (int r = 0; r < 4; r++)
        {
            KK_CUDA_CHECK(cudaEventRecord(e->ev[0], e->stream));
            gather_probe_kernel<<<blocks, threads, 0, e->stream>>>(buf, n, iters, out);
            count_launch(e);
            KK_CUDA_CHECK(cudaGetLastError());
            KK_CUDA_CHECK(cudaEventRecord(e->ev[1], e->stream));
            KK_CUDA_CHECK(cudaEventSynchronize(e->ev[1]));
            float ms = 0.0f;
            KK_CUDA_CHECK(cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]));
            if (r > 0 && ms < best)
                best = ms;
        }
        cudaFree(buf);
        cudaFree(out);
        *reads_per_s = 2.0 * iters * (double)blocks * threads / (best / 1e3);
    });
}

static __global__ void philox_blocks_kernel(uint32_t k0, uint32_t k1, uint32_t n, const uint4 *ctr, uint4 *out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = kk::philox4x32_10(ctr[i], k0, k1);
}

kk_status kk_philox_blocks(uint64_t seed, uint32_t n, const uint32_t *ctr, uint32_t *out)
{
    if (n == 0 || !ctr || !out)
        return KK_ERR_INVALID_CONFIG;
    uint4 *d = nullptr;
    if (cudaMalloc(&d, (size_t)n * 32) != cudaSuccess)
        return KK_ERR_OOM;
    kk_status st = KK_OK;
    if (cudaMemcpy(d, ctr, (size_t)n * 16, cudaMemcpyHostToDevice) != cudaSuccess)
        st = KK_ERR_CUDA;
    if (st == KK_OK)
    {
        philox_blocks_kernel<<<(n + 255) / 256, 256>>>((uint32_t)seed, (uint32_t)(seed >> 32), n, d, d + n);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out, d + n, (size_t)n * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = KK_ERR_CUDA;
    }
    cudaFree(d);
    return st;
}

kk_status kk_engine_launch_count(const kk_engine *e, uint64_t *count)
{
    if (!e || !count)
        return KK_ERR_INVALID_CONFIG;
    *count = e->launches.load(std::memory_order_relaxed);
    return KK_OK;
}

kk_status kk_last_walk_timing(const kk_engine *e, float *alias_ms, float *walk_ms)
{
    if (!e)
        return KK_ERR_INVALID_CONFIG;
    if (alias_ms)
        *alias_ms = e->alias_ms;
    if (walk_ms)
        *walk_ms = e->walk_ms;
    return KK_OK;
}

void kk_paths_free(kk_paths *p)
{
    if (!p)
        return;
    if (p->owner != nullptr)
    {
        kk::PooledPaths *o = (kk::PooledPaths *)p->owner;
        o->pool->put(o->block, o->cls);
        delete o;
    }
    else
    {
        free(p->length);
        free(p->offset);
        free(p->vertices);
    }
    free(p);
}

kk_status kk_paths_dump(const kk_paths *p, const char *path, const char *mode, int with_head, int seg_num)
{
    if (!p || !path || !mode || seg_num < 1)
        return KK_ERR_INVALID_CONFIG;
    FILE *f = fopen(path, mode);
    if (!f)
        return KK_ERR_IO;
    uint32_t per = p->epoch_walkers ? p->epoch_walkers : p->walker_num;
    for (uint32_t eb = 0; eb < p->walker_num; eb += per)
    {
        uint32_t en = p->walker_num - eb < per ? p->walker_num - eb : per;
        for (int t = 0; t < seg_num; t++)
        {
            for (uint32_t i = (uint32_t)t; i < en; i += (uint32_t)seg_num)
            {
                uint32_t w = eb + i;
                if (with_head)
                    fprintf(f, "%u %u", p->walker_begin + w, p->length[w]);
                const uint32_t *v = p->vertices + p->offset[w];
                for (uint32_t k = 0; k < p->length[w]; k++)
                    fprintf(f, " %u", v[k]);
                fprintf(f, "\n");
            }
        }
    }
    fclose(f);
    return KK_OK;
}

} /* extern "C" */
