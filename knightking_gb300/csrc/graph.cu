/*
 * Graph ingestion into HBM.
 *
 * - Binary edge-list files in the reference's format (include/storage.hpp:35-55,
 *   Edge<T> of include/type.hpp:43-85), optionally mirrored edge by edge as
 *   --make-undirected does (include/graph.hpp:430-443), grouped by source with
 *   file order kept (include/graph.hpp:309-330).
 * - Host CSR arrays.
 * - A seeded R-MAT generator that builds the graph on the device:
 *     draw i, level l: word l%4 of Philox4x32-10(key=seed, counter=(i, 0, l/4, 3));
 *     quadrant by integer thresholds floor(a*2^32), floor((a+b)*2^32),
 *     floor((a+b+c)*2^32) -> a:(0,0) b:(0,1) c:(1,0) d:(1,1), level 0 = top bit;
 *     self-loops dropped, (min,max) pairs deduplicated, mirrored, sorted by
 *     (src, dst);  per pair (u<v): Philox(key=seed+1000, counter=(u, v, 0, 4))
 *     word0 -> uniform [1,5) weight 1 + 4*(w0>>8)*2^-24, or (words 2,3) a
 *     lognormal(0,1) weight by Box-Muller; word1 -> type floor(w1*types/2^32).
 */
#include <fcntl.h>
#include <stdio.h>
#include <sys/stat.h>
#include <unistd.h>

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cub/cub.cuh>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "knightking_gb300/engine.cuh"

namespace kk
{

void exclusive_scan_u64(kk_engine *e, const uint64_t *in, uint64_t *out, uint64_t n, cudaStream_t st, DevBuf &tmpb)
{
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)n, st));
    void *tmp = tmpb.ensure(bytes);
    KK_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, (int64_t)n, st));
}

void exclusive_scan_u64(kk_engine *e, const uint64_t *in, uint64_t *out, uint64_t n)
{
    exclusive_scan_u64(e, in, out, n, e->stream, e->cub_tmp);
}

void sort_pairs_u32(kk_engine *e, const uint32_t *keys_in, uint32_t *keys_out, const uint32_t *vals_in,
                    uint32_t *vals_out, uint32_t n, int bits)
{
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, vals_in, vals_out, (int64_t)n, 0,
                                                  bits, e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(e->cub_tmp.ensure(bytes), bytes, keys_in, keys_out, vals_in,
                                                  vals_out, (int64_t)n, 0, bits, e->stream));
}

namespace
{

__global__ void check_sorted_kernel(const int64_t *off, const uint32_t *nbr, uint32_t V, int *unsorted)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    {
        for (int64_t e = off[v] + 1; e < off[v + 1]; e++)
        {
            if (nbr[e - 1] > nbr[e])
            {
                atomicExch(unsorted, 1);
                break;
            }
        }
    }
}

__global__ void iota_u32_kernel(uint32_t *x, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        x[i] = (uint32_t)i;
}

template <typename T>
__global__ void gather_kernel(const T *src, const uint32_t *idx, T *dst, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

/* ---- R-MAT -------------------------------------------------------------- */

struct RmatThresholds
{
    uint64_t ta, tab, tabc;
};

__global__ void rmat_draw_kernel(uint64_t m, uint32_t scale, uint64_t seed, RmatThresholds t, uint64_t *keys)
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    {
        uint64_t src = 0, dst = 0;
        for (uint32_t blk = 0; blk * 4 < scale; blk++)
        {
            uint4 wv = philox4x32_10(make_uint4((uint32_t)i, 0, blk, 3), k0, k1);
            uint32_t words[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
            for (int j = 0; j < 4; j++)
            {
                if (blk * 4 + j >= scale)
                    break;
                uint64_t w = words[j];
                uint64_t sbit = w >= t.tab;
                uint64_t dbit = ((w >= t.ta) && (w < t.tab)) || (w >= t.tabc);
                src = (src << 1) | sbit;
                dst = (dst << 1) | dbit;
            }
        }
        uint64_t lo = src < dst ? src : dst, hi = src < dst ? dst : src;
        keys[i] = (src == dst) ? ~0ull : ((lo << 32) | hi);
    }
}

__global__ void rmat_mirror_kernel(const uint64_t *pairs, uint64_t u, uint64_t *out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < u; i += (uint64_t)gridDim.x * blockDim.x)
    {
        uint64_t k = pairs[i];
        out[2 * i] = k;
        out[2 * i + 1] = (k << 32) | (k >> 32);
    }
}

__global__ void rmat_csr_kernel(const uint64_t *keys, uint64_t e_num, uint32_t *nbr, unsigned int *deg, uint64_t seed,
                                float *w, int weights, uint8_t *type, uint32_t types)
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < e_num; i += (uint64_t)gridDim.x * blockDim.x)
    {
        uint64_t k = keys[i];
        uint32_t s = (uint32_t)(k >> 32), d = (uint32_t)k;
        nbr[i] = d;
        atomicAdd(deg + s, 1u);
        if (w != nullptr || type != nullptr)
        {
            uint32_t lo = s < d ? s : d, hi = s < d ? d : s;
            uint4 r = philox4x32_10(make_uint4(lo, hi, 0, 4), k0, k1);
            if (w != nullptr)
            {
                if (weights == 1)
                {
                    w[i] = fadd(1.0f, fmul(map_gen_float(r.x, 1.0f), 4.0f));
                }
                else
                {
                    float u1 = ((float)((r.z >> 8) + 1)) * 5.9604644775390625e-8f;
                    float u2 = ((float)(r.w >> 8)) * 5.9604644775390625e-8f;
                    float z = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
                    w[i] = expf(z);
                }
            }
            if (type != nullptr)
                type[i] = (uint8_t)__umulhi(r.y, types);
        }
    }
}

__global__ void deg_to_u64_kernel(const unsigned int *deg, uint64_t *out, uint32_t V)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= V; v += gridDim.x * blockDim.x)
        out[v] = v < V ? deg[v] : 0;
}

} // namespace

const uint32_t *vertex_order(kk_engine *e)
{
    if (e->order_valid)
        return (const uint32_t *)e->order.p;
    const uint32_t V = e->V;
    uint32_t *deg = nullptr, *deg_sorted = nullptr, *ids = nullptr, *bounds = nullptr;
    KK_CUDA_CHECK(cudaMalloc(&deg, (size_t)V * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&deg_sorted, (size_t)V * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&ids, (size_t)V * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&bounds, kTierBounds * sizeof(uint32_t)));
    uint32_t *order = e->order.as<uint32_t>(V);
    degree_keys_kernel<<<grid_for(e, V, 256), 256, 0, e->stream>>>(e->view(), deg, ids);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairsDescending(nullptr, bytes, deg, deg_sorted, ids, order, (int64_t)V, 0,
                                                            32, e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairsDescending(e->cub_tmp.ensure(bytes), bytes, deg, deg_sorted, ids,
                                                            order, (int64_t)V, 0, 32, e->stream));
    KK_CUDA_CHECK(cudaMemsetAsync(bounds, 0, kTierBounds * sizeof(uint32_t), e->stream));
    TierThresholds thr;
    for (uint32_t k = 0; k < kAliasClasses; k++)
        thr.thr[k] = kAliasClassMax[k];
    thr.thr[kAliasClasses] = 0;
    tier_bounds_kernel<<<grid_for(e, V, 256), 256, 0, e->stream>>>(deg_sorted, V, thr, bounds);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    KK_CUDA_CHECK(cudaMemcpyAsync(e->tier, bounds, kTierBounds * sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    cudaFree(deg);
    cudaFree(deg_sorted);
    cudaFree(ids);
    cudaFree(bounds);
    e->n_hub = e->tier[0];
    e->n_nz = e->tier[kAliasClasses];
    RowDesc *rows = e->rows.as<RowDesc>(V > 0 ? V : 1);
    row_desc_kernel<<<grid_for(e, V, 256), 256, 0, e->stream>>>(e->view(), order, rows);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    e->order_valid = true;
    return order;
}

const uint64_t *vertex_cursors(kk_engine *e)
{
    uint64_t *cur = e->vcur.as<uint64_t>(e->V);
    if (!e->vcur_valid)
    {
        if (e->E >= kCursorMaxEdges)
            fail(KK_ERR_INVALID_CONFIG, "vertex cursors hold edge offsets below 2^40");
        vertex_cursor_kernel<<<grid_for(e, e->V, 256), 256, 0, e->stream>>>(e->view(), cur);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        e->vcur_valid = true;
    }
    return cur;
}

bool graph_no_dead_ends(kk_engine *e)
{
    if (!e->dead_ends_valid)
    {
        int *flag = (int *)e->small.ensure(64) + 12; /* a word the walks' status does not use */
        KK_CUDA_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), e->stream));
        dead_end_kernel<<<grid_for(e, e->E, 256), 256, 0, e->stream>>>(e->view(), flag);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        words_to_host(e, (const uint32_t *)flag, 40, 1);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        e->no_dead_ends = ((volatile uint32_t *)e->h_status)[40] == 0;
        e->dead_ends_valid = true;
    }
    return e->no_dead_ends;
}

const uint4 *cursor_adjacency_of(kk_engine *e)
{
    if (!e->adjc_valid)
    {
        const uint64_t *cur = vertex_cursors(e);
        uint4 *a = e->adjc.as<uint4>(e->E > 0 ? e->E : 1);
        KK_CUDA_CHECK(cudaEventRecord(e->ev[0], e->stream));
        adj_cursor_kernel<<<grid_for(e, e->E, 256), 256, 0, e->stream>>>(e->view(), cur, a);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        KK_CUDA_CHECK(cudaEventRecord(e->ev[1], e->stream));
        KK_CUDA_CHECK(cudaEventSynchronize(e->ev[1]));
        KK_CUDA_CHECK(cudaEventElapsedTime(&e->adjc_ms, e->ev[0], e->ev[1]));
        e->adjc_valid = true;
    }
    return (const uint4 *)e->adjc.p;
}

EdgeSetView node2vec_edge_set(kk_engine *e)
{
    if (e->n2v_adjacency != 0)
        return EdgeSetView{nullptr, 0};
    if (!e->edge_set_valid)
    {
        const uint64_t nb = e->E > 0 ? e->E : 1; /* four slots per bucket: load <= 1/4 */
        uint64_t *buckets = e->edge_set.as<uint64_t>(nb * kEdgeSetWords);
        /* empty keys and (pos, weight) words at their maximum for atomicMin */
        KK_CUDA_CHECK(cudaMemsetAsync(buckets, 0xff, nb * kEdgeSetWords * sizeof(uint64_t), e->stream));
        const uint32_t *order = vertex_order(e);
        const GraphView g = e->view();
        if (e->n_hub)
        {
            const unsigned grid = e->n_hub < 4u * e->sm_count ? e->n_hub : 4u * e->sm_count;
            edge_set_block_kernel<<<grid, 1024, 0, e->stream>>>(g, buckets, nb, order, 0, e->n_hub);
            count_launch(e);
            KK_CUDA_CHECK(cudaGetLastError());
        }
        if (e->n_nz > e->n_hub)
        {
            edge_set_warp_kernel<<<grid_for(e, (uint64_t)(e->n_nz - e->n_hub) * 32, 256), 256, 0, e->stream>>>(
                g, buckets, nb, order, e->n_hub, e->n_nz);
            count_launch(e);
            KK_CUDA_CHECK(cudaGetLastError());
        }
        e->edge_set_nb = nb;
        e->edge_set_valid = true;
    }
    return EdgeSetView{(const uint64_t *)e->edge_set.p, e->edge_set_nb};
}

const uint8_t *metapath_vertex_masks(kk_engine *e)
{
    uint8_t *vmask = e->vmask.as<uint8_t>(e->V);
    if (!e->vmask_valid)
    {
        apps::metapath_vertex_mask_kernel<<<grid_for(e, e->V, 256), 256, 0, e->stream>>>(e->view(), vmask);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
        e->vmask_valid = true;
    }
    return vmask;
}

void graph_check_sorted(kk_engine *e)
{
    int *flag = (int *)e->small.ensure(64);
    KK_CUDA_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), e->stream));
    check_sorted_kernel<<<grid_for(e, e->V, 256), 256, 0, e->stream>>>(e->d_off, e->d_nbr, e->V, flag);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    int h = 0;
    KK_CUDA_CHECK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    e->sorted = h ? 0 : 1;
}

/* Sorts every adjacency by neighbour, carrying weights and types (what
 * node2vec() does with std::sort, src/apps/node2vec.hpp:122-125).  Stable, so
 * with duplicate neighbours the file order of the duplicates is kept. */
void graph_sort_adjacency(kk_engine *e)
{
    require_graph(e);
    if (e->sorted < 0)
        graph_check_sorted(e);
    if (e->sorted == 1)
        return;
    e->alias_cached = -1;      /* the tables follow the adjacency order */
    e->edge_set_valid = false; /* and so do the edge set's indices */
    e->adjc_valid = false;     /* and the cursor adjacency */
    uint64_t E = e->E;
    uint32_t *nbr_out = nullptr, *idx_in = nullptr, *idx_out = nullptr;
    KK_CUDA_CHECK(cudaMalloc(&nbr_out, E * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&idx_in, E * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&idx_out, E * 4 + 4));
    iota_u32_kernel<<<grid_for(e, E, 256), 256, 0, e->stream>>>(idx_in, E);
    count_launch(e);
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceSegmentedSort::StableSortPairs(nullptr, bytes, e->d_nbr, nbr_out, idx_in, idx_out,
                                                            (int64_t)E, (int64_t)e->V, e->d_off, e->d_off + 1,
                                                            e->stream));
    void *tmp = e->cub_tmp.ensure(bytes);
    KK_CUDA_CHECK(cub::DeviceSegmentedSort::StableSortPairs(tmp, bytes, e->d_nbr, nbr_out, idx_in, idx_out, (int64_t)E,
                                                            (int64_t)e->V, e->d_off, e->d_off + 1, e->stream));
    if (e->d_w)
    {
        float *w2 = nullptr;
        KK_CUDA_CHECK(cudaMalloc(&w2, E * 4 + 4));
        gather_kernel<float><<<grid_for(e, E, 256), 256, 0, e->stream>>>(e->d_w, idx_out, w2, E);
        count_launch(e);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        cudaFree(e->d_w);
        e->d_w = w2;
    }
    if (e->d_type)
    {
        uint8_t *t2 = nullptr;
        KK_CUDA_CHECK(cudaMalloc(&t2, E + 4));
        gather_kernel<uint8_t><<<grid_for(e, E, 256), 256, 0, e->stream>>>(e->d_type, idx_out, t2, E);
        count_launch(e);
        KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
        cudaFree(e->d_type);
        e->d_type = t2;
    }
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    cudaFree(e->d_nbr);
    e->d_nbr = nbr_out;
    cudaFree(idx_in);
    cudaFree(idx_out);
    e->sorted = 1;
}

void graph_upload(kk_engine *e, uint32_t V, uint64_t E, const int64_t *off, const uint32_t *nbr, const float *w,
                  const uint8_t *type)
{
    e->free_graph();
    KK_CUDA_CHECK(cudaMalloc(&e->d_off, (V + 1) * sizeof(int64_t)));
    KK_CUDA_CHECK(cudaMalloc(&e->d_nbr, E * 4 + 4));
    KK_CUDA_CHECK(cudaMemcpyAsync(e->d_off, off, (V + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, e->stream));
    KK_CUDA_CHECK(cudaMemcpyAsync(e->d_nbr, nbr, E * 4, cudaMemcpyHostToDevice, e->stream));
    if (w)
    {
        KK_CUDA_CHECK(cudaMalloc(&e->d_w, E * 4 + 4));
        KK_CUDA_CHECK(cudaMemcpyAsync(e->d_w, w, E * 4, cudaMemcpyHostToDevice, e->stream));
    }
    if (type)
    {
        KK_CUDA_CHECK(cudaMalloc(&e->d_type, E + 4));
        KK_CUDA_CHECK(cudaMemcpyAsync(e->d_type, type, E, cudaMemcpyHostToDevice, e->stream));
    }
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    e->V = V;
    e->E = E;
    e->has_graph = true;
    e->sorted = -1;
}

void graph_load_arrays(kk_engine *e, uint32_t V, uint64_t E, const int64_t *off, const uint32_t *nbr, const float *w,
                       const uint8_t *type)
{
    if (V == 0 || off == nullptr || (E > 0 && nbr == nullptr))
        fail(KK_ERR_INVALID_CONFIG, "graph needs V > 0, off and nbr");
    if (off[0] != 0 || (uint64_t)off[V] != E)
        fail(KK_ERR_INVALID_CONFIG, "off[0] must be 0 and off[V] must be E");
    for (uint32_t v = 0; v < V; v++)
        if (off[v + 1] < off[v])
            fail(KK_ERR_INVALID_CONFIG, "offsets must be non-decreasing");
    for (uint64_t i = 0; i < E; i++)
        if (nbr[i] >= V)
            fail(KK_ERR_INVALID_CONFIG, "neighbour id out of range");
    if (type)
        for (uint64_t i = 0; i < E; i++)
            if (type[i] >= 8)
                fail(KK_ERR_INVALID_CONFIG, "edge types must be < 8 (8-bit type masks)");
    graph_upload(e, V, E, off, nbr, w, type);
}

/* include/storage.hpp:35-55 + include/graph.hpp:408-530 on one rank. */
namespace
{

__global__ void count_sources_kernel(const uint32_t *src, uint64_t m, unsigned long long *cnt)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + src[i], 1ull);
}

template <typename T>
__global__ void permute_kernel(const T *in, const uint32_t *perm, T *out, uint64_t m)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[perm[i]];
}

/* One record of a binary edge file (words 32-bit words: src, dst[, weight])
 * per thread: the source as the sort key, the destination and the weight's
 * bits as the value; with --make-undirected the record at 2i and its mirror
 * at 2i + 1.  An endpoint >= V sets *bad. */
__global__ void split_records_kernel(const uint32_t *rec, uint32_t words, uint64_t n, uint32_t V, bool weighted,
                                     bool undirected, uint32_t *key, uint64_t *val, uint32_t *bad)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t *r = rec + i * words;
        const uint32_t s = r[0], d = r[1];
        const uint64_t wb = weighted ? (uint64_t)r[2] << 32 : 0;
        if (s >= V || d >= V)
            atomicOr(bad, 1u);
        const uint64_t j = undirected ? 2 * i : i;
        key[j] = s;
        val[j] = d | wb;
        if (undirected)
        {
            key[j + 1] = d;
            val[j + 1] = s | wb;
        }
    }
}

/* Offsets from the sorted sources: off[v] is the first position whose source
 * is >= v (off[V] = m), written once per v by the position where the source
 * steps past it. */
__global__ void offsets_from_sorted_kernel(const uint32_t *s, uint64_t m, uint32_t V, int64_t *off)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= m; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const int64_t lo = i == 0 ? -1 : (int64_t)s[i - 1];
        const int64_t hi = i == m ? (int64_t)V : (int64_t)s[i];
        for (int64_t v = lo + 1; v <= hi; v++)
            off[v] = (int64_t)i;
    }
}

__global__ void unpack_values_kernel(const uint64_t *val, uint64_t m, uint32_t *nbr, float *w)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t x = val[i];
        nbr[i] = (uint32_t)x;
        if (w != nullptr)
            w[i] = __uint_as_float((uint32_t)(x >> 32));
    }
}

} // namespace

/* CSR in HBM from the raw records of an untyped binary edge file (8-byte
 * src/dst or 12-byte src/dst/weight, include/storage.hpp:35-55), which
 * fill(d) puts into device memory at d as they are; they are split (and mirrored,
 * include/graph.hpp:430-443) there, and a stable radix sort of the sources
 * carrying each edge's destination and weight keeps file order within each
 * source (include/graph.hpp:309-330); the offsets come from the sorted
 * sources.  The CSR equals csr_from_edges' of the same edges. */
template <typename Fill>
void csr_from_records(kk_engine *e, uint32_t V, uint64_t n, size_t rec, bool undirected, Fill fill)
{
    const uint64_t m = undirected ? 2 * n : n;
    if (m >= 0xffffffffull)
        fail(KK_ERR_INVALID_CONFIG, "edge lists are limited to 2^32 - 1 edges");
    const bool weighted = rec == 12;
    struct Temps
    {
        DevBuf raw, key, key2, val, val2;
        ~Temps()
        {
            DevBuf *b[] = {&raw, &key, &key2, &val, &val2};
            for (DevBuf *x : b)
                x->release();
        }
    } tmp;
    uint32_t *d_raw = tmp.raw.as<uint32_t>(n * (rec / 4) + 1);
    uint32_t *d_key = tmp.key.as<uint32_t>(m + 1), *d_key2 = tmp.key2.as<uint32_t>(m + 1);
    uint64_t *d_val = tmp.val.as<uint64_t>(m + 1), *d_val2 = tmp.val2.as<uint64_t>(m + 1);
    uint32_t *bad = (uint32_t *)e->small.ensure(64) + 13; /* a word the walks' status does not use */
    /* the records in HBM, as read (fill returns once they have arrived) */
    fill((unsigned char *)d_raw);
    /* the device part: from the records in HBM to the CSR */
    const auto t0 = std::chrono::steady_clock::now();
    KK_CUDA_CHECK(cudaMemsetAsync(bad, 0, sizeof(uint32_t), e->stream));
    split_records_kernel<<<grid_for(e, n ? n : 1, 256), 256, 0, e->stream>>>(d_raw, (uint32_t)(rec / 4), n, V, weighted,
                                                                             undirected, d_key, d_val, bad);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    words_to_host(e, bad, 41, 1);
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    if (((volatile uint32_t *)e->h_status)[41] != 0)
        fail(KK_ERR_INVALID_CONFIG, "edge endpoint >= v_num"); /* the engine keeps its graph */
    tmp.raw.release();
    e->free_graph();
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < V)
        bits++;
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_key, d_key2, d_val, d_val2, (int64_t)m, 0, bits,
                                                  e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(e->cub_tmp.ensure(bytes), bytes, d_key, d_key2, d_val, d_val2,
                                                  (int64_t)m, 0, bits, e->stream));
    KK_CUDA_CHECK(cudaMalloc(&e->d_off, ((uint64_t)V + 1) * sizeof(int64_t)));
    offsets_from_sorted_kernel<<<grid_for(e, m + 1, 256), 256, 0, e->stream>>>(d_key2, m, V, e->d_off);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    KK_CUDA_CHECK(cudaMalloc(&e->d_nbr, m * 4 + 4));
    if (weighted)
        KK_CUDA_CHECK(cudaMalloc(&e->d_w, m * 4 + 4));
    unpack_values_kernel<<<grid_for(e, m ? m : 1, 256), 256, 0, e->stream>>>(d_val2, m, e->d_nbr,
                                                                             weighted ? e->d_w : nullptr);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    e->V = V;
    e->E = m;
    e->has_graph = true;
    e->sorted = -1;
    e->load_device_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

/* CSR in HBM from an edge list in file order (include/graph.hpp:309-330):
 * a stable radix sort of the edge positions by source keeps file order within
 * each source; offsets are the exclusive scan of the source counts. */
void csr_from_edges(kk_engine *e, uint32_t V, uint64_t m, const uint32_t *h_src, const uint32_t *h_dst,
                    const float *h_w, const uint8_t *h_t)
{
    if (m >= 0xffffffffull)
        fail(KK_ERR_INVALID_CONFIG, "edge lists are limited to 2^32 - 1 edges");
    const auto t0 = std::chrono::steady_clock::now();
    e->free_graph();
    struct Temps
    {
        DevBuf src, src2, idx, perm, cnt, in;
        ~Temps()
        {
            DevBuf *b[] = {&src, &src2, &idx, &perm, &cnt, &in};
            for (DevBuf *x : b)
                x->release();
        }
    } tmp;
    uint32_t *d_src = tmp.src.as<uint32_t>(m), *d_src2 = tmp.src2.as<uint32_t>(m);
    uint32_t *d_idx = tmp.idx.as<uint32_t>(m), *d_perm = tmp.perm.as<uint32_t>(m);
    KK_CUDA_CHECK(cudaMemcpyAsync(d_src, h_src, m * 4, cudaMemcpyHostToDevice, e->stream));
    iota_u32_kernel<<<grid_for(e, m, 256), 256, 0, e->stream>>>(d_idx, m);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < V)
        bits++;
    size_t bytes = 0;
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d_src, d_src2, d_idx, d_perm, (int64_t)m, 0, bits,
                                                  e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(e->cub_tmp.ensure(bytes), bytes, d_src, d_src2, d_idx, d_perm,
                                                  (int64_t)m, 0, bits, e->stream));
    /* offsets */
    unsigned long long *cnt = tmp.cnt.as<unsigned long long>((uint64_t)V + 1);
    KK_CUDA_CHECK(cudaMemsetAsync(cnt, 0, ((uint64_t)V + 1) * 8, e->stream));
    count_sources_kernel<<<grid_for(e, m, 256), 256, 0, e->stream>>>(d_src, m, cnt);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    KK_CUDA_CHECK(cudaMalloc(&e->d_off, ((uint64_t)V + 1) * sizeof(int64_t)));
    exclusive_scan_u64(e, (const uint64_t *)cnt, (uint64_t *)e->d_off, (uint64_t)V + 1);
    /* neighbours, weights, types in sorted order */
    KK_CUDA_CHECK(cudaMalloc(&e->d_nbr, m * 4 + 4));
    uint32_t *d_in = tmp.in.as<uint32_t>(m);
    KK_CUDA_CHECK(cudaMemcpyAsync(d_in, h_dst, m * 4, cudaMemcpyHostToDevice, e->stream));
    permute_kernel<uint32_t><<<grid_for(e, m, 256), 256, 0, e->stream>>>(d_in, d_perm, e->d_nbr, m);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    if (h_w)
    {
        KK_CUDA_CHECK(cudaMalloc(&e->d_w, m * 4 + 4));
        KK_CUDA_CHECK(cudaMemcpyAsync(d_in, h_w, m * 4, cudaMemcpyHostToDevice, e->stream));
        permute_kernel<float><<<grid_for(e, m, 256), 256, 0, e->stream>>>((const float *)d_in, d_perm, e->d_w, m);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
    }
    if (h_t)
    {
        KK_CUDA_CHECK(cudaMalloc(&e->d_type, m + 4));
        KK_CUDA_CHECK(cudaMemcpyAsync(d_in, h_t, m, cudaMemcpyHostToDevice, e->stream));
        permute_kernel<uint8_t><<<grid_for(e, m, 256), 256, 0, e->stream>>>((const uint8_t *)d_in, d_perm, e->d_type,
                                                                            m);
        count_launch(e);
        KK_CUDA_CHECK(cudaGetLastError());
    }
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    e->V = V;
    e->E = m;
    e->has_graph = true;
    e->sorted = -1;
    e->load_device_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

/* Text edge lists (read_edge_txt, include/storage.hpp:107-115): "src dst" or
 * "src dst weight" per line, parsed in parallel over newline-aligned chunks of
 * the file and kept in file order.  Lines that start with '#' or '%' are
 * comments; any other malformed line is an error (the reference's fscanf loop
 * stops or spins there). */
void parse_text_edges(const char *path, bool weighted, uint32_t V, std::vector<uint32_t> &src,
                      std::vector<uint32_t> &dst, std::vector<float> &w)
{
    FILE *f = fopen(path, "rb");
    if (!f)
        fail(KK_ERR_IO, std::string("cannot open ") + path);
    fseek(f, 0, SEEK_END);
    const size_t bytes = (size_t)ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> buf(bytes + 1);
    const size_t got = bytes ? fread(buf.data(), 1, bytes, f) : 0;
    fclose(f);
    if (got != bytes)
        fail(KK_ERR_IO, std::string("short read from ") + path);
    buf[bytes] = '\0';
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0)
        nt = 1;
    if (nt > 64)
        nt = 64;
    if (bytes < (1u << 20))
        nt = 1;
    std::vector<size_t> cut(nt + 1, bytes);
    cut[0] = 0;
    for (unsigned t = 1; t < nt; t++)
    {
        size_t c = bytes / nt * t;
        while (c < bytes && buf[c - 1] != '\n')
            c++;
        cut[t] = c < cut[t - 1] ? cut[t - 1] : c;
    }
    struct Part
    {
        std::vector<uint32_t> s, d;
        std::vector<float> w;
        std::string err;
    };
    std::vector<Part> parts(nt);
    auto work = [&](unsigned t) {
        Part &pt = parts[t];
        const char *p = buf.data() + cut[t], *end = buf.data() + cut[t + 1];
        while (p < end)
        {
            const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
            if (!eol)
                eol = end;
            const char *q = p;
            while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r'))
                q++;
            if (q < eol && *q != '#' && *q != '%')
            {
                char *x;
                const unsigned long a = strtoul(q, &x, 10);
                const bool ok_a = x != q;
                q = x;
                const unsigned long b = strtoul(q, &x, 10);
                const bool ok_b = x != q;
                q = x;
                float wt = 0.0f;
                bool ok_w = true;
                if (weighted)
                {
                    wt = strtof(q, &x);
                    ok_w = x != q;
                    q = x;
                }
                while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r'))
                    q++;
                if (!ok_a || !ok_b || !ok_w || q != eol || a >= V || b >= V)
                {
                    pt.err = std::string(p, (size_t)(eol - p));
                    return;
                }
                pt.s.push_back((uint32_t)a);
                pt.d.push_back((uint32_t)b);
                if (weighted)
                    pt.w.push_back(wt);
            }
            p = eol + 1;
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++)
        th.emplace_back(work, t);
    work(0);
    for (auto &x : th)
        x.join();
    size_t total = 0;
    for (auto &pt : parts)
    {
        if (!pt.err.empty())
            fail(KK_ERR_IO, "malformed edge line (or vertex id >= v_num): " + pt.err.substr(0, 80));
        total += pt.s.size();
    }
    src.reserve(total);
    dst.reserve(total);
    w.reserve(weighted ? total : 0);
    for (auto &pt : parts)
    {
        src.insert(src.end(), pt.s.begin(), pt.s.end());
        dst.insert(dst.end(), pt.d.begin(), pt.d.end());
        if (weighted)
            w.insert(w.end(), pt.w.begin(), pt.w.end());
    }
}

void graph_load_text(kk_engine *e, uint32_t V, const char *path, int weighted, int undirected)
{
    if (V == 0)
        fail(KK_ERR_INVALID_CONFIG, "v_num must be > 0");
    std::vector<uint32_t> src, dst;
    std::vector<float> w;
    parse_text_edges(path, weighted != 0, V, src, dst, w);
    if (undirected)
    {
        /* --make-undirected (include/graph.hpp:430-443): every edge followed by its mirror */
        const size_t n = src.size();
        std::vector<uint32_t> s2(2 * n), d2(2 * n);
        std::vector<float> w2(weighted ? 2 * n : 0);
        for (size_t i = 0; i < n; i++)
        {
            s2[2 * i] = src[i];
            d2[2 * i] = dst[i];
            s2[2 * i + 1] = dst[i];
            d2[2 * i + 1] = src[i];
            if (weighted)
                w2[2 * i] = w2[2 * i + 1] = w[i];
        }
        src.swap(s2);
        dst.swap(d2);
        w.swap(w2);
    }
    csr_from_edges(e, V, src.size(), src.data(), dst.data(), weighted ? w.data() : nullptr, nullptr);
}

void graph_load_binary(kk_engine *e, uint32_t V, const char *path, int kind, int undirected)
{
    size_t rec;
    switch (kind)
    {
    case KK_EDGE_UNWEIGHTED:
        rec = 8;
        break;
    case KK_EDGE_F32:
    case KK_EDGE_META:
        rec = 12;
        break;
    case KK_EDGE_META_F32:
        rec = 16;
        break;
    default:
        fail(KK_ERR_INVALID_CONFIG, "unknown edge kind");
    }
    if (V == 0)
        fail(KK_ERR_INVALID_CONFIG, "v_num must be > 0");
    struct File
    {
        int fd;
        ~File()
        {
            if (fd >= 0)
                close(fd);
        }
    } file{open(path, O_RDONLY)};
    const int fd = file.fd;
    if (fd < 0)
        fail(KK_ERR_IO, std::string("cannot open ") + path);
    struct stat sb;
    if (fstat(fd, &sb) != 0)
        fail(KK_ERR_IO, std::string("cannot stat ") + path);
    const size_t n = (size_t)sb.st_size / rec;
    const bool has_w = kind == KK_EDGE_F32 || kind == KK_EDGE_META_F32;
    const bool has_t = kind == KK_EDGE_META || kind == KK_EDGE_META_F32;
    const uint64_t m = undirected ? 2 * (uint64_t)n : n;
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt == 0 ? 1 : nt > 32 ? 32 : nt;
    if (n < (1u << 16))
        nt = 1;
    if (!has_t)
    {
        /* untyped records go to the device as read and are split there:
         * each reader thread takes its share of the file in blocks, reading
         * one block into a pinned buffer while the copy of the previous one
         * (its other buffer) runs on its own stream */
        const unsigned nr = nt < (unsigned)kk_engine::kReaders ? nt : (unsigned)kk_engine::kReaders;
        const size_t blk = kk_engine::kReadBlock;
        if (e->read_pinned == nullptr)
        {
            KK_CUDA_CHECK(cudaHostAlloc((void **)&e->read_pinned, (size_t)kk_engine::kReaders * 2 * blk,
                                        cudaHostAllocDefault));
            for (int r = 0; r < kk_engine::kReaders; r++)
            {
                KK_CUDA_CHECK(cudaStreamCreateWithFlags(&e->read_st[r], cudaStreamNonBlocking));
                for (int b = 0; b < 2; b++)
                    KK_CUDA_CHECK(cudaEventCreateWithFlags(&e->read_ev[r][b], cudaEventDisableTiming));
            }
        }
        auto fill = [&](unsigned char *d_raw) {
            const size_t total = n * rec;
            std::vector<int> failed(nr, 0); /* 1: short read, 2: CUDA */
            auto read_share = [&](unsigned th) {
                size_t pos = total / nr * th;
                const size_t hi = th + 1 == nr ? total : total / nr * (th + 1);
                unsigned char *buf[2] = {e->read_pinned + (size_t)th * 2 * blk,
                                         e->read_pinned + ((size_t)th * 2 + 1) * blk};
                for (unsigned k = 0; pos < hi; k++)
                {
                    const size_t len = hi - pos < blk ? hi - pos : blk;
                    /* the buffer's previous copy has left it */
                    if (k >= 2 && cudaEventSynchronize(e->read_ev[th][k & 1]) != cudaSuccess)
                    {
                        failed[th] = 2;
                        return;
                    }
                    size_t got = 0;
                    while (got < len)
                    {
                        const ssize_t r = pread(fd, buf[k & 1] + got, len - got, (off_t)(pos + got));
                        if (r <= 0)
                        {
                            failed[th] = 1;
                            return;
                        }
                        got += (size_t)r;
                    }
                    if (cudaMemcpyAsync(d_raw + pos, buf[k & 1], len, cudaMemcpyHostToDevice, e->read_st[th]) !=
                            cudaSuccess ||
                        cudaEventRecord(e->read_ev[th][k & 1], e->read_st[th]) != cudaSuccess)
                    {
                        failed[th] = 2;
                        return;
                    }
                    pos += len;
                }
            };
            {
                std::vector<std::thread> pool;
                for (unsigned th = 1; th < nr; th++)
                    pool.emplace_back(read_share, th);
                read_share(0);
                for (std::thread &x : pool)
                    x.join();
            }
            /* every copy issued has landed before the buffers are reused or
             * the records are read */
            for (unsigned th = 0; th < nr; th++)
                if (cudaStreamSynchronize(e->read_st[th]) != cudaSuccess)
                    failed[th] = 2;
            for (int x : failed)
            {
                if (x == 1)
                    fail(KK_ERR_IO, std::string("short read from ") + path);
                if (x == 2)
                    fail(KK_ERR_CUDA, "copy of the edge records to the device");
            }
        };
        csr_from_records(e, V, n, rec, undirected, fill);
        return;
    }
    /* typed records: split into columns on the host */
    /* the columns, left uninitialised: every slot is written below */
    std::unique_ptr<uint32_t[]> src(new uint32_t[m + 1]), dst(new uint32_t[m + 1]);
    std::unique_ptr<float[]> w(has_w ? new float[m] : nullptr);
    std::unique_ptr<uint8_t[]> t(has_t ? new uint8_t[m] : nullptr);
    /* the records split among the host threads, each reading its share
     * with pread in blocks and writing its columns' slots */
    enum : int
    {
        kOk = 0,
        kShort,
        kEndpoint,
        kType,
        kAlloc
    };
    std::vector<int> err(nt, kOk);
    auto split = [&](unsigned th) {
        const size_t lo = n / nt * th + (th < n % nt ? th : n % nt);
        const size_t hi = lo + n / nt + (th < n % nt ? 1 : 0);
        const size_t block = ((size_t)4 << 20) / rec;
        std::unique_ptr<unsigned char[]> buf(new unsigned char[block * rec]);
        for (size_t b = lo; b < hi; b += block)
        {
            const size_t cnt = hi - b < block ? hi - b : block;
            size_t done = 0;
            while (done < cnt * rec)
            {
                const ssize_t r = pread(fd, buf.get() + done, cnt * rec - done, (off_t)(b * rec + done));
                if (r <= 0)
                {
                    err[th] = kShort;
                    return;
                }
                done += (size_t)r;
            }
            for (size_t k = 0; k < cnt; k++)
            {
                const unsigned char *r = buf.get() + k * rec;
                uint32_t s, d;
                memcpy(&s, r, 4);
                memcpy(&d, r + 4, 4);
                if (s >= V || d >= V)
                {
                    err[th] = kEndpoint;
                    return;
                }
                float wt = 0.0f;
                int32_t ty = 0;
                if (kind == KK_EDGE_F32 || kind == KK_EDGE_META_F32)
                    memcpy(&wt, r + 8, 4);
                if (kind == KK_EDGE_META)
                    memcpy(&ty, r + 8, 4);
                if (kind == KK_EDGE_META_F32)
                    memcpy(&ty, r + 12, 4);
                if (has_t && (ty < 0 || ty >= 8))
                {
                    err[th] = kType;
                    return;
                }
                const size_t i = b + k;
                const size_t j = undirected ? 2 * i : i;
                src[j] = s;
                dst[j] = d;
                if (has_w)
                    w[j] = wt;
                if (has_t)
                    t[j] = (uint8_t)ty;
                if (undirected)
                {
                    /* --make-undirected: each edge followed by its mirror */
                    src[j + 1] = d;
                    dst[j + 1] = s;
                    if (has_w)
                        w[j + 1] = wt;
                    if (has_t)
                        t[j + 1] = (uint8_t)ty;
                }
            }
        }
    };
    auto work = [&](unsigned th) {
        try
        {
            split(th);
        }
        catch (...)
        {
            err[th] = kAlloc;
        }
    };
    {
        std::vector<std::thread> pool;
        for (unsigned th = 1; th < nt; th++)
            pool.emplace_back(work, th);
        work(0);
        for (std::thread &x : pool)
            x.join();
    }
    for (int x : err)
    {
        if (x == kAlloc)
            fail(KK_ERR_OOM, "host allocation failed");
        if (x == kShort)
            fail(KK_ERR_IO, std::string("short read from ") + path);
        if (x == kEndpoint)
            fail(KK_ERR_INVALID_CONFIG, "edge endpoint >= v_num");
        if (x == kType)
            fail(KK_ERR_INVALID_CONFIG, "edge types must be in [0, 8)");
    }
    /* file order within a source, sorted on the device */
    csr_from_edges(e, V, m, src.get(), dst.get(), w.get(), t.get());
}

void graph_generate_rmat(kk_engine *e, uint32_t scale, uint32_t ef, double a, double b, double c, uint64_t seed,
                         int weights, int types)
{
    if (scale < 1 || scale > 30 || ef < 1)
        fail(KK_ERR_INVALID_CONFIG, "R-MAT needs 1 <= scale <= 30 and edge_factor >= 1");
    if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0))
        fail(KK_ERR_INVALID_CONFIG, "R-MAT probabilities must be >= 0 with a+b+c <= 1");
    if (types < 0 || types > 8 || weights < 0 || weights > 2)
        fail(KK_ERR_INVALID_CONFIG, "R-MAT weights in {0,1,2}, types in [0, 8]");
    e->free_graph();
    uint32_t V = 1u << scale;
    uint64_t m = (uint64_t)ef << scale;
    RmatThresholds t;
    t.ta = (uint64_t)floor(a * 4294967296.0);
    t.tab = (uint64_t)floor((a + b) * 4294967296.0);
    t.tabc = (uint64_t)floor((a + b + c) * 4294967296.0);
    uint64_t *k1 = nullptr, *k2 = nullptr;
    int64_t *d_count = nullptr;
    KK_CUDA_CHECK(cudaMalloc(&k1, m * 8 + 8));
    KK_CUDA_CHECK(cudaMalloc(&k2, m * 8 + 8));
    KK_CUDA_CHECK(cudaMalloc(&d_count, 16));
    rmat_draw_kernel<<<grid_for(e, m, 256), 256, 0, e->stream>>>(m, scale, seed, t, k1);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    size_t bytes = 0;
    int end_bit = 64;
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, bytes, k1, k2, m, 0, end_bit, e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortKeys(e->cub_tmp.ensure(bytes), bytes, k1, k2, m, 0, end_bit, e->stream));
    KK_CUDA_CHECK(cub::DeviceSelect::Unique(nullptr, bytes, k2, k1, d_count, (int64_t)m, e->stream));
    KK_CUDA_CHECK(cub::DeviceSelect::Unique(e->cub_tmp.ensure(bytes), bytes, k2, k1, d_count, (int64_t)m, e->stream));
    int64_t u = 0;
    KK_CUDA_CHECK(cudaMemcpyAsync(&u, d_count, 8, cudaMemcpyDeviceToHost, e->stream));
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    uint64_t last = 0;
    if (u > 0)
    {
        KK_CUDA_CHECK(cudaMemcpy(&last, k1 + u - 1, 8, cudaMemcpyDeviceToHost));
        if (last == ~0ull)
            u--; /* the self-loop sentinel sorts last */
    }
    uint64_t E = 2 * (uint64_t)u;
    /* mirror into k2 (size >= E since E <= 2m and k2 holds m... grow if needed) */
    uint64_t *mir = nullptr, *mir_sorted = nullptr;
    KK_CUDA_CHECK(cudaMalloc(&mir, E * 8 + 8));
    KK_CUDA_CHECK(cudaMalloc(&mir_sorted, E * 8 + 8));
    rmat_mirror_kernel<<<grid_for(e, u, 256), 256, 0, e->stream>>>(k1, (uint64_t)u, mir);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    cudaFree(k1);
    cudaFree(k2);
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, bytes, mir, mir_sorted, E, 0, 64, e->stream));
    KK_CUDA_CHECK(cub::DeviceRadixSort::SortKeys(e->cub_tmp.ensure(bytes), bytes, mir, mir_sorted, E, 0, 64, e->stream));
    cudaFree(mir);
    KK_CUDA_CHECK(cudaMalloc(&e->d_nbr, E * 4 + 4));
    if (weights)
        KK_CUDA_CHECK(cudaMalloc(&e->d_w, E * 4 + 4));
    if (types)
        KK_CUDA_CHECK(cudaMalloc(&e->d_type, E + 4));
    unsigned int *deg = nullptr;
    uint64_t *deg64 = nullptr;
    KK_CUDA_CHECK(cudaMalloc(&deg, (size_t)V * 4 + 4));
    KK_CUDA_CHECK(cudaMalloc(&deg64, ((size_t)V + 1) * 8));
    KK_CUDA_CHECK(cudaMemsetAsync(deg, 0, (size_t)V * 4, e->stream));
    rmat_csr_kernel<<<grid_for(e, E, 256), 256, 0, e->stream>>>(mir_sorted, E, e->d_nbr, deg, seed + 1000, e->d_w,
                                                                weights, e->d_type, (uint32_t)types);
    count_launch(e);
    KK_CUDA_CHECK(cudaGetLastError());
    deg_to_u64_kernel<<<grid_for(e, (uint64_t)V + 1, 256), 256, 0, e->stream>>>(deg, deg64, V);
    count_launch(e);
    KK_CUDA_CHECK(cudaMalloc(&e->d_off, ((size_t)V + 1) * 8));
    exclusive_scan_u64(e, deg64, (uint64_t *)e->d_off, (uint64_t)V + 1);
    KK_CUDA_CHECK(cudaStreamSynchronize(e->stream));
    cudaFree(mir_sorted);
    cudaFree(deg);
    cudaFree(deg64);
    cudaFree(d_count);
    e->V = V;
    e->E = E;
    e->has_graph = true;
    e->sorted = 1;
}

} // namespace kk
