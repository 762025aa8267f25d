/*
 * knightking_gb300 walk engine: configuration types and sm_103a kernels.
 *
 * The reference's plugin API (include/walk.hpp:105-363) with its hooks as
 * templated __device__ functors instead of std::function members.  A hook left
 * as NoHook is the reference's nullptr.  Hook signatures:
 *
 *   extension_comp     real_t (const Walker<S>&, vertex_id_t)
 *   static_comp        real_t (vertex_id_t, const AdjUnit&)
 *   dynamic_comp       real_t (const Walker<S>&, vertex_id_t, const AdjUnit&)          first order
 *                      real_t (const Walker<S>&, const R&, vertex_id_t, const AdjUnit&) second order
 *   dcomp_upperbound   real_t (vertex_id_t, const AdjList&)   (pure: called per use)
 *   dcomp_lowerbound   real_t (vertex_id_t, const AdjList&)   (pure: called per use)
 *   outlier_upperbound void   (const Walker<S>&, vertex_id_t, const AdjList&, real_t& area, vertex_id_t& num)
 *                             (pure: called once per step)
 *   outlier_search     bool   (const Walker<S>&, vertex_id_t, const AdjList&, vertex_id_t idx, AdjUnit& out)
 *                             (false = the reference's nullptr)
 *   post_query         bool   (const Walker<S>&, vertex_id_t cur, const AdjUnit& cand, vertex_id_t& target, Q&)
 *                             (true = a query to `target` is posted; the reference's emit)
 *   respond_query      void   (vertex_id_t target, const Q&, const AdjList& target_adj, R&)
 *   walker_init_dist   vertex_id_t (walker_id_t, Sampler&)            draws on stream 2
 *   walker_init_state  void   (Walker<S>&, vertex_id_t, Sampler&)     draws on stream 1
 *   walker_update_state void  (Walker<S>&, vertex_id_t cur, const AdjUnit& taken)
 *
 * Walker state starts value-initialised (all zero) before walker_init_state.
 */
#pragma once

#include "device.cuh"

namespace kk
{

/* ---- configuration types -------------------------------------------------- */

/* WalkerConfig (include/walk.hpp:147-193). */
template <typename S, typename InitDist = NoHook, typename InitState = NoHook, typename Update = NoHook>
struct WalkerConfig
{
    typedef S state_type;
    walker_id_t walker_num;
    InitDist walker_init_dist;
    InitState walker_init_state;
    Update walker_update_state;
};

/* TransitionConfig (include/walk.hpp:195-271); validity rules of :251-261. */
template <typename S, typename Ext, typename Static = NoHook, typename Dyn = NoHook, typename UB = NoHook,
          typename LB = NoHook, typename OutUB = NoHook, typename OutSearch = NoHook>
struct TransitionConfig
{
    static constexpr int order = 1;
    typedef S state_type;
    typedef EmptyData query_type;
    typedef EmptyData response_type;
    typedef Static static_type;
    typedef Dyn dyn_type;
    typedef NoHook post_query_type;
    static constexpr bool has_static = is_hook<Static>();
    static constexpr bool has_dynamic = is_hook<Dyn>();
    static constexpr bool has_lowerbound = is_hook<LB>();
    static constexpr bool has_outlier = is_hook<OutUB>();
    static_assert(is_hook<Ext>(), "extension_comp is required");
    static_assert(is_hook<Dyn>() || (!is_hook<UB>() && !is_hook<LB>() && !is_hook<OutUB>() && !is_hook<OutSearch>()),
                  "bounds and outlier hooks need a dynamic_comp");
    static_assert(!is_hook<Dyn>() || is_hook<UB>(), "dynamic_comp needs dcomp_upperbound");
    static_assert(is_hook<OutUB>() == is_hook<OutSearch>(), "outlier_upperbound and outlier_search go together");

    Ext extension_comp;
    Static static_comp;
    Dyn dynamic_comp;
    UB dcomp_upperbound;
    LB dcomp_lowerbound;
    OutUB outlier_upperbound;
    OutSearch outlier_search;
};

/* SecondOrderTransitionConfig (include/walk.hpp:273-363); rules of :339-351. */
template <typename S, typename Q, typename R, typename Ext, typename Static, typename PostQuery, typename Respond,
          typename Dyn, typename UB, typename LB = NoHook, typename OutUB = NoHook, typename OutSearch = NoHook>
struct SecondOrderTransitionConfig
{
    static constexpr int order = 2;
    typedef S state_type;
    typedef Q query_type;
    typedef R response_type;
    typedef Static static_type;
    typedef Dyn dyn_type;
    typedef PostQuery post_query_type;
    static constexpr bool has_static = is_hook<Static>();
    static constexpr bool has_dynamic = true;
    static constexpr bool has_lowerbound = is_hook<LB>();
    static constexpr bool has_outlier = is_hook<OutUB>();
    static_assert(is_hook<Ext>(), "extension_comp is required");
    static_assert(is_hook<PostQuery>() && is_hook<Respond>(), "post_query and respond_query are required");
    static_assert(is_hook<Dyn>() && is_hook<UB>(), "second order needs dynamic_comp and dcomp_upperbound");
    static_assert(is_hook<OutUB>() == is_hook<OutSearch>(), "outlier_upperbound and outlier_search go together");

    Ext extension_comp;
    Static static_comp;
    PostQuery post_query;
    Respond respond_query;
    Dyn dynamic_comp;
    UB dcomp_upperbound;
    LB dcomp_lowerbound;
    OutUB outlier_upperbound;
    OutSearch outlier_search;
};

/* ---- edge set ---------------------------------------------------------------
 * Exact lookup of directed edges (u, v): open addressing over 64 B buckets,
 * linear probing bucket by bucket from bucket mulhi(mix(key), nbuckets), with
 * 4 * nbuckets >= 4E slots so the load is at most 1/4 and a lookup rarely
 * leaves its first bucket.  A bucket is eight 64-bit words: four keys
 * u << 32 | v (one 32 B sector), then per slot (pos << 32 | weight bits):
 * the smallest index of (u, v) within u's adjacency, which for a sorted
 * adjacency is std::lower_bound's position of v in N(u), and the weight of
 * that edge (0 without weights).  A membership test reads the key sector; the
 * return-edge lookup of node2vec's outlier bound reads the whole bucket and
 * has the edge's position and weight in the same access.  Keys only go from
 * empty to filled and an insert moves past a bucket only when all four of its
 * slots hold other keys, so a lookup that meets an empty slot may stop. */
constexpr uint64_t kEdgeSetEmpty = ~0ull;
constexpr uint32_t kEdgeSetWords = 8; /* 64-bit words per bucket */

struct EdgeSetView
{
    const uint64_t *keys; /* nbuckets buckets of kEdgeSetWords words; nullptr: no set */
    uint64_t nbuckets;
};

/* splitmix64 finalizer (Steele, Lea, Flood, OOPSLA 2014) */
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

/* The slot (bucket * 4 + j) of edge (u, v), or ~0 when (u, v) is not an edge. */
__device__ __forceinline__ uint64_t edge_set_slot(const EdgeSetView &s, vertex_id_t u, vertex_id_t v)
{
    const uint64_t key = ((uint64_t)u << 32) | v;
    uint64_t b = __umul64hi(mix64(key), s.nbuckets);
    for (uint64_t probe = 0; probe < s.nbuckets; probe++)
    {
        const uint4 *p = reinterpret_cast<const uint4 *>(s.keys + b * kEdgeSetWords);
        uint4 q[2];
#pragma unroll
        for (int j = 0; j < 2; j++)
            q[j] = __ldg(p + j);
#pragma unroll
        for (int j = 0; j < 2; j++)
        {
            const uint64_t k0 = ((uint64_t)q[j].y << 32) | q[j].x, k1 = ((uint64_t)q[j].w << 32) | q[j].z;
            if (k0 == key)
                return b * 4 + 2 * j;
            if (k1 == key)
                return b * 4 + 2 * j + 1;
            if (k0 == kEdgeSetEmpty || k1 == kEdgeSetEmpty)
                return ~0ull;
        }
        b = b + 1 == s.nbuckets ? 0 : b + 1;
    }
    return ~0ull;
}

/* Edge (u, v)'s first position in N(u) and its weight, read with the keys in
 * one access per bucket probed; false when (u, v) is not an edge. */
__device__ __forceinline__ bool edge_set_find(const EdgeSetView &s, vertex_id_t u, vertex_id_t v, uint32_t &pos,
                                              float &weight)
{
    const uint64_t key = ((uint64_t)u << 32) | v;
    uint64_t b = __umul64hi(mix64(key), s.nbuckets);
    for (uint64_t probe = 0; probe < s.nbuckets; probe++)
    {
        const uint4 *p = reinterpret_cast<const uint4 *>(s.keys + b * kEdgeSetWords);
        uint4 q[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
            q[j] = __ldg(p + j);
        const uint64_t k[4] = {((uint64_t)q[0].y << 32) | q[0].x, ((uint64_t)q[0].w << 32) | q[0].z,
                               ((uint64_t)q[1].y << 32) | q[1].x, ((uint64_t)q[1].w << 32) | q[1].z};
        const uint32_t pw[8] = {q[2].x, q[2].y, q[2].z, q[2].w, q[3].x, q[3].y, q[3].z, q[3].w};
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
            if (k[j] == key)
            {
                weight = __uint_as_float(pw[2 * j]);
                pos = pw[2 * j + 1];
                return true;
            }
            if (k[j] == kEdgeSetEmpty)
                return false;
        }
        b = b + 1 == s.nbuckets ? 0 : b + 1;
    }
    return false;
}

/* Adds edge (u, v) at local index `local` of N(u), weight wt: the smallest
 * index of the key wins, with its weight (one 64-bit atomicMin on
 * local << 32 | weight bits). */
__device__ __forceinline__ void edge_set_insert(uint64_t *buckets, uint64_t nbuckets, vertex_id_t u, vertex_id_t v,
                                                uint32_t local, float wt)
{
    const uint64_t key = ((uint64_t)u << 32) | v;
    uint64_t b = __umul64hi(mix64(key), nbuckets);
    for (uint64_t probe = 0; probe < nbuckets; probe++)
    {
        for (int j = 0; j < 4; j++)
        {
            unsigned long long *k = reinterpret_cast<unsigned long long *>(buckets + b * kEdgeSetWords + j);
            const unsigned long long old = atomicCAS(k, (unsigned long long)kEdgeSetEmpty, (unsigned long long)key);
            if (old == kEdgeSetEmpty || old == key)
            {
                atomicMin(reinterpret_cast<unsigned long long *>(buckets + b * kEdgeSetWords + 4 + j),
                          ((unsigned long long)local << 32) | __float_as_uint(wt));
                return;
            }
        }
        b = b + 1 == nbuckets ? 0 : b + 1;
    }
}

/* Inserts the out-edges of the vertices order[lo, hi): a block per vertex
 * (hubs) or a warp per vertex. */
static __global__ void edge_set_block_kernel(GraphView g, uint64_t *buckets, uint64_t nbuckets,
                                             const uint32_t *order, uint32_t lo, uint32_t hi)
{
    for (uint32_t k = lo + blockIdx.x; k < hi; k += gridDim.x)
    {
        const uint32_t v = order[k];
        const int64_t e0 = g.off[v];
        for (int64_t e = e0 + threadIdx.x; e < g.off[v + 1]; e += blockDim.x)
            edge_set_insert(buckets, nbuckets, v, g.nbr[e], (uint32_t)(e - e0), g.w ? g.w[e] : 0.0f);
    }
}

static __global__ void edge_set_warp_kernel(GraphView g, uint64_t *buckets, uint64_t nbuckets,
                                            const uint32_t *order, uint32_t lo, uint32_t hi)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); k < hi; k += nwarps)
    {
        const uint32_t v = order[k];
        const int64_t e0 = g.off[v];
        for (int64_t e = e0 + lane; e < g.off[v + 1]; e += 32)
            edge_set_insert(buckets, nbuckets, v, g.nbr[e], (uint32_t)(e - e0), g.w ? g.w[e] : 0.0f);
    }
}

/* ---- vertex cursors --------------------------------------------------------
 * A vertex's adjacency position packed in 64 bits: begin offset in the low 40
 * bits, degree in the high 24 (kCursorDegMax means "this or more": the degree
 * is then read from the offsets).  Cursor alias buckets carry the cursors of
 * their two candidates, so a walker that moves to a candidate already holds
 * the next vertex's adjacency position. */
constexpr uint32_t kCursorDegMax = 0xFFFFFFu;
constexpr uint64_t kCursorBeginMask = (1ull << 40) - 1;
constexpr uint64_t kCursorMaxEdges = 1ull << 40;

__host__ __device__ __forceinline__ uint64_t make_cursor(int64_t begin, uint32_t deg)
{
    return (uint64_t)begin | ((uint64_t)(deg < kCursorDegMax ? deg : kCursorDegMax) << 40);
}

/* Adjacency position of the vertex a walker stands on. */
struct Pos
{
    int64_t e0;
    uint32_t deg;
};

__device__ __forceinline__ Pos pos_from_offsets(const GraphView &g, vertex_id_t v)
{
    const int64_t e0 = gather(g.off + v);
    return Pos{e0, (uint32_t)(gather(g.off + v + 1) - e0)};
}

__device__ __forceinline__ Pos pos_from_cursor(const GraphView &g, vertex_id_t v, uint64_t c)
{
    Pos p{(int64_t)(c & kCursorBeginMask), (uint32_t)(c >> 40)};
    if (p.deg == kCursorDegMax)
        p.deg = (uint32_t)(gather(g.off + v + 1) - p.e0);
    return p;
}

/* cursors of all vertices */
static __global__ void vertex_cursor_kernel(GraphView g, uint64_t *cur)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x)
        cur[v] = make_cursor(g.off[v], (uint32_t)(g.off[v + 1] - g.off[v]));
}

/* Dead ends: flag set when some edge's target has no out-edges. */
static __global__ void dead_end_kernel(GraphView g, int *flag)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < g.E; e += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t v = g.nbr[e];
        if (__ldg(g.off + v + 1) == __ldg(g.off + v))
            *flag = 1;
    }
}

/* Exact path capacities of fixed-length walks that end only by their
 * extension: cap vertices, one for a walker whose start vertex is isolated.
 * The start vertex is the walk's (start list, or walker id mod V); an
 * out-of-range one gets 1 (the walk fails the call on it). */
static __global__ void exact_caps_kernel(GraphView g, const uint32_t *start, uint32_t n_start, walker_id_t begin,
                                         uint32_t n, uint32_t cap, uint64_t *caps)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const walker_id_t id = begin + i;
        const uint32_t v = start != nullptr ? start[id % n_start] : (uint32_t)(id % g.V);
        const bool alive = v < g.V && g.off[v + 1] > g.off[v];
        caps[i] = alive ? cap : 1;
    }
}

/* cursor adjacency: every edge's neighbour with that neighbour's cursor */
static __global__ void adj_cursor_kernel(GraphView g, const uint64_t *cur, uint4 *adjc)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < g.E; e += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t n = g.nbr[e];
        const uint64_t c = __ldg(cur + n);
        adjc[e] = make_uint4(n, 0u, (uint32_t)c, (uint32_t)(c >> 32));
    }
}

/* One alias bucket (AliasBucket, include/walk.hpp:52-57), in one of two 32 B
 * layouts (one DRAM sector each) or a 16 B one:
 *
 * IndexBucket: p, p_idx, q_idx (indices local to the vertex's adjacency;
 *   q_idx == kNone is the reference's q_ptr == nullptr) and the two edges'
 *   neighbours, so a walker gets its candidate's neighbour without a second
 *   dependent gather.  Used when a hook reads the taken edge's index.
 * CursorBucket: p, the two neighbours (q_nbr == kNone: no alias) and their
 *   vertex cursors; used when no hook reads the edge index, so one 32 B read
 *   per step gives the next vertex and its adjacency position.
 * NeighbourBucket: p, the two neighbours and their edge types (type | 0x100
 *   in the low and high halves of the last word, 0 without types), 16 B;
 *   used when no hook reads the edge index.  The build writes half the
 *   bytes, and a step reads the next vertex's offsets (in L2 while they fit)
 *   besides the bucket. */
struct __align__(32) IndexBucket
{
    float p;
    uint32_t p_idx;
    uint32_t q_idx;
    uint32_t pad0;
    uint32_t p_nbr;
    uint32_t q_nbr;
    uint32_t pad1;
    uint32_t pad2;

    static constexpr bool cursor = false;
    static constexpr bool compact = false;
    /* pn, qn: the neighbours of edges pi, qi (qn unused when qi == kNone);
     * ty: the row's edge types, stored as type | 0x100 in pad1 / pad2 so a
     * pick also knows its candidate's type (nullptr: no types) */
    __device__ __forceinline__ static IndexBucket make_n(float p, uint32_t pi, uint32_t qi, uint32_t pn, uint32_t qn,
                                                         const uint64_t *, const uint8_t *ty)
    {
        uint32_t pt = 0, qt = 0;
        if (ty != nullptr)
        {
            pt = 0x100u | ty[pi];
            if (qi != kNone)
                qt = 0x100u | ty[qi];
        }
        return IndexBucket{p, pi, qi, 0, pn, qi == kNone ? kNone : qn, pt, qt};
    }
    __device__ __forceinline__ static IndexBucket make(float p, uint32_t pi, uint32_t qi, const uint32_t *nb,
                                                       const uint64_t *vcur, const uint8_t *ty)
    {
        return make_n(p, pi, qi, nb[pi], qi == kNone ? kNone : nb[qi], vcur, ty);
    }
};

struct __align__(32) CursorBucket
{
    float p;
    uint32_t p_nbr;
    uint32_t q_nbr;
    uint32_t pad0;
    uint64_t p_cur;
    uint64_t q_cur;

    static constexpr bool cursor = true;
    static constexpr bool compact = false;
    __device__ __forceinline__ static CursorBucket make_n(float p, uint32_t, uint32_t qi, uint32_t pn, uint32_t qn,
                                                          const uint64_t *vcur, const uint8_t *)
    {
        if (qi == kNone)
            return CursorBucket{p, pn, kNone, 0, gather(vcur + pn), 0};
        return CursorBucket{p, pn, qn, 0, gather(vcur + pn), gather(vcur + qn)};
    }
    __device__ __forceinline__ static CursorBucket make(float p, uint32_t pi, uint32_t qi, const uint32_t *nb,
                                                        const uint64_t *vcur, const uint8_t *ty)
    {
        return make_n(p, pi, qi, nb[pi], qi == kNone ? kNone : nb[qi], vcur, ty);
    }
};
struct __align__(16) NeighbourBucket
{
    float p;
    uint32_t p_nbr;
    uint32_t q_nbr;
    uint32_t types;

    static constexpr bool cursor = false;
    static constexpr bool compact = true;
    __device__ __forceinline__ static NeighbourBucket make_n(float p, uint32_t pi, uint32_t qi, uint32_t pn,
                                                             uint32_t qn, const uint64_t *, const uint8_t *ty)
    {
        uint32_t t = 0;
        if (ty != nullptr)
        {
            t = 0x100u | ty[pi];
            if (qi != kNone)
                t |= (0x100u | ty[qi]) << 16;
        }
        return NeighbourBucket{p, pn, qi == kNone ? kNone : qn, t};
    }
    __device__ __forceinline__ static NeighbourBucket make(float p, uint32_t pi, uint32_t qi, const uint32_t *nb,
                                                           const uint64_t *vcur, const uint8_t *ty)
    {
        return make_n(p, pi, qi, nb[pi], qi == kNone ? kNone : nb[qi], vcur, ty);
    }
};
static_assert(sizeof(IndexBucket) == 32 && sizeof(CursorBucket) == 32, "one sector per bucket");
static_assert(sizeof(NeighbourBucket) == 16, "two buckets per sector");
typedef IndexBucket AliasBucket;

/* Whether a hook reads the index of the edge it is given: hooks declare
 * `static constexpr bool reads_edge_index = false` to allow cursor buckets;
 * hooks that do not say are assumed to read it. */
template <typename F, typename = void>
struct hook_reads_index
{
    static constexpr bool value = is_hook<F>();
};
template <typename F>
struct hook_reads_index<F, std::void_t<decltype(F::reads_edge_index)>>
{
    static constexpr bool value = F::reads_edge_index;
};

/* Whether a hook reads the picked edge's type from the bucket's type tag
 * (`static constexpr bool needs_type_tag = true`): index and neighbour
 * buckets carry the tags, cursor buckets do not. */
template <typename F, typename = void>
struct hook_needs_type_tag
{
    static constexpr bool value = false;
};
template <typename F>
struct hook_needs_type_tag<F, std::void_t<decltype(F::needs_type_tag)>>
{
    static constexpr bool value = F::needs_type_tag;
};

/* The walk of (WC, TC) may use neighbour buckets: it samples by alias tables
 * and none of the hooks that see the picked edge reads its index. */
template <typename WC, typename TC>
constexpr bool use_neighbour_buckets()
{
    return TC::has_static && !hook_reads_index<typename TC::dyn_type>::value &&
           !hook_reads_index<typename TC::post_query_type>::value &&
           !hook_reads_index<decltype(WC::walker_update_state)>::value;
}

/* The walk of (WC, TC) may use cursor buckets: neighbour buckets may, and no
 * hook needs the edge's type tag. */
template <typename WC, typename TC>
constexpr bool use_cursor_buckets()
{
    return use_neighbour_buckets<WC, TC>() && !hook_needs_type_tag<typename TC::dyn_type>::value;
}

/* ---- alias-table build (init_alias_tables, include/walk.hpp:538-652) -------
 *
 * Per vertex, the reference's order: prob[e] = static_comp in CSR order with a
 * sequential float sum; ave = sum / deg; edges below ave go to the p queue,
 * the rest to the q queue, both in edge order; then FIFO pairing: pop p, pop
 * q, bucket = (prob[p]/ave, p, q), prob[q] -= ave - prob[p], q goes to the p
 * or q tail by the same test; leftovers get p = 1 and no alias.
 *
 * Queue entries carry (index, current prob): an index sits in at most one
 * queue at a time and its prob only changes when it is popped from q, so the
 * entry's value is always the reference's prob[index].  Both queues are linear
 * arrays of deg entries (the q tail never passes deg: q_tail = B + I - C <= deg
 * for B initial bigs, I pairings and C conversions, since I <= S + C).  Every
 * p pop writes one bucket, so bucket k of a vertex is its k-th p pop and the
 * whole pairing state is (ph, pt, qh, qt).
 *
 * Batched exact pairing: while both queues hold at least b live entries, the
 * next b iterations read only entries that already exist (p[ph..ph+b),
 * q[qh..qh+b)) and write only past the tails, so they are independent.  They
 * run as one parallel batch: iteration i of the batch is lane/thread i, and
 * the conversions and survivors are appended to the p and q tails in
 * iteration order by a stable ballot/prefix compaction.  The result is the
 * sequential algorithm's, bucket for bucket and bit for bit; only the serial
 * sum stays sequential (one FADD chain per vertex).
 *
 * Vertices run over a degree-descending vertex order, in degree classes
 * (kAliasClassMax), each taken largest first from an atomic counter:
 *   hubs (deg > 16384): a 1024-thread block per vertex does sum, split and
 *        pairing, queues in the 16 B/edge scratch at 2*off[v]; batches of 64
 *        or fewer go to one warp (no block barrier); on a side stream;
 *   4097..16384: the same kernel with 256-thread blocks, several per SM;
 *   2049..4096: a block per vertex, the row and its queues in shared memory
 *        (alias_block_row_kernel);
 *   1..2048: groups of G lanes per vertex, 32/G vertices per warp, rows and
 *        queues in shared memory (alias_group_kernel): G = 32 above 512,
 *        16 above 128, 8 above 32, 4 above 16, else 2.
 * A group's batches are at most G wide; the average batch of a FIFO pairing
 * over lognormal weights is about deg/30 wide, so narrow groups on small rows
 * keep the lanes busy, and the groups of a warp run converged (every loop to
 * the warp's maximum), sharing each instruction. */

constexpr uint32_t kAliasHubMin = 16385; /* degree from which a vertex is a hub */
/* largest degree of each class after the hubs; class c holds the vertices of
 * degree in (kAliasClassMax[c], kAliasClassMax[c - 1]] */
constexpr uint32_t kAliasClasses = 8;
constexpr uint32_t kAliasClassMax[kAliasClasses] = {16384, 4096, 2048, 1024, 512, 128, 32, 16};
constexpr unsigned kFullMask = 0xffffffffu;

/* A vertex of the degree-descending order with its adjacency range, so an
 * alias kernel reaches a row with one 16-byte load instead of order[] then
 * off[] (two dependent round trips). */
struct __align__(16) RowDesc
{
    int64_t e0;
    uint32_t v;
    uint32_t deg;
};

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename TC>
__device__ __forceinline__ float static_at(const GraphView &g, const TC &tc, uint32_t v, int64_t e)
{
    return tc.static_comp(v, AdjUnit{g.nbr[e], (edge_id_t)e});
}

/* One warp runs pairing batches of at most 32 iterations, with the short
 * queue in a shared-memory ring: while one queue holds few entries, each
 * batch consumes entries the previous batch appended, and a global-memory
 * queue turns every batch into an L2 round trip.  The short queue (Q when QRing, else P) is copied into R (kRingSize
 * entries, index j at R[j % kRingSize]) on entry and back on exit; the long
 * queue stays in global memory, where its reads are far from its appends.
 * The warp leaves when both queues are long again (stop_above), when the
 * ring is nearly full, or when the pairing ends. */
constexpr uint32_t kRingSize = 512;
template <bool QRing>
__device__ __forceinline__ void warp_pairing_ring(uint2 *P, uint2 *Q, uint2 *R, uint2 *Lr, uint32_t &ph, uint32_t &pt,
                                                  uint32_t &qh, uint32_t &qt, float ave, uint32_t stop_above)
{
    const uint32_t lane = threadIdx.x & 31, lt = lanemask_lt();
    constexpr uint32_t M = kRingSize - 1;
    uint2 *G = QRing ? Q : P;
    uint2 *GL = QRing ? P : Q; /* the long queue */
    const uint32_t h0 = QRing ? qh : ph, t0 = QRing ? qt : pt;
    for (uint32_t j = h0 + lane; j < t0; j += 32)
        R[j & M] = G[j];
    /* the long queue's head is staged in Lr, refilled up to kRingSize
     * entries ahead whenever a batch would pass the staged end (one L2 round
     * trip per refill instead of one per batch); its appends go to global
     * memory, where a later refill finds them */
    uint32_t le = QRing ? ph : qh;
    __syncwarp();
    while (ph < pt)
    {
        const uint32_t lp = pt - ph, lq = qt - qh;
        if (lq == 0)
            break; /* the p leftovers: written by the caller's bucket pass */
        uint32_t b = min(lp, lq);
        if (b > stop_above || (QRing ? lq : lp) > kRingSize - 64)
            break;
        if (b > 32)
            b = 32;
        const uint32_t lh = QRing ? ph : qh, ltail = QRing ? pt : qt;
        if (lh + b > le)
        {
            const uint32_t to = min(ltail, lh + kRingSize);
            for (uint32_t j = le + lane; j < to; j += 32)
                Lr[j & M] = GL[j];
            __syncwarp();
            le = to;
        }
        const bool act = lane < b;
        bool conv = false;
        uint2 ne = make_uint2(0, 0);
        if (act)
        {
            const uint2 pe = QRing ? Lr[(ph + lane) & M] : R[(ph + lane) & M];
            const uint2 qe = QRing ? R[(qh + lane) & M] : Lr[(qh + lane) & M];
            /* the popped ring entry goes to its place in the global queue,
             * the record the bucket pass reads */
            if (QRing)
                Q[qh + lane] = qe;
            else
                P[ph + lane] = pe;
            const float pv = __uint_as_float(pe.y), qv = __uint_as_float(qe.y);
            const float r = fsub(qv, fsub(ave, pv));
            conv = r < ave;
            ne = make_uint2(qe.x, __float_as_uint(r));
        }
        const uint32_t mc = __ballot_sync(kFullMask, act && conv), ms = __ballot_sync(kFullMask, act && !conv);
        __syncwarp(); /* every lane has read its ring entries before any append lands */
        if (act)
        {
            if (conv)
            {
                const uint32_t j = pt + __popc(mc & lt);
                if (QRing)
                    P[j] = ne;
                else
                    R[j & M] = ne;
            }
            else
            {
                const uint32_t j = qt + __popc(ms & lt);
                if (QRing)
                    R[j & M] = ne;
                else
                    Q[j] = ne;
            }
        }
        __syncwarp();
        ph += b;
        qh += b;
        pt += __popc(mc);
        qt += __popc(ms);
    }
    const uint32_t h1 = QRing ? qh : ph, t1 = QRing ? qt : pt;
    for (uint32_t j = h1 + lane; j < t1; j += 32)
        G[j] = R[j & M];
    __syncwarp();
}

/* ---- a row's sum, exact and in parallel ------------------------------------
 *
 * The alias build needs each row's sum as the reference adds it: one float
 * rounding per term, in edge order (include/walk.hpp:579-584).  As a serial
 * FADD chain it costs one thread several cycles per edge (a 163,585-edge hub
 * row: ~0.4 ms while the rest of its block waits).  For non-negative finite
 * terms the partial sums never decrease, so they pass through each binade
 * [2^e, 2^(e+1)) once.  Inside one binade every partial sum is a multiple of
 * u = 2^(e-23), and s + x rounds to s + m*u or s + (m+1)*u with m = floor(x/u):
 * to the nearest, a tie to the even significand, which depends only on the
 * parity of S = s/u.  So each term acts on the significand as a map
 * S -> S + a[S & 1], and such maps compose:
 *     (f then g)[p] = f[p] + g[(p + f[p]) & 1].
 * A block scan of the maps over a window of terms gives every partial sum of
 * the window at once.  The first term whose partial sum would reach 2^(e+1)
 * is added with a real FADD to the exact partial sum before it, and the next
 * window starts after it in the new binade.  Partial sums below 2^-103 and
 * rows with a negative, negative-zero or non-finite term take the serial
 * chain.  The result is the serial chain's, bit for bit. */
struct SumMap
{
    uint32_t a0, a1; /* increments of S, in units of u, for S even / odd */
};
constexpr uint32_t kSumSat = 1u << 26; /* saturation: past any binade */

__device__ __forceinline__ SumMap summap_then(SumMap f, SumMap g)
{
    const uint32_t c0 = f.a0 + ((f.a0 & 1u) ? g.a1 : g.a0);
    const uint32_t c1 = f.a1 + ((f.a1 & 1u) ? g.a0 : g.a1);
    return SumMap{min(c0, kSumSat), min(c1, kSumSat)};
}

/* The map of adding term x, scale = 1/u (a power of two). */
__device__ __forceinline__ SumMap summap_term(float x, float scale)
{
    const float xs = fmul(x, scale); /* exact: a power-of-two scaling */
    if (!(xs < 33554432.0f))         /* 2^25 (and inf): past the binade */
        return SumMap{kSumSat, kSumSat};
    const uint32_t m = __float2uint_rz(xs);
    const float fr = fsub(xs, u2f(m)); /* exact */
    if (fr > 0.5f)
        return SumMap{m + 1u, m + 1u};
    if (fr < 0.5f)
        return SumMap{m, m};
    return SumMap{m + (m & 1u), m + ((m + 1u) & 1u)};
}

/* Inclusive and exclusive scans of the block's maps in thread order.
 * s_maps: 33 SumMaps of shared memory. */
__device__ __forceinline__ void block_scan_maps(SumMap mine, SumMap &inc, SumMap &exc, SumMap *s_maps)
{
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    inc = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const SumMap prev{__shfl_up_sync(kFullMask, inc.a0, o), __shfl_up_sync(kFullMask, inc.a1, o)};
        if (lane >= (uint32_t)o)
            inc = summap_then(prev, inc);
    }
    SumMap wexc{__shfl_up_sync(kFullMask, inc.a0, 1), __shfl_up_sync(kFullMask, inc.a1, 1)};
    if (lane == 0)
        wexc = SumMap{0u, 0u};
    if (lane == 31)
        s_maps[wid] = inc;
    __syncthreads();
    if (wid == 0)
    {
        SumMap t = lane < nw ? s_maps[lane] : SumMap{0u, 0u};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const SumMap prev{__shfl_up_sync(kFullMask, t.a0, o), __shfl_up_sync(kFullMask, t.a1, o)};
            if (lane >= (uint32_t)o)
                t = summap_then(prev, t);
        }
        SumMap te{__shfl_up_sync(kFullMask, t.a0, 1), __shfl_up_sync(kFullMask, t.a1, 1)};
        if (lane == 0)
            te = SumMap{0u, 0u};
        if (lane < nw)
            s_maps[lane] = te; /* the maps of the warps before `lane` */
    }
    __syncthreads();
    const SumMap before = s_maps[wid];
    inc = summap_then(before, inc);
    exc = summap_then(before, wexc);
    __syncthreads(); /* s_maps is free again */
}

/* The row's sum (every thread of the block gets it): terms load(0..deg), K
 * per thread per window after a serial head of 2 * blockDim.x terms.
 * s_maps: 33 SumMaps, s_f: 1 float, s_u: 1 word of shared memory; s_head:
 * 2 * blockDim.x floats of shared memory the block stages the head in (so
 * that the serial chain reads shared memory, not one global load after
 * another), or nullptr when load() already reads shared memory. */
template <uint32_t K, typename Load>
__device__ float block_exact_sum(Load load, uint32_t deg, SumMap *s_maps, float *s_f, uint32_t *s_u,
                                 float *s_head)
{
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t head = deg < 2u * nt ? deg : 2u * nt;
    if (s_head != nullptr)
    {
        for (uint32_t i = tid; i < head; i += nt)
            s_head[i] = load(i);
        __syncthreads();
    }
    /* the first terms on one thread: the partial sums double every few
     * terms there, which would end a window every few terms */
    if (tid == 0)
    {
        float s = 0.0f;
        uint32_t i = 0;
        if (s_head != nullptr)
        {
            for (; i + 8 <= head; i += 8)
                s = fadd(fadd(fadd(fadd(fadd(fadd(fadd(fadd(s, s_head[i]), s_head[i + 1]), s_head[i + 2]),
                                                 s_head[i + 3]),
                                            s_head[i + 4]),
                                       s_head[i + 5]),
                                  s_head[i + 6]),
                             s_head[i + 7]);
            for (; i < head; i++)
                s = fadd(s, s_head[i]);
        }
        else
        {
            for (; i < head; i++)
                s = fadd(s, load(i));
        }
        *s_f = s;
        *s_u = i;
    }
    __syncthreads();
    float s = *s_f;
    uint32_t pos = *s_u;
    __syncthreads();
    while (pos < deg)
    {
        const uint32_t bits = __float_as_uint(s), ex = (bits >> 23) & 0xFFu;
        const uint32_t base = pos + tid * K;
        float xk[K];
        /* sums below 2^-103, inf, NaN and negative sums take the serial chain */
        bool odd = !(ex >= 24u && ex < 255u) || bits >= 0x80000000u;
        SumMap m{0u, 0u};
        const float scale = __uint_as_float((277u - (ex < 24u ? 24u : ex > 254u ? 254u : ex)) << 23);
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            const float x = base + j < deg ? load(base + j) : 0.0f;
            xk[j] = x;
            odd = odd || __float_as_uint(x) >= 0x7F800000u; /* negative (incl. -0), inf, NaN */
            m = summap_then(m, summap_term(x, scale));
        }
        if (__syncthreads_or(odd))
        {
            /* the serial chain for the rest of the row */
            if (tid == 0)
            {
                for (uint32_t i = pos; i < deg; i++)
                    s = fadd(s, load(i));
                *s_f = s;
            }
            __syncthreads();
            s = *s_f;
            __syncthreads();
            break;
        }
        const uint32_t S = (bits & 0x7FFFFFu) | 0x800000u, p0 = S & 1u;
        const float u = __uint_as_float((ex - 23u) << 23);
        SumMap inc, exc;
        block_scan_maps(m, inc, exc, s_maps);
        const uint32_t end = S + (p0 ? inc.a1 : inc.a0);
        /* partial sums never decrease, so the threads whose terms stay in
         * the binade come first */
        const uint32_t stay = (uint32_t)__syncthreads_count(end < (1u << 24));
        if (stay == nt)
        {
            if (tid == nt - 1)
                *s_f = fmul(u2f(end), u);
            __syncthreads();
            s = *s_f;
            pos += nt * K;
            __syncthreads();
            continue;
        }
        if (tid == stay)
        {
            uint32_t Sj = S + (p0 ? exc.a1 : exc.a0);
            bool found = false;
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                const SumMap t = summap_term(xk[j], scale);
                const uint32_t a = (Sj & 1u) ? t.a1 : t.a0;
                if (!found && Sj + a >= (1u << 24))
                {
                    *s_f = fadd(fmul(u2f(Sj), u), xk[j]);
                    *s_u = base + j + 1;
                    found = true;
                }
                Sj += a;
            }
            if (!found)
            {
                /* unreachable by the argument above; should it ever be
                 * reached, the serial chain finishes the row exactly */
                float r = fmul(u2f(S + (p0 ? exc.a1 : exc.a0)), u);
                for (uint32_t i = base; i < deg; i++)
                    r = fadd(r, load(i));
                *s_f = r;
                *s_u = deg;
            }
        }
        __syncthreads();
        s = *s_f;
        pos = *s_u;
        __syncthreads();
    }
    return s;
}

/* The same exact sum for one row in shared memory on one warp (every lane
 * gets it): a serial head of 64 terms on lane 0, then windows of 32 K terms
 * scanned across the lanes. */
template <uint32_t K>
__device__ float warp_exact_sum(const float *F, uint32_t deg)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t head = deg < 64u ? deg : 64u;
    float s = 0.0f;
    if (lane == 0)
        for (uint32_t i = 0; i < head; i++)
            s = fadd(s, F[i]);
    s = __shfl_sync(kFullMask, s, 0);
    uint32_t pos = head;
    while (pos < deg)
    {
        const uint32_t bits = __float_as_uint(s), ex = (bits >> 23) & 0xFFu;
        const uint32_t base = pos + lane * K;
        float xk[K];
        bool odd = !(ex >= 24u && ex < 255u) || bits >= 0x80000000u;
        SumMap m{0u, 0u};
        const float scale = __uint_as_float((277u - (ex < 24u ? 24u : ex > 254u ? 254u : ex)) << 23);
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            const float x = base + j < deg ? F[base + j] : 0.0f;
            xk[j] = x;
            odd = odd || __float_as_uint(x) >= 0x7F800000u;
            m = summap_then(m, summap_term(x, scale));
        }
        if (__any_sync(kFullMask, odd))
        {
            if (lane == 0)
                for (uint32_t i = pos; i < deg; i++)
                    s = fadd(s, F[i]);
            s = __shfl_sync(kFullMask, s, 0);
            break;
        }
        const uint32_t S = (bits & 0x7FFFFFu) | 0x800000u, p0 = S & 1u;
        const float u = __uint_as_float((ex - 23u) << 23);
        SumMap inc = m;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const SumMap prev{__shfl_up_sync(kFullMask, inc.a0, o), __shfl_up_sync(kFullMask, inc.a1, o)};
            if (lane >= (uint32_t)o)
                inc = summap_then(prev, inc);
        }
        SumMap exc{__shfl_up_sync(kFullMask, inc.a0, 1), __shfl_up_sync(kFullMask, inc.a1, 1)};
        if (lane == 0)
            exc = SumMap{0u, 0u};
        const uint32_t end = S + (p0 ? inc.a1 : inc.a0);
        const uint32_t stay = (uint32_t)__popc(__ballot_sync(kFullMask, end < (1u << 24)));
        if (stay == 32u)
        {
            s = fmul(u2f(__shfl_sync(kFullMask, end, 31)), u);
            pos += 32u * K;
            continue;
        }
        float ns = 0.0f;
        uint32_t np = 0;
        if (lane == stay)
        {
            uint32_t Sj = S + (p0 ? exc.a1 : exc.a0);
            bool found = false;
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                const SumMap t = summap_term(xk[j], scale);
                const uint32_t a = (Sj & 1u) ? t.a1 : t.a0;
                if (!found && Sj + a >= (1u << 24))
                {
                    ns = fadd(fmul(u2f(Sj), u), xk[j]);
                    np = base + j + 1;
                    found = true;
                }
                Sj += a;
            }
            if (!found)
            {
                /* unreachable (see block_exact_sum); the serial chain if not */
                ns = fmul(u2f(S + (p0 ? exc.a1 : exc.a0)), u);
                for (uint32_t i = base; i < deg; i++)
                    ns = fadd(ns, F[i]);
                np = deg;
            }
        }
        s = __shfl_sync(kFullMask, ns, stay);
        pos = __shfl_sync(kFullMask, np, stay);
    }
    return s;
}

/* Block-wide exclusive scan of two counts packed as a | b << 16 (each total
 * below 2^16): exclusive prefix and total.  s_w: 33 words of shared memory. */
__device__ __forceinline__ uint32_t block_scan_packed(uint32_t x, uint32_t &total, uint32_t *s_w)
{
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(kFullMask, inc, o);
        if (lane >= (uint32_t)o)
            inc += y;
    }
    if (lane == 31)
        s_w[wid] = inc;
    __syncthreads();
    if (wid == 0)
    {
        const uint32_t t = lane < nw ? s_w[lane] : 0u;
        uint32_t ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(kFullMask, ti, o);
            if (lane >= (uint32_t)o)
                ti += y;
        }
        if (lane < nw)
            s_w[lane] = ti - t;
        if (lane == 31)
            s_w[32] = ti;
    }
    __syncthreads();
    const uint32_t ex = s_w[wid] + inc - x;
    total = s_w[32];
    __syncthreads();
    return ex;
}

/* Stable block-wide split, K consecutive terms per thread per pass: terms
 * below ave to the p queue, the rest to the q queue, in edge order
 * (:593-602). */
template <uint32_t K, typename Load>
__device__ __forceinline__ void block_split_wide(Load load, uint32_t deg, float ave, uint2 *P, uint2 *Q,
                                                 uint32_t &pt, uint32_t &qt, uint32_t *s_w)
{
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    pt = 0;
    qt = 0;
    /* the next pass's terms are loaded before this pass's scan, so their
     * latency hides behind its barriers */
    float nx[K];
#pragma unroll
    for (uint32_t j = 0; j < K; j++)
        nx[j] = tid * K + j < deg ? load(tid * K + j) : 0.0f;
    for (uint32_t base = 0; base < deg; base += nt * K)
    {
        const uint32_t i0 = base + tid * K;
        float xk[K];
        uint32_t cs = 0, cb = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            const bool valid = i0 + j < deg;
            xk[j] = nx[j];
            cs += valid && xk[j] < ave;
            cb += valid && !(xk[j] < ave);
        }
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
            nx[j] = i0 + nt * K + j < deg ? load(i0 + nt * K + j) : 0.0f;
        uint32_t tot;
        const uint32_t ex = block_scan_packed(cs | (cb << 16), tot, s_w);
        uint32_t ps = pt + (ex & 0xFFFFu), qs = qt + (ex >> 16);
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            if (i0 + j < deg)
            {
                const uint2 ent = make_uint2(i0 + j, __float_as_uint(xk[j]));
                if (xk[j] < ave)
                    P[ps++] = ent;
                else
                    Q[qs++] = ent;
            }
        }
        pt += tot & 0xFFFFu;
        qt += tot >> 16;
    }
    __syncthreads();
}

/* Pairing loop of a block (:603-638) with K iterations per thread per batch:
 * batches of up to nt * K iterations while both queues are long, warp 0
 * alone for short stretches; then the q leftovers. */
template <uint32_t K, typename Bucket>
__device__ __forceinline__ void block_pairing_wide(uint2 *P, uint2 *Q, uint32_t pt, uint32_t qt, float ave,
                                                   Bucket *ob, const uint32_t *nb, const uint64_t *vcur,
                                                   const uint8_t *ty, uint32_t *s_w, uint32_t *s_state, uint2 *ring)
{
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t deg = pt + qt;
    uint32_t ph = 0, qh = 0;
    while (ph < pt)
    {
        const uint32_t lp = pt - ph, lq = qt - qh;
        if (lq == 0)
            break;
        const uint32_t b = min(min(lp, lq), nt * K);
        if (b <= 64)
        {
            if (tid < 32)
            {
                if (lq <= lp)
                    warp_pairing_ring<true>(P, Q, ring, ring + kRingSize, ph, pt, qh, qt, ave, 128);
                else
                    warp_pairing_ring<false>(P, Q, ring, ring + kRingSize, ph, pt, qh, qt, ave, 128);
                if (tid == 0)
                {
                    s_state[0] = ph;
                    s_state[1] = pt;
                    s_state[2] = qh;
                    s_state[3] = qt;
                }
            }
            __syncthreads();
            ph = s_state[0];
            pt = s_state[1];
            qh = s_state[2];
            qt = s_state[3];
            __syncthreads();
            continue;
        }
        /* iterations tid*K .. tid*K + K - 1 of the batch */
        const uint32_t i0 = tid * K;
        uint2 ne[K];
        uint32_t convm = 0, nc = 0, ns = 0;
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            const uint32_t i = i0 + j;
            ne[j] = make_uint2(0u, 0u);
            if (i < b)
            {
                const uint2 pe = P[ph + i], qe = Q[qh + i];
                const float pv = __uint_as_float(pe.y), qv = __uint_as_float(qe.y);
                const float r = fsub(qv, fsub(ave, pv));
                ne[j] = make_uint2(qe.x, __float_as_uint(r));
                if (r < ave)
                {
                    convm |= 1u << j;
                    nc++;
                }
                else
                {
                    ns++;
                }
            }
        }
        uint32_t tot;
        const uint32_t ex = block_scan_packed(nc | (ns << 16), tot, s_w);
        uint32_t pc = pt + (ex & 0xFFFFu), qs = qt + (ex >> 16);
#pragma unroll
        for (uint32_t j = 0; j < K; j++)
        {
            if (i0 + j < b)
            {
                if (convm & (1u << j))
                    P[pc++] = ne[j];
                else
                    Q[qs++] = ne[j];
            }
        }
        __syncthreads();
        ph += b;
        qh += b;
        pt += tot & 0xFFFFu;
        qt += tot >> 16;
    }
    /* the buckets in pop order: iteration k popped P[k] and Q[k] (both kept
     * in the linear queues; a p entry's value is final when pushed), then
     * the leftovers of whichever queue is non-empty with p = 1 (:623-638) */
    for (uint32_t k = tid; k < deg; k += nt)
    {
        if (k < ph)
        {
            const uint2 pe = P[k], qe = Q[k];
            ob[k] = Bucket::make(fdiv(__uint_as_float(pe.y), ave), pe.x, qe.x, nb, vcur, ty);
        }
        else
        {
            const uint32_t x = k < pt ? P[k].x : Q[qh + (k - pt)].x;
            ob[k] = Bucket::make(1.0f, x, kNone, nb, vcur, ty);
        }
    }
    __syncthreads();
}

/* Group tiers: a group of G lanes per vertex of degree <= DMAX, 32/G vertices
 * per warp side by side, each row staged in shared memory at 8 B/edge:
 *   F[i]   its probability (static_comp), then its residual (prob[] of :582,
 *          updated in place as :613 does);
 *   Pq, Qq the two queues as linear arrays of 16-bit edge indices (each
 *          receives at most deg entries), which also record every pairing:
 *          iteration k pops Pq[k] and Qq[k].
 * A pairing batch is min(lp, lq, G) iterations on the group's lanes, so a
 * vertex whose batches are short shares its warp with other vertices instead
 * of idling 32 - b lanes.  The pairing loop only moves queue entries and
 * residuals; the buckets are written after it in one converged pass, which
 * reads the candidates' neighbours from the row in global memory (keeping
 * them out of shared memory lets more warps share an SM).  Vertices are
 * taken from *next in degree-descending order, 32/G consecutive ones per
 * warp (vertices of similar degree side by side). */
/* The end of a pairing whose q queue holds one entry q, the usual way a FIFO
 * pairing ends (one heavy edge left, include/walk.hpp:603-630).  Every
 * iteration then pops the next p and the same q: r -= ave - prob[p], and q
 * goes back to the q tail while r >= ave.  The pairing ends at the first
 * r < ave (q to the p tail, the q queue empty) or when the p queue runs out
 * (q left in the q queue).  A group runs those iterations as one chain of
 * subtractions with the reference's roundings in its order, G pops at a
 * time: lane j of the group computes ave - prob[P[ph + j]] and every lane of
 * the group folds the differences in turn from shuffles, at a few
 * instructions per iteration instead of a batch's ballots and compaction.
 * Q[k] = q records each pop for the bucket pass.  Groups in any other state
 * run empty chains, so the warp stays converged. */
template <uint32_t G>
__device__ __forceinline__ void alias_q1_chain(float *F, uint16_t *Pq, uint16_t *Qq, uint32_t &ph, uint32_t &pt,
                                               uint32_t &qh, uint32_t &qt, float ave, uint32_t gl, uint32_t gsh)
{
    bool chain = ph < pt && qt - qh == 1;
    if (!__any_sync(kFullMask, chain))
        return;
    const uint32_t q = chain ? Qq[qh] : 0u;
    float r = chain ? F[q] : 0.0f;
    while (__any_sync(kFullMask, chain))
    {
        const uint32_t avail = chain ? min(pt - ph, G) : 0u;
        const float dj = gl < avail ? fsub(ave, F[Pq[ph + gl]]) : 0.0f;
        const uint32_t wmax = __reduce_max_sync(kFullMask, avail);
        uint32_t n = avail;
        bool conv = false;
        for (uint32_t j = 0; j < wmax; j++)
        {
            const float d = __shfl_sync(kFullMask, dj, gsh + j);
            if (j < n)
            {
                r = fsub(r, d);
                if (r < ave)
                {
                    conv = true;
                    n = j + 1;
                }
            }
        }
        if (gl < n)
            Qq[qh + gl] = (uint16_t)q;
        ph += n;
        qh += n;
        if (chain)
        {
            if (conv)
            {
                if (gl == 0)
                {
                    Pq[pt] = (uint16_t)q;
                    F[q] = r;
                }
                pt += 1;
                qt = qh;
                chain = false;
            }
            else
            {
                qt = qh + 1;
                if (ph == pt)
                {
                    if (gl == 0)
                    {
                        Qq[qh] = (uint16_t)q;
                        F[q] = r;
                    }
                    chain = false;
                }
            }
        }
        __syncwarp();
    }
}

template <uint32_t G, uint32_t DMAX>
constexpr size_t alias_group_smem_per_warp()
{
    return (size_t)(32 / G) * DMAX * 8;
}

/* Warps per block of the lane-group kernels: each warp works alone (its own
 * rows, its own slice of shared memory).  Four to a block measured slower
 * on every class at scale 22 (residency is held by registers and shared
 * memory before the limit of 32 blocks per SM), so a block is one warp. */
constexpr uint32_t kAliasGroupWarps = 1;

template <typename TC, typename Bucket, uint32_t G, uint32_t DMAX>
__global__ void __launch_bounds__(32 * kAliasGroupWarps) alias_group_kernel(GraphView g, TC tc, Bucket *out,
                                                                          const uint64_t *vcur, float *sum_out,
                                                                          const RowDesc *rows, uint32_t lo,
                                                                          uint32_t hi, uint32_t *next)
{
    static_assert(G == 1 || G == 2 || G == 4 || G == 8 || G == 16 || G == 32, "group of 1 to 32 lanes");
    static_assert(DMAX % 4 == 0 && DMAX <= 65535, "16-bit queue entries");
    constexpr uint32_t RPW = 32 / G;
    constexpr uint32_t gbits = G == 32 ? kFullMask : (1u << G) - 1u;
    extern __shared__ uint32_t smem_all[];
    /* this warp's slice: 8 B per edge of its RPW rows */
    uint32_t *smem = smem_all + (size_t)(threadIdx.x >> 5) * RPW * DMAX * 2;
    const uint32_t lane = threadIdx.x & 31, grp = lane / G, gl = lane % G, gsh = grp * G;
    const uint32_t glt = (1u << gl) - 1u;
    float *F = reinterpret_cast<float *>(smem) + (size_t)grp * DMAX;
    uint16_t *Pq = reinterpret_cast<uint16_t *>(smem + (size_t)RPW * DMAX) + (size_t)grp * 2 * DMAX;
    uint16_t *Qq = Pq + DMAX;
    /* every loop below runs to the warp's maximum with per-group predicates,
     * so the groups stay converged and share each instruction.  The next
     * vertices' counter value and row descriptors are fetched while the
     * current ones are processed. */
    const uint32_t n = hi - lo;
    uint32_t t = 0;
    if (lane == 0)
        t = atomicAdd(next, RPW);
    t = __shfl_sync(kFullMask, t, 0);
    RowDesc d{0, 0, 0};
    if (t + grp < n)
        d = rows[lo + t + grp];
    while (t < n)
    {
        uint32_t tn = 0;
        if (lane == 0)
            tn = atomicAdd(next, RPW);
        const uint32_t v = d.v, deg = d.deg;
        const int64_t e0 = d.e0;
        const uint32_t wdeg = __reduce_max_sync(kFullMask, deg);
        /* stage the rows' probabilities, G consecutive edges per load */
#pragma unroll 4
        for (uint32_t i = gl; i < wdeg; i += G)
            if (i < deg)
                F[i] = static_at(g, tc, v, e0 + i);
        __syncwarp();
        tn = __shfl_sync(kFullMask, tn, 0);
        RowDesc dn{0, 0, 0};
        if (tn + grp < n)
            dn = rows[lo + tn + grp];
        /* the sum in edge order (:579-584), one lane per group */
        float sum = 0.0f;
        if constexpr (RPW == 1)
        {
            /* rows of 513..2048 edges: the exact warp scan */
            sum = warp_exact_sum<8>(F, deg);
            if (lane == 0 && deg != 0 && sum_out != nullptr)
                sum_out[v] = sum;
        }
        else if (gl == 0)
        {
            /* a group past its row's end adds +0.0f, which leaves a sum of
             * non-negative terms unchanged, so the FADD chain has no select */
            uint32_t i = 0;
            for (; i + 4 <= wdeg; i += 4)
            {
                const float a0 = i < deg ? F[i] : 0.0f, a1 = i + 1 < deg ? F[i + 1] : 0.0f;
                const float a2 = i + 2 < deg ? F[i + 2] : 0.0f, a3 = i + 3 < deg ? F[i + 3] : 0.0f;
                sum = fadd(fadd(fadd(fadd(sum, a0), a1), a2), a3);
            }
            for (; i < wdeg; i++)
                sum = fadd(sum, i < deg ? F[i] : 0.0f);
            if (deg != 0 && sum_out != nullptr)
                sum_out[v] = sum;
        }
        sum = __shfl_sync(kFullMask, sum, gsh);
        const float ave = fdiv(sum, u2f(deg));
        /* split in edge order (:593-602) into two linear queues of 16-bit
         * edge indices, P from the front of its array, Q from the front of
         * its own (each queue gets at most deg entries over the whole
         * pairing: the q tail is B + I - C <= deg) */
        uint32_t pt = 0, qt = 0;
        for (uint32_t base = 0; base < wdeg; base += G)
        {
            const uint32_t i = base + gl;
            const bool valid = i < deg;
            const float x = valid ? F[i] : 0.0f;
            const bool sm = valid && x < ave, bg = valid && !(x < ave);
            const uint32_t mp = (__ballot_sync(kFullMask, sm) >> gsh) & gbits;
            const uint32_t mq = (__ballot_sync(kFullMask, bg) >> gsh) & gbits;
            if (sm)
                Pq[pt + __popc(mp & glt)] = (uint16_t)i;
            if (bg)
                Qq[qt + __popc(mq & glt)] = (uint16_t)i;
            pt += __popc(mp);
            qt += __popc(mq);
        }
        __syncwarp();
        /* pairing (:603-630) in batches of at most G iterations, queue
         * mechanics and residuals only: iteration k pops P[k] and Q[k], so
         * the queues themselves record every pairing, and the buckets are
         * written afterwards in one converged pass.  A p entry's value is
         * final when it is popped (only popped q entries change), so the
         * pass reads the same F[P[k]] the iteration saw.  A batch of b = 0
         * leaves a finished group's state unchanged.  A group whose q queue
         * holds a single entry leaves the batches for the chain below. */
        uint32_t ph = 0, qh = 0;
        for (;;)
        {
            const bool live = ph < pt && qt - qh > 1;
            if (!__any_sync(kFullMask, live))
                break;
            const uint32_t b = live ? min(min(pt - ph, qt - qh), G) : 0;
            const bool act = gl < b;
            bool conv = false;
            uint32_t qi = 0;
            if (act)
            {
                const uint32_t pi = Pq[ph + gl];
                qi = Qq[qh + gl];
                const float r = fsub(F[qi], fsub(ave, F[pi]));
                F[qi] = r;
                conv = r < ave;
            }
            const uint32_t mc = (__ballot_sync(kFullMask, act && conv) >> gsh) & gbits;
            const uint32_t ms = (__ballot_sync(kFullMask, act && !conv) >> gsh) & gbits;
            if (act)
            {
                if (conv)
                    Pq[pt + __popc(mc & glt)] = (uint16_t)qi;
                else
                    Qq[qt + __popc(ms & glt)] = (uint16_t)qi;
            }
            __syncwarp();
            ph += b;
            qh += b;
            pt += __popc(mc);
            qt += __popc(ms);
        }
        alias_q1_chain<G>(F, Pq, Qq, ph, pt, qh, qt, ave, gl, gsh);
        /* the buckets in pop order: pairs (P[k], Q[k]) for k < ph (= qh),
         * then the leftovers of whichever queue is non-empty with p = 1
         * (:623-638) */
        Bucket *ob = out + e0;
        const uint8_t *ty = g.type != nullptr ? g.type + e0 : nullptr;
        const uint32_t *N = g.nbr + e0; /* the row's neighbours, read from the L1-cached row */
#pragma unroll 2
        for (uint32_t base = 0; base < wdeg; base += G)
        {
            const uint32_t k = base + gl;
            if (k < deg)
            {
                if (k < ph)
                {
                    const uint32_t pi = Pq[k], qi = Qq[k];
                    ob[k] = Bucket::make_n(fdiv(F[pi], ave), pi, qi, N[pi], N[qi], vcur, ty);
                }
                else
                {
                    const uint32_t x = k - ph < pt - ph ? Pq[k] : Qq[qh + (k - pt)];
                    ob[k] = Bucket::make_n(1.0f, x, kNone, N[x], 0, vcur, ty);
                }
            }
        }
        __syncwarp();
        t = tn;
        d = dn;
    }
}

/* Block-row tier: one NT-thread block per vertex of degree <= DMAX, the row
 * staged in shared memory (8 B/edge): F[i] its probability then residual,
 * and the p and q queues as linear arrays of 16-bit edge indices (each holds
 * at most deg entries over the whole pairing, and iteration k pops P[k] and
 * Q[k]).  The split and the pairing batches take four terms or iterations
 * per thread per pass (b = min(lp, lq, 4 NT), conversions and survivors
 * appended by a block-wide scan of per-thread counts) while both queues are
 * long, and warp 0 alone runs them in batches of 32 while one is short.  The
 * buckets are written after the pairing in one pass.  Vertices come from
 * *next, largest first. */
template <uint32_t DMAX>
constexpr size_t alias_block_row_smem()
{
    return (size_t)DMAX * 8;
}

template <typename TC, typename Bucket, uint32_t NT, uint32_t DMAX>
__global__ void __launch_bounds__(NT) alias_block_row_kernel(GraphView g, TC tc, Bucket *out, const uint64_t *vcur,
                                                             float *sum_out, const uint32_t *order, uint32_t lo,
                                                             uint32_t hi, uint32_t *next)
{
    static_assert(NT % 32 == 0 && NT <= 1024 && DMAX % 8 == 0 && DMAX <= 65535, "block-row tier shape");
    extern __shared__ uint32_t smem[];
    constexpr uint32_t K = 4; /* terms or iterations per thread per pass */
    __shared__ uint32_t s_w[33], s_row[4];
    __shared__ SumMap s_maps[33];
    __shared__ float s_f;
    __shared__ uint32_t s_u;
    float *F = reinterpret_cast<float *>(smem);
    uint16_t *P = reinterpret_cast<uint16_t *>(smem + DMAX);
    uint16_t *Q = P + DMAX;
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    for (;;)
    {
        if (tid == 0)
            s_row[0] = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t t = s_row[0];
        if (t >= hi - lo)
            break;
        const uint32_t v = order[lo + t];
        const int64_t e0 = g.off[v];
        const uint32_t deg = (uint32_t)(g.off[v + 1] - e0);
#pragma unroll 4
        for (uint32_t i = tid; i < deg; i += NT)
            F[i] = static_at(g, tc, v, e0 + i);
        __syncthreads();
        /* the sum in edge order (:579-584), exact block scan */
        const float sum = block_exact_sum<4>([&](uint32_t i) { return F[i]; }, deg, s_maps, &s_f, &s_u, nullptr);
        if (tid == 0 && sum_out != nullptr)
            sum_out[v] = sum;
        const float ave = fdiv(sum, u2f(deg));
        /* stable split in edge order (:593-602), K consecutive terms per
         * thread per pass */
        uint32_t pt = 0, qt = 0;
        for (uint32_t base = 0; base < deg; base += NT * K)
        {
            const uint32_t i0 = base + tid * K;
            uint32_t cs = 0, cb = 0;
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                const bool valid = i0 + j < deg;
                const bool sm = valid && F[i0 + j] < ave;
                cs += sm;
                cb += valid && !sm;
            }
            uint32_t tot;
            const uint32_t ex = block_scan_packed(cs | (cb << 16), tot, s_w);
            uint32_t ps = pt + (ex & 0xFFFFu), qs = qt + (ex >> 16);
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                if (i0 + j < deg)
                {
                    if (F[i0 + j] < ave)
                        P[ps++] = (uint16_t)(i0 + j);
                    else
                        Q[qs++] = (uint16_t)(i0 + j);
                }
            }
            pt += tot & 0xFFFFu;
            qt += tot >> 16;
        }
        __syncthreads();
        /* pairing (:603-630); bucket k is the k-th p pop */
        Bucket *ob = out + e0;
        const uint8_t *ty = g.type != nullptr ? g.type + e0 : nullptr;
        uint32_t ph = 0, qh = 0;
        while (ph < pt && qh < qt)
        {
            const uint32_t b = min(min(pt - ph, qt - qh), NT * K);
            if (b <= 64)
            {
                /* warp 0 alone until the pairing ends or both queues are long again */
                if (tid < 32)
                {
                    uint32_t wph = ph, wpt = pt, wqh = qh, wqt = qt;
                    const uint32_t lt = (1u << lane) - 1u;
                    while (wph < wpt && wqh < wqt)
                    {
                        const uint32_t wb = min(min(wpt - wph, wqt - wqh), 32u);
                        if (wb == 32u && min(wpt - wph, wqt - wqh) > 128u)
                            break;
                        const bool act = lane < wb;
                        bool conv = false;
                        uint32_t qi = 0;
                        if (act)
                        {
                            const uint32_t pi = P[wph + lane];
                            qi = Q[wqh + lane];
                            const float r = fsub(F[qi], fsub(ave, F[pi]));
                            F[qi] = r;
                            conv = r < ave;
                        }
                        const uint32_t mc = __ballot_sync(kFullMask, act && conv);
                        const uint32_t ms = __ballot_sync(kFullMask, act && !conv);
                        if (act)
                        {
                            if (conv)
                                P[wpt + __popc(mc & lt)] = (uint16_t)qi;
                            else
                                Q[wqt + __popc(ms & lt)] = (uint16_t)qi;
                        }
                        __syncwarp();
                        wph += wb;
                        wqh += wb;
                        wpt += __popc(mc);
                        wqt += __popc(ms);
                    }
                    if (tid == 0)
                    {
                        s_row[0] = wph;
                        s_row[1] = wpt;
                        s_row[2] = wqh;
                        s_row[3] = wqt;
                    }
                }
                __syncthreads();
                ph = s_row[0];
                pt = s_row[1];
                qh = s_row[2];
                qt = s_row[3];
                __syncthreads();
                continue;
            }
            /* iterations tid*K .. tid*K + K - 1 of the batch */
            const uint32_t i0 = tid * K;
            uint32_t qk[K], convm = 0, nc = 0, ns = 0;
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                qk[j] = 0;
                if (i0 + j < b)
                {
                    const uint32_t pi = P[ph + i0 + j];
                    qk[j] = Q[qh + i0 + j];
                    const float r = fsub(F[qk[j]], fsub(ave, F[pi]));
                    F[qk[j]] = r;
                    if (r < ave)
                    {
                        convm |= 1u << j;
                        nc++;
                    }
                    else
                    {
                        ns++;
                    }
                }
            }
            uint32_t tot;
            const uint32_t ex = block_scan_packed(nc | (ns << 16), tot, s_w);
            uint32_t pc = pt + (ex & 0xFFFFu), qs = qt + (ex >> 16);
#pragma unroll
            for (uint32_t j = 0; j < K; j++)
            {
                if (i0 + j < b)
                {
                    if (convm & (1u << j))
                        P[pc++] = (uint16_t)qk[j];
                    else
                        Q[qs++] = (uint16_t)qk[j];
                }
            }
            __syncthreads();
            ph += b;
            qh += b;
            pt += tot & 0xFFFFu;
            qt += tot >> 16;
        }
        /* the buckets in pop order (iteration k popped P[k] and Q[k]; a p
         * entry's value is final once popped), then the leftovers of
         * whichever queue is non-empty with p = 1 (:623-638) */
        const uint32_t *N = g.nbr + e0; /* the row's neighbours, from global memory */
        for (uint32_t k2 = tid; k2 < deg; k2 += NT)
        {
            if (k2 < ph)
            {
                const uint32_t pi = P[k2], qi2 = Q[k2];
                ob[k2] = Bucket::make_n(fdiv(F[pi], ave), pi, qi2, N[pi], N[qi2], vcur, ty);
            }
            else
            {
                const uint32_t x = k2 < pt ? P[k2] : Q[qh + (k2 - pt)];
                ob[k2] = Bucket::make_n(1.0f, x, kNone, N[x], 0, vcur, ty);
            }
        }
        __syncthreads();
    }
}

/* Hub tier: a 1024-thread block per vertex (256 threads for 4097..16384),
 * queues in global scratch at 2 * off[v].  The row's sum by the exact block
 * scan (block_exact_sum), then the split and the pairing with four terms or
 * iterations per thread per pass, so a 163,585-edge row takes ~40 passes of
 * each instead of one thread's FADD chain and ~160 barrier rounds. */
template <typename TC, typename Bucket>
__global__ void __launch_bounds__(1024) alias_build_hub_kernel(GraphView g, TC tc, Bucket *out, const uint64_t *vcur,
                                                               float *sum_out, uint2 *scratch, const uint32_t *order,
                                                               uint32_t lo, uint32_t hi, uint32_t *next)
{
    __shared__ SumMap s_maps[33];
    __shared__ uint32_t s_w[33], s_state[4];
    __shared__ float s_f;
    __shared__ uint32_t s_u, s_k;
    __shared__ uint2 s_ring[2 * kRingSize]; /* the short queue's ring, the long queue's staged head */
    __shared__ float s_head[2048];
    const uint32_t tid = threadIdx.x;
    for (;;)
    {
        /* vertices from *next, largest first */
        if (tid == 0)
            s_k = lo + atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t k = s_k;
        __syncthreads();
        if (k >= hi)
            break;
        const uint32_t v = order[k];
        const int64_t e0 = g.off[v];
        const uint32_t deg = (uint32_t)(g.off[v + 1] - e0);
        auto load = [&](uint32_t i) { return static_at(g, tc, v, e0 + i); };
        const float sum = block_exact_sum<4>(load, deg, s_maps, &s_f, &s_u, s_head);
        const float ave = fdiv(sum, u2f(deg));
        if (tid == 0 && sum_out != nullptr)
            sum_out[v] = sum;
        uint2 *P = scratch + 2 * e0;
        uint2 *Q = P + deg;
        uint32_t pt, qt;
        block_split_wide<4>(load, deg, ave, P, Q, pt, qt, s_w);
        block_pairing_wide<4>(P, Q, pt, qt, ave, out + e0, g.nbr + e0, vcur, g.type != nullptr ? g.type + e0 : nullptr,
                              s_w, s_state, s_ring);
    }
}

/* Row descriptors of the vertex order. */
static __global__ void row_desc_kernel(GraphView g, const uint32_t *order, RowDesc *rows)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < g.V; i += gridDim.x * blockDim.x)
    {
        const uint32_t v = order[i];
        const int64_t e0 = g.off[v];
        rows[i] = RowDesc{e0, v, (uint32_t)(g.off[v + 1] - e0)};
    }
}

/* Degree-descending vertex order support: degrees and iota for a radix sort. */
static __global__ void degree_keys_kernel(GraphView g, uint32_t *deg, uint32_t *ids)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x)
    {
        deg[v] = (uint32_t)(g.off[v + 1] - g.off[v]);
        ids[v] = v;
    }
}

/* Tier boundaries in the descending degrees: bounds[i] = number of vertices
 * of degree > thr[i] (bounds zeroed by the caller). */
constexpr int kTierBounds = kAliasClasses + 1; /* the class maxima, then 0 */
struct TierThresholds
{
    uint32_t thr[kTierBounds];
};

static __global__ void tier_bounds_kernel(const uint32_t *sorted_deg, uint32_t n, TierThresholds t, uint32_t *bounds)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t d = sorted_deg[i], dn = i + 1 < n ? sorted_deg[i + 1] : 0;
#pragma unroll
        for (int k = 0; k < kTierBounds; k++)
            if (d > t.thr[k] && dn <= t.thr[k])
                bounds[k] = i + 1;
    }
}

/* regular_area (include/walk.hpp:750-781): sum * ub with a static component,
 * deg * ub without. */
template <typename TC>
__global__ void regular_area_kernel(GraphView g, TC tc, const float *sum, float *ra)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x)
    {
        AdjList adj{(edge_id_t)g.off[v], (edge_id_t)g.off[v + 1]};
        float ub = tc.dcomp_upperbound(v, adj);
        if (TC::has_static)
            ra[v] = fmul(sum[v], ub);
        else
            ra[v] = fmul(u2f(adj.degree()), ub);
    }
}

/* ---- walk kernels -------------------------------------------------------- */

/* walk status words: an OR of these flags */
#define KK_STATUS_OK 0
#define KK_STATUS_TRIAL_LIMIT 4
#define KK_STATUS_PATH_CAPACITY 8
#define KK_STATUS_BAD_START 16

struct WalkLaunch
{
    uint64_t seed;
    walker_id_t walker_begin;
    uint32_t walker_num;
    const uint64_t *path_off; /* per-walker path offsets (walker_num+1), or nullptr: i * cap */
    uint32_t cap;             /* fixed path capacity (vertices) when path_off is nullptr */
    uint32_t *path;           /* nullptr: lengths only */
    uint32_t *length;
    const uint32_t *start;    /* optional start-vertex list, start[id % n_start] */
    uint32_t n_start;
    unsigned long long *total_steps;
    const float *alias_sum; /* static-component sums, for regular_area when ra is not precomputed */
    int *status;
    uint32_t trial_limit;
    unsigned long long *stats; /* trials, queries, probes of the launch, or nullptr */
    /* streamed copy-out (kk_walk_into): finished walkers counted per segment
     * of 2^seg_shift walkers; the segment's last walker sets its flag in
     * mapped host memory, and the host copies the segment's paths out while
     * the walk goes on.  seg_count == nullptr: no counting. */
    uint32_t *seg_count = nullptr;
    volatile uint32_t *seg_flag = nullptr;
    uint32_t seg_shift = 0;
    /* a segment's status word (batches of served requests: each request is a
     * segment with its own status), reported in its flag as 1 + status;
     * nullptr: the flag is 1 */
    const int *seg_status = nullptr;
    /* parking (first-order walks with rejection trials): once fewer than
     * park_below of a warp's lanes are still walking, each of them stops at
     * its next step boundary and is appended to park (a ParkedWalker<S>
     * array, park_count entries), so that the warp ends and a later launch
     * resumes the stragglers 32 to a warp.  park == nullptr: no parking. */
    void *park = nullptr;
    uint32_t *park_count = nullptr;
    uint32_t park_below = 0;
};

/* Trials each lane runs on its own between a parking warp's ballots (metapath
 * S22: 1 -> 16.8 ms, 8 -> 13.6 ms, 16 -> 13.7 ms per walk). */
constexpr uint32_t kParkCheck = 8;

/* Walker i has written its whole path and its length.  The lanes that end a
 * walker of the same segment together are counted by one of them (a counter
 * per walker serialises the resident threads on the few segments they are
 * all finishing: +40% walk time at 4 M walkers).  The warp barrier orders the
 * lanes' writes before that lane's release add (performed in device memory
 * no later than the count; no acquire, so the SM's L1 keeps its lines).  The
 * segment's last count is followed by an acquire-release fence at device
 * scope, which orders every counted walker's writes before the flag's store
 * to host memory.  The host issues the segment's copy on seeing the flag, and
 * the copy engine reads device memory through the same L2, so it reads
 * finished paths; no system-scope fence is needed (the data never goes to
 * the host by any other route). */
__device__ __forceinline__ void segment_done(const WalkLaunch &L, uint32_t i)
{
    if (L.seg_count == nullptr)
        return;
    const uint32_t s = i >> L.seg_shift;
    /* lanes of one warp may walk for different launches' segments (the jobs
     * of a batch): they count together only on the same counter */
    const unsigned peers = __match_any_sync(__activemask(), (unsigned long long)(L.seg_count + s));
    __syncwarp(peers);
    if ((int)(threadIdx.x & 31) != __ffs(peers) - 1)
        return;
    const uint32_t left = L.walker_num - (s << L.seg_shift);
    const uint32_t size = left < (1u << L.seg_shift) ? left : (1u << L.seg_shift);
    const uint32_t add = (uint32_t)__popc(peers);
    uint32_t old;
    asm volatile("atom.release.gpu.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(L.seg_count + s), "r"(add) : "memory");
    if (old + add == size)
    {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        /* every walker of the segment released its status update before its
         * count: the status word is final here */
        const uint32_t f = L.seg_status != nullptr ? 1u + (uint32_t)*(const volatile int *)L.seg_status : 1u;
        asm volatile("st.relaxed.sys.u32 [%0], %1;" ::"l"(L.seg_flag + s), "r"(f) : "memory");
    }
}

template <typename S, typename WC>
__device__ __forceinline__ vertex_id_t walker_start(const GraphView &g, const WC &wc, const WalkLaunch &L,
                                                    Walker<S> &w, Sampler &rng)
{
    vertex_id_t v;
    if constexpr (is_hook<decltype(wc.walker_init_dist)>())
    {
        rng.enter(w.id, 0, 2);
        v = wc.walker_init_dist(w.id, rng);
    }
    else if (L.start != nullptr)
    {
        v = L.start[w.id % L.n_start];
    }
    else
    {
        v = w.id % g.V;
    }
    if (v >= g.V)
    {
        /* a start vertex outside the graph fails the call (the host reads
         * the status); the walker stands on vertex 0 meanwhile */
        atomicOr(L.status, KK_STATUS_BAD_START);
        v = 0;
    }
    if constexpr (is_hook<decltype(wc.walker_init_state)>())
    {
        rng.enter(w.id, 0, 1);
        wc.walker_init_state(w, v, rng);
    }
    return v;
}

/* Whether a respond_query hook reads the target's adjacency: hooks may say
 * so per call with `bool needs_adjacency() const`; others always get it. */
template <typename F, typename = void>
struct has_needs_adjacency : std::false_type
{
};
template <typename F>
struct has_needs_adjacency<F, std::void_t<decltype(std::declval<const F &>().needs_adjacency())>> : std::true_type
{
};
template <typename F>
__device__ __forceinline__ bool respond_needs_adjacency(const F &f)
{
    if constexpr (has_needs_adjacency<F>::value)
        return f.needs_adjacency();
    else
        return true;
}

/* Whether a post_query hook offers query_matters(walker, candidate, dart). */
template <typename F, typename S, typename = void>
struct has_query_matters : std::false_type
{
};
template <typename F, typename S>
struct has_query_matters<F, S,
                         std::void_t<decltype(std::declval<const F &>().query_matters(
                             std::declval<const Walker<S> &>(), std::declval<const AdjUnit &>(), 0.0f))>>
    : std::true_type
{
};

/* A picked candidate: index local to the adjacency (kNone when the bucket
 * does not carry it), neighbour, and the neighbour's cursor when the bucket
 * carries one (has_cur). */
struct Cand
{
    uint32_t idx;
    vertex_id_t nbr;
    uint64_t cur;
    bool has_cur;
    uint32_t tag; /* AdjUnit::type_tag of the candidate edge */
};

/* Candidate pick: uniform (include/walk.hpp:1016-1018) or alias
 * (:1020-1028; the coin is drawn only when the bucket has an alias).  A
 * bucket is read as the two 16 B halves of its 32 B sector. */
template <typename TC, typename Bucket>
__device__ __forceinline__ Cand pick_candidate(const GraphView &g, const Bucket *alias, const Pos &pos, Sampler &rng)
{
    if constexpr (TC::has_static && Bucket::compact)
    {
        /* b = {p, p_nbr, q_nbr, p_type tag | q_type tag << 16} */
        const uint4 b = gather(reinterpret_cast<const uint4 *>(alias + pos.e0 + rng.gen(pos.deg)));
        if (b.z == kNone || rng.gen_float(1.0f) < __uint_as_float(b.x))
            return Cand{kNone, b.y, 0, false, b.w & 0xffffu};
        return Cand{kNone, b.z, 0, false, b.w >> 16};
    }
    else if constexpr (TC::has_static)
    {
        const uint4 *b4 = reinterpret_cast<const uint4 *>(alias + pos.e0 + rng.gen(pos.deg));
        const uint4 lo = gather(b4), hi = gather(b4 + 1);
        if constexpr (Bucket::cursor)
        {
            /* lo = {p, p_nbr, q_nbr, -}, hi = {p_cur, q_cur} */
            if (lo.z == kNone || rng.gen_float(1.0f) < __uint_as_float(lo.x))
                return Cand{kNone, lo.y, ((uint64_t)hi.y << 32) | hi.x, true, 0};
            return Cand{kNone, lo.z, ((uint64_t)hi.w << 32) | hi.z, true, 0};
        }
        else
        {
            /* lo = {p, p_idx, q_idx, -}, hi = {p_nbr, q_nbr, p_type tag, q_type tag} */
            if (lo.z == kNone || rng.gen_float(1.0f) < __uint_as_float(lo.x))
                return Cand{lo.y, hi.x, 0, false, hi.z};
            return Cand{lo.z, hi.y, 0, false, hi.w};
        }
    }
    else
    {
        const uint32_t c = rng.gen(pos.deg);
        if (g.adjc != nullptr)
        {
            const uint4 a = gather(g.adjc + pos.e0 + c);
            return Cand{c, a.x, ((uint64_t)a.w << 32) | a.z, true, 0};
        }
        return Cand{c, gather(g.nbr + pos.e0 + c), 0, false, 0};
    }
}

__device__ __forceinline__ void flush_steps(unsigned long long *total, unsigned long long mine)
{
    for (int o = 16; o > 0; o >>= 1)
        mine += __shfl_down_sync(0xffffffffu, mine, o);
    if ((threadIdx.x & 31) == 0 && mine != 0)
        atomicAdd(total, mine);
}


/* regular_area[v] (include/walk.hpp:750-781): precomputed, or computed per
 * use with the same two roundings, sum * ub or deg * ub, when the upper
 * bound differs per job of a batch. */
template <typename TC>
__device__ __forceinline__ float regular_area(const TC &tc, const float *ra, const WalkLaunch &L, vertex_id_t v,
                                              const AdjList &adj)
{
    if (ra != nullptr)
        return gather(ra + v);
    const float base = TC::has_static ? gather(L.alias_sum + v) : u2f(adj.degree());
    return fmul(base, tc.dcomp_upperbound(v, adj));
}

/* One walker's loop state: the walker, the vertex it stands on and that
 * vertex's adjacency position (pos.e0 < 0: not read yet), the vertex it came
 * from with its position (second-order queries to it need no offset read),
 * and its path slot. */
template <typename S>
struct WalkerRun
{
    Walker<S> w;
    vertex_id_t v;
    Pos pos;
    vertex_id_t pv;
    Pos ppos;
    uint32_t *out;
    uint32_t cap;
    uint32_t len;
    /* the current step: started (stream entered), extension still to test,
     * its trials so far, and its outlier bound once computed */
    bool in_step, need_ext, ob_known;
    uint32_t step_trials;
    real_t ob_c;
    vertex_id_t on_c;
    /* access counts of the walk (reported when the launch asks for them):
     * rejection trials, second-order queries, and the probes a binary search
     * of the target's sorted adjacency takes for those queries */
    uint32_t trials, queries, probes;
};

/* Per-thread access counts of finished walks, flushed once per thread. */
struct WalkCounts
{
    unsigned long long trials = 0, queries = 0, probes = 0;
    template <typename S>
    __device__ __forceinline__ void add(const WalkerRun<S> &r)
    {
        trials += r.trials;
        queries += r.queries;
        probes += r.probes;
    }
    __device__ __forceinline__ void flush(unsigned long long *stats)
    {
        if (stats == nullptr)
            return;
        flush_steps(stats, trials);
        flush_steps(stats + 1, queries);
        flush_steps(stats + 2, probes);
    }
};

/* Starts walker i of the launch: id, value-initialised state, start vertex,
 * init state, path slot with the start vertex (include/walk.hpp:440-497). */
template <typename S, typename WC>
__device__ __forceinline__ void walk_begin(const GraphView &g, const WC &wc, const WalkLaunch &L, uint32_t i,
                                           WalkerRun<S> &r, Sampler &rng)
{
    r.w.id = L.walker_begin + i;
    r.w.step = 0;
    r.w.data = S{};
    r.v = walker_start<S>(g, wc, L, r.w, rng);
    r.pos = Pos{-1, 0};
    r.pv = kNone;
    r.ppos = Pos{-1, 0};
    const uint64_t pbase = L.path_off ? L.path_off[i] : (uint64_t)i * L.cap;
    r.cap = L.path_off ? (uint32_t)(L.path_off[i + 1] - pbase) : L.cap;
    r.out = L.path ? L.path + pbase : nullptr;
    if (r.out)
        r.out[0] = r.v;
    r.len = 1;
    r.in_step = r.need_ext = r.ob_known = false;
    r.step_trials = 0;
    r.ob_c = 0.0f;
    r.on_c = 0;
    r.trials = r.queries = r.probes = 0;
}

/* One rejection trial of one walker; false when its walk ends.  The kernels
 * loop over trials, not steps: a lane whose trial is accepted starts its next
 * step on the next iteration instead of waiting for the warp's slowest
 * walker to finish its trials (the reference's second order likewise runs one
 * trial per walker per superstep).  The draws are those of the per-step loop:
 * the stream is entered once per step and its counter runs across the step's
 * trials.
 *
 * First order (include/walk.hpp:954-1063): at a step's first trial, degree 0
 * ends the walk, then the extension test (its draw only when 0 < ext < 1).  A
 * trial: [outlier appendix: r = gen_float(area * num + regular_area) -
 * regular_area, r > 0 picks an outlier], candidate by uniform or alias pick,
 * dart = gen_float(ub) accepted under the lower bound or the dynamic
 * component.
 *
 * Second order (include/walk.hpp:1082-1381): a trial is the reference's three
 * supersteps (candidate + query, response, accept), inline.  It starts by
 * re-evaluating the extension (and its draw) as the reference does at the
 * start of every superstep (:1167-1172); a lower-bound pre-accept takes the
 * step at once (:1226-1257); an outlier search that returns no edge retries
 * without a new extension test (:1176-1258).
 *
 * An accepted trial: step++, walker_update_state, the path write
 * (include/walk.hpp:1043-1052).  The new vertex's adjacency position comes
 * from the taken bucket's cursor when it has one, else it is read from the
 * offsets when its step starts. */
template <typename S, typename WC, typename TC, typename Bucket>
__device__ __forceinline__ bool walk_trial(const GraphView &g, const WC &wc, const TC &tc, const Bucket *alias,
                                           const float *ra, const WalkLaunch &L, WalkerRun<S> &run, Sampler &rng)
{
    Walker<S> &w = run.w;
    const vertex_id_t v = run.v;
    if constexpr (TC::order == 1 && !TC::has_dynamic)
    {
        /* every trial is accepted (no dynamic component, hence no outlier):
         * a step is one trial, without the trial state */
        if (run.pos.e0 < 0)
            run.pos = pos_from_offsets(g, v);
        const Pos pos = run.pos;
        if (pos.deg == 0)
            return false;
        rng.enter(w.id, w.step, 0);
        const real_t ext = tc.extension_comp(w, v);
        if (ext == 0.0f || (ext < 1.0f && rng.gen_float(1.0f) > ext))
            return false;
        run.trials++;
        const Cand ac = pick_candidate<TC>(g, alias, pos, rng);
        w.step++;
        if constexpr (is_hook<decltype(wc.walker_update_state)>())
            wc.walker_update_state(w, v, AdjUnit{ac.nbr, (edge_id_t)(pos.e0 + ac.idx)});
        if (run.out)
        {
            if (run.len >= run.cap)
            {
                atomicOr(L.status, KK_STATUS_PATH_CAPACITY);
                return false;
            }
            run.out[run.len] = ac.nbr;
        }
        run.len++;
        run.pv = v;
        run.ppos = pos;
        run.v = ac.nbr;
        run.pos = ac.has_cur ? pos_from_cursor(g, ac.nbr, ac.cur) : Pos{-1, 0};
        return true;
    }
    if (!run.in_step)
    {
        if (run.pos.e0 < 0)
            run.pos = pos_from_offsets(g, v);
        if (run.pos.deg == 0)
            return false;
        rng.enter(w.id, w.step, 0);
        run.in_step = true;
        run.need_ext = true;
        run.step_trials = 0;
        run.ob_known = false;
    }
    const Pos pos = run.pos;
    const int64_t e0 = pos.e0;
    const AdjList adj{(edge_id_t)e0, (edge_id_t)(e0 + pos.deg)};
    Cand ac{kNone, 0, 0, false};
    bool taken = false;
    if (run.need_ext)
    {
        /* first order: once per step; second order: at every superstep */
        const real_t ext = tc.extension_comp(w, v);
        if (ext == 0.0f || (ext < 1.0f && rng.gen_float(1.0f) > ext))
        {
            run.trials += run.step_trials;
            return false;
        }
        run.need_ext = false;
    }
    if (++run.step_trials > L.trial_limit)
    {
        atomicOr(L.status, KK_STATUS_TRIAL_LIMIT);
        run.trials += run.step_trials;
        return false;
    }
    /* outlier appendix; the bound is a pure function of (walker, vertex,
     * adjacency), all fixed within a step, so one call serves every trial */
    bool in_app = false, found = false;
    Cand cd{kNone, 0, 0, false};
    float randval = 0.0f;
    if constexpr (TC::has_outlier)
    {
        if (!run.ob_known)
        {
            tc.outlier_upperbound(w, v, adj, run.ob_c, run.on_c);
            run.ob_known = true;
        }
        const real_t ob = run.ob_c;
        const vertex_id_t on = run.on_c;
        if (ob > 0.0f && on > 0)
        {
            const float rav = regular_area<TC>(tc, ra, L, v, adj);
            const float r = fsub(rng.gen_float(fadd(fmul(ob, u2f(on)), rav)), rav);
            if (r > 0.0f)
            {
                in_app = true;
                uint32_t oi = (uint32_t)fdiv(r, ob);
                if (oi + 1 > on)
                    oi = on - 1;
                AdjUnit cu;
                if (tc.outlier_search(w, v, adj, oi, cu))
                {
                    found = true;
                    float sc = 1.0f;
                    if constexpr (TC::has_static)
                        sc = tc.static_comp(v, cu);
                    randval = fadd(fdiv(fsub(r, fmul(u2f(oi), ob)), sc), tc.dcomp_upperbound(v, adj));
                    cd = Cand{(uint32_t)(cu.index - (edge_id_t)e0), cu.neighbour, 0, false};
                }
            }
        }
    }
    if constexpr (TC::order == 1)
    {
        bool outlier_trial = false;
        if constexpr (TC::has_outlier)
        {
            /* an outlier trial: accepted against the dynamic component, and
             * in any case the next trial follows (no extension test) */
            outlier_trial = in_app;
            if (in_app && found && randval <= tc.dynamic_comp(w, v, AdjUnit{cd.nbr, (edge_id_t)(e0 + cd.idx)}))
            {
                ac = cd;
                taken = true;
            }
        }
        if (!outlier_trial)
        {
            const Cand pc = pick_candidate<TC>(g, alias, pos, rng);
            if constexpr (TC::has_dynamic)
            {
                const float dart = rng.gen_float(tc.dcomp_upperbound(v, adj));
                bool acc = false;
                if constexpr (TC::has_lowerbound)
                    acc = dart <= tc.dcomp_lowerbound(v, adj);
                if (!acc)
                    acc = dart <= tc.dynamic_comp(w, v, AdjUnit{pc.nbr, (edge_id_t)(e0 + pc.idx), pc.tag});
                if (acc)
                {
                    ac = pc;
                    taken = true;
                }
            }
            else
            {
                ac = pc;
                taken = true;
            }
        }
    }
    else
    {
        typedef typename TC::query_type Q;
        typedef typename TC::response_type R;
        if (in_app && !found)
            return true; /* the reference's retry within the superstep: no extension test */
        bool accepted = false;
        if (!in_app)
        {
            cd = pick_candidate<TC>(g, alias, pos, rng);
            randval = rng.gen_float(tc.dcomp_upperbound(v, adj));
            if constexpr (TC::has_lowerbound)
                accepted = randval <= tc.dcomp_lowerbound(v, adj);
        }
        const AdjUnit cu{cd.nbr, (edge_id_t)(e0 + cd.idx), cd.tag};
        if (!accepted)
        {
            R resp{};
            Q query{};
            vertex_id_t target = 0;
            if (tc.post_query(w, v, cu, target, query))
            {
                /* the reference asks here; a post_query hook that can tell
                 * when the answer cannot change the outcome skips the
                 * question.  Counts: queries this engine asks, and the binary
                 * search probes of every question the reference asks (a
                 * launch counting accesses tallies those of skipped ones
                 * too) */
                bool ask = true;
                if constexpr (has_query_matters<decltype(tc.post_query), S>::value)
                    ask = tc.post_query.query_matters(w, cu, randval);
                if (ask || L.stats != nullptr)
                {
                    AdjList tadj{0, 0};
                    if (respond_needs_adjacency(tc.respond_query))
                    {
                        const Pos tp =
                            (target == run.pv && run.ppos.e0 >= 0) ? run.ppos : pos_from_offsets(g, target);
                        tadj = AdjList{(edge_id_t)tp.e0, (edge_id_t)(tp.e0 + tp.deg)};
                        run.probes += 32 - __clz(tp.deg);
                    }
                    if (ask)
                    {
                        run.queries++;
                        tc.respond_query(target, query, tadj, resp);
                    }
                }
            }
            accepted = randval <= tc.dynamic_comp(w, resp, v, cu);
        }
        if (!accepted)
        {
            run.need_ext = true; /* the next superstep re-tests the extension */
            return true;
        }
        ac = cd;
        taken = true;
    }
    if (!taken)
        return true;
    run.trials += run.step_trials;
    run.in_step = false;
    w.step++;
    if constexpr (is_hook<decltype(wc.walker_update_state)>())
        wc.walker_update_state(w, v, AdjUnit{ac.nbr, (edge_id_t)(e0 + ac.idx)});
    if (run.out)
    {
        if (run.len >= run.cap)
        {
            atomicOr(L.status, KK_STATUS_PATH_CAPACITY);
            return false;
        }
        run.out[run.len] = ac.nbr;
    }
    run.len++;
    run.pv = v;
    run.ppos = pos;
    run.v = ac.nbr;
    if (ac.has_cur)
        run.pos = pos_from_cursor(g, ac.nbr, ac.cur);
    else
        run.pos = Pos{-1, 0};
    return true;
}

/* A walker stopped at a step boundary between launches (first-order walks):
 * its position i in the launch, the vertex it stands on, its step, its path
 * length so far and its state.  The stream is keyed by (walker, step), so
 * a walk resumed from this record draws and writes what it would have. */
template <typename S>
struct ParkedWalker
{
    uint32_t i;
    vertex_id_t v;
    step_t step;
    uint32_t len;
    S data;
};

/* Walks that park: first order with rejection trials (a step takes a
 * geometric number of trials and a walk may end at any step, so the lanes
 * of a warp finish far apart). */
template <typename TC>
constexpr bool parks()
{
    return TC::order == 1 && TC::has_dynamic;
}

/* Ends walker i's record in the launch: its length, its segment count, its
 * steps and access counts. */
template <typename S>
__device__ __forceinline__ void walk_finish(const WalkLaunch &L, uint32_t i, const WalkerRun<S> &run,
                                            unsigned long long &my_steps, WalkCounts &counts)
{
    L.length[i] = run.len;
    segment_done(L, i);
    my_steps += run.len - 1;
    counts.add(run);
}

/* Restores parked walker i (its record pw) of launch L at its step boundary. */
template <typename S>
__device__ __forceinline__ void resume_run(const WalkLaunch &L, uint32_t i, const ParkedWalker<S> &pw,
                                           WalkerRun<S> &run)
{
    run.w.id = L.walker_begin + i;
    run.w.step = pw.step;
    run.w.data = pw.data;
    run.v = pw.v;
    run.pos = Pos{-1, 0};
    run.pv = kNone;
    run.ppos = Pos{-1, 0};
    const uint64_t pbase = L.path_off ? L.path_off[i] : (uint64_t)i * L.cap;
    run.cap = L.path_off ? (uint32_t)(L.path_off[i + 1] - pbase) : L.cap;
    run.out = L.path ? L.path + pbase : nullptr;
    run.len = pw.len;
    run.in_step = run.need_ext = run.ob_known = false;
    run.step_trials = 0;
    run.ob_c = 0.0f;
    run.on_c = 0;
    run.trials = run.queries = run.probes = 0;
}

/* Runs the warp's walkers (alive: lane holds walker i) to their ends, or,
 * with parking on, until fewer than L.park_below lanes are walking; then each
 * lane still walking finishes its step and parks (record under park_id),
 * once it has taken a step in this launch (so every launch moves every walker
 * it holds).  Every lane of the warp calls it with the same L.park and
 * L.park_below (the ballots take the full warp). */
template <typename S, typename WC, typename TC, typename Bucket>
__device__ __forceinline__ void walk_lanes(const GraphView &g, const WC &wc, const TC &tc, const Bucket *alias,
                                           const float *ra, const WalkLaunch &L, bool alive, uint32_t i,
                                           WalkerRun<S> &run, Sampler &rng, unsigned long long &my_steps,
                                           WalkCounts &counts, uint32_t park_id)
{
    /* between the warp's ballots each lane runs up to kParkCheck trials on
     * its own, so lanes in different phases of a step overlap their reads (a
     * ballot per trial forces the warp to reconverge every trial: 16.8 vs
     * 13.6 ms); a lane that may park stops at its step boundary.  Without
     * parking one pass runs every walk to its end. */
    const uint32_t check = L.park != nullptr ? kParkCheck : 0xffffffffu;
    bool parking = false;
    const step_t step0 = alive ? run.w.step : 0;
    for (;;)
    {
        const unsigned live = __ballot_sync(kFullMask, alive);
        if (live == 0)
            return;
        if (L.park != nullptr)
        {
            if ((unsigned)__popc(live) < L.park_below)
                parking = true;
            const bool stop = alive && parking && !run.in_step && run.w.step != step0;
            const unsigned stops = __ballot_sync(kFullMask, stop);
            if (stops != 0)
            {
                const unsigned lane = threadIdx.x & 31;
                uint32_t base = 0;
                if (lane == (unsigned)(__ffs(stops) - 1))
                    base = atomicAdd(L.park_count, (uint32_t)__popc(stops));
                base = __shfl_sync(kFullMask, base, __ffs(stops) - 1);
                if (stop)
                {
                    ParkedWalker<S> *q = (ParkedWalker<S> *)L.park;
                    q[base + __popc(stops & ((1u << lane) - 1u))] = ParkedWalker<S>{park_id, run.v, run.w.step,
                                                                                   run.len, run.w.data};
                    counts.add(run);
                    alive = false;
                }
            }
        }
        bool ended = false;
        for (uint32_t k = 0; alive && k < check; k++)
        {
            if (parking && !run.in_step && run.w.step != step0)
                break;
            if (!walk_trial<S>(g, wc, tc, alias, ra, L, run, rng))
            {
                ended = true;
                break;
            }
        }
        /* outside the divergent loop: walk_finish's segment count synchronises
         * lanes (inside it the walk took 25 instead of 19 ms) */
        if (ended)
        {
            walk_finish<S>(L, i, run, my_steps, counts);
            alive = false;
        }
    }
}

/* One thread per walker for its whole walk, walker state in registers. */
template <typename S, typename WC, typename TC, typename Bucket>
__global__ void __launch_bounds__(256, 4) walk_static_kernel(GraphView g, WC wc, TC tc, const Bucket *alias,
                                                          const float *ra, WalkLaunch L)
{
    unsigned long long my_steps = 0;
    WalkCounts counts;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_iter = (L.walker_num + stride - 1) / stride;
    for (uint32_t it = 0; it < n_iter; it++)
    {
        const uint32_t i = (it * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        if constexpr (parks<TC>())
        {
            /* every lane takes part in walk_lanes' ballots */
            const bool alive = i < L.walker_num;
            Sampler rng;
            WalkerRun<S> run;
            if (alive)
            {
                rng.init(L.seed);
                walk_begin<S>(g, wc, L, i, run, rng);
            }
            walk_lanes<S>(g, wc, tc, alias, ra, L, alive, i, run, rng, my_steps, counts, i);
        }
        else if (i < L.walker_num)
        {
            Sampler rng;
            rng.init(L.seed);
            WalkerRun<S> run;
            walk_begin<S>(g, wc, L, i, run, rng);
            while (walk_trial<S>(g, wc, tc, alias, ra, L, run, rng))
            {
            }
            walk_finish<S>(L, i, run, my_steps, counts);
        }
    }
    flush_steps(L.total_steps, my_steps);
    counts.flush(L.stats);
}

/* Resumes the walkers parked by the previous launch (*in_count of them),
 * 32 to a warp, parking again into L.park (or running them to their ends
 * when L.park is nullptr). */
template <typename S, typename WC, typename TC, typename Bucket>
__global__ void __launch_bounds__(256, 4) walk_resume_kernel(GraphView g, WC wc, TC tc, const Bucket *alias,
                                                          const float *ra, WalkLaunch L,
                                                          const ParkedWalker<S> *in, const uint32_t *in_count)
{
    unsigned long long my_steps = 0;
    WalkCounts counts;
    const uint32_t n = *in_count;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x)
    {
        const uint32_t k = b + threadIdx.x;
        const bool alive = k < n;
        uint32_t i = 0;
        Sampler rng;
        WalkerRun<S> run;
        if (alive)
        {
            const ParkedWalker<S> pw = in[k];
            i = pw.i;
            rng.init(L.seed);
            resume_run<S>(L, i, pw, run);
        }
        walk_lanes<S>(g, wc, tc, alias, ra, L, alive, i, run, rng, my_steps, counts, i);
    }
    flush_steps(L.total_steps, my_steps);
    counts.flush(L.stats);
}

/* Regrouping walkers by the vertex they stand on (option regroup_interval =
 * k > 0).  The walk runs in phases of k steps.  A phase takes its walkers in
 * the order of the previous phase's records sorted by vertex (in[perm[t]],
 * *in_count of them; the first phase starts walkers 0..n-1 in id order), runs
 * each to its first step boundary at or past k more steps, and records every
 * walker still walking in out (a ParkedWalker<S>: node2vec's previous vertex
 * is in its state) with its vertex as the next phase's sort key and its
 * record index as the sort value.  Lanes of a warp then start on the same or
 * nearby vertices, so their offset and first bucket reads share sectors.  The
 * stream is keyed by (walker, step), so the paths are those of one walk. */
template <typename S, typename WC, typename TC, typename Bucket>
__global__ void __launch_bounds__(256, 4) walk_regroup_kernel(GraphView g, WC wc, TC tc, const Bucket *alias,
                                                           const float *ra, WalkLaunch L,
                                                           const ParkedWalker<S> *in, const uint32_t *perm,
                                                           const uint32_t *in_count, ParkedWalker<S> *out,
                                                           uint32_t *out_keys, uint32_t *out_vals,
                                                           uint32_t *out_count, uint32_t k)
{
    unsigned long long my_steps = 0;
    WalkCounts counts;
    const uint32_t n = in != nullptr ? *in_count : L.walker_num;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x)
    {
        const uint32_t t = b + threadIdx.x;
        bool park = false, ended = false;
        uint32_t i = 0;
        Sampler rng;
        WalkerRun<S> run;
        if (t < n)
        {
            rng.init(L.seed);
            if (in != nullptr)
            {
                const ParkedWalker<S> pw = in[perm[t]];
                i = pw.i;
                resume_run<S>(L, i, pw, run);
            }
            else
            {
                i = t;
                walk_begin<S>(g, wc, L, i, run, rng);
            }
            const step_t end = run.w.step + k;
            for (;;)
            {
                if (!run.in_step && run.w.step >= end)
                {
                    park = true;
                    break;
                }
                if (!walk_trial<S>(g, wc, tc, alias, ra, L, run, rng))
                {
                    ended = true;
                    break;
                }
            }
        }
        if (ended)
            walk_finish<S>(L, i, run, my_steps, counts);
        const unsigned pm = __ballot_sync(kFullMask, park);
        if (pm != 0)
        {
            uint32_t base = 0;
            if (lane == (unsigned)(__ffs(pm) - 1))
                base = atomicAdd(out_count, (uint32_t)__popc(pm));
            base = __shfl_sync(kFullMask, base, __ffs(pm) - 1);
            if (park)
            {
                const uint32_t slot = base + __popc(pm & ((1u << lane) - 1u));
                out[slot] = ParkedWalker<S>{i, run.v, run.w.step, run.len, run.w.data};
                out_keys[slot] = run.v;
                out_vals[slot] = slot;
                counts.add(run);
            }
        }
    }
    flush_steps(L.total_steps, my_steps);
    counts.flush(L.stats);
}

/* Several walkers per thread for walks whose every trial is accepted (first
 * order without a dynamic component: DeepWalk, PPR).  A step is two dependent
 * gathers (the adjacency position, when the bucket did not carry it, then the
 * bucket); the thread runs its W walkers in lockstep phases so that the
 * gathers of all W are in flight together instead of one at a time.  Each
 * walker keeps its own stream and state, so the paths are those of
 * walk_static_kernel.  Thread t walks t, t + T, t + 2T, ... (T threads),
 * taking the next as soon as one of its walks ends. */
template <typename S, typename WC, typename TC, typename Bucket, int W>
__global__ void __launch_bounds__(256, 4) walk_multi_kernel(GraphView g, WC wc, TC tc, const Bucket *alias,
                                                            WalkLaunch L)
{
    static_assert(TC::order == 1 && !TC::has_dynamic, "every trial accepted");
    const uint32_t T = gridDim.x * blockDim.x;
    const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long my_steps = 0;
    WalkCounts counts;
    WalkerRun<S> run[W];
    Sampler rng[W];
    uint32_t idx[W];
    bool act[W];
    uint32_t next = t0;
#pragma unroll
    for (int k = 0; k < W; k++)
    {
        act[k] = next < L.walker_num;
        idx[k] = next;
        if (act[k])
        {
            rng[k].init(L.seed);
            walk_begin<S>(g, wc, L, next, run[k], rng[k]);
        }
        next += T;
    }
    for (;;)
    {
        bool any = false;
#pragma unroll
        for (int k = 0; k < W; k++)
            any |= act[k];
        if (!any)
            break;
        /* phase 1: adjacency positions not carried by a bucket */
        int64_t o0[W], o1[W];
#pragma unroll
        for (int k = 0; k < W; k++)
            if (act[k] && run[k].pos.e0 < 0)
            {
                o0[k] = gather(g.off + run[k].v);
                o1[k] = gather(g.off + run[k].v + 1);
            }
#pragma unroll
        for (int k = 0; k < W; k++)
            if (act[k] && run[k].pos.e0 < 0)
                run[k].pos = Pos{o0[k], (uint32_t)(o1[k] - o0[k])};
        /* phase 2: end tests, draws and the bucket (or neighbour) gathers */
        bool live[W];
        uint4 lo[W], hi[W];
        uint32_t c[W];
#pragma unroll
        for (int k = 0; k < W; k++)
        {
            live[k] = false;
            if (!act[k])
                continue;
            const Pos pos = run[k].pos;
            Walker<S> &w = run[k].w;
            bool ends = pos.deg == 0;
            if (!ends)
            {
                rng[k].enter(w.id, w.step, 0);
                const real_t ext = tc.extension_comp(w, run[k].v);
                ends = ext == 0.0f || (ext < 1.0f && rng[k].gen_float(1.0f) > ext);
            }
            if (ends)
            {
                L.length[idx[k]] = run[k].len;
                segment_done(L, idx[k]);
                my_steps += run[k].len - 1;
                counts.add(run[k]);
                act[k] = next < L.walker_num;
                idx[k] = next;
                if (act[k])
                {
                    rng[k].init(L.seed);
                    walk_begin<S>(g, wc, L, next, run[k], rng[k]);
                }
                next += T;
                continue;
            }
            live[k] = true;
            c[k] = rng[k].gen(pos.deg);
            if constexpr (TC::has_static)
            {
                const uint4 *b4 = reinterpret_cast<const uint4 *>(alias + pos.e0 + c[k]);
                lo[k] = gather(b4);
                if constexpr (!Bucket::compact)
                    hi[k] = gather(b4 + 1);
            }
            else
            {
                lo[k].y = gather(g.nbr + pos.e0 + c[k]);
            }
        }
        /* phase 3: the coin, the step, the path write */
#pragma unroll
        for (int k = 0; k < W; k++)
        {
            if (!live[k])
                continue;
            Cand ac;
            if constexpr (TC::has_static)
            {
                if constexpr (Bucket::compact)
                {
                    if (lo[k].z == kNone || rng[k].gen_float(1.0f) < __uint_as_float(lo[k].x))
                        ac = Cand{kNone, lo[k].y, 0, false, lo[k].w & 0xffffu};
                    else
                        ac = Cand{kNone, lo[k].z, 0, false, lo[k].w >> 16};
                }
                else if constexpr (Bucket::cursor)
                {
                    if (lo[k].z == kNone || rng[k].gen_float(1.0f) < __uint_as_float(lo[k].x))
                        ac = Cand{kNone, lo[k].y, ((uint64_t)hi[k].y << 32) | hi[k].x, true, 0};
                    else
                        ac = Cand{kNone, lo[k].z, ((uint64_t)hi[k].w << 32) | hi[k].z, true, 0};
                }
                else
                {
                    if (lo[k].z == kNone || rng[k].gen_float(1.0f) < __uint_as_float(lo[k].x))
                        ac = Cand{lo[k].y, hi[k].x, 0, false, hi[k].z};
                    else
                        ac = Cand{lo[k].z, hi[k].y, 0, false, hi[k].w};
                }
            }
            else
            {
                ac = Cand{c[k], lo[k].y, 0, false, 0};
            }
            WalkerRun<S> &r = run[k];
            const Pos pos = r.pos;
            const vertex_id_t v = r.v;
            r.trials++;
            r.w.step++;
            if constexpr (is_hook<decltype(wc.walker_update_state)>())
                wc.walker_update_state(r.w, v, AdjUnit{ac.nbr, (edge_id_t)(pos.e0 + ac.idx), ac.tag});
            bool over = false;
            if (r.out)
            {
                if (r.len >= r.cap)
                {
                    atomicOr(L.status, KK_STATUS_PATH_CAPACITY);
                    over = true;
                }
                else
                {
                    r.out[r.len] = ac.nbr;
                }
            }
            if (over)
            {
                L.length[idx[k]] = r.len;
                segment_done(L, idx[k]);
                my_steps += r.len - 1;
                counts.add(r);
                act[k] = false;
                continue;
            }
            r.len++;
            r.pv = v;
            r.ppos = pos;
            r.v = ac.nbr;
            r.pos = ac.has_cur ? pos_from_cursor(g, ac.nbr, ac.cur) : Pos{-1, 0};
        }
    }
    flush_steps(L.total_steps, my_steps);
    counts.flush(L.stats);
}

/* Device-resident walker pool: persistent blocks, each owning a contiguous
 * range of walker ids handed out by a shared-memory counter.  Every loop
 * iteration advances each lane's walker by one step; a lane whose walk ends
 * writes its length and takes the next walker at once, so lanes do not idle
 * on finished walks until the block's range runs dry.  Results are those of
 * walk_static_kernel: every walker's draws depend only on its id. */
template <typename S, typename WC, typename TC, typename Bucket>
__global__ void __launch_bounds__(256) walk_pool_kernel(GraphView g, WC wc, TC tc, const Bucket *alias,
                                                        const float *ra, WalkLaunch L)
{
    __shared__ uint32_t s_next;
    const uint32_t per = (uint32_t)(((uint64_t)L.walker_num + gridDim.x - 1) / gridDim.x);
    const uint32_t lo = (uint32_t)min((uint64_t)blockIdx.x * per, (uint64_t)L.walker_num);
    const uint32_t hi = (uint32_t)min((uint64_t)lo + per, (uint64_t)L.walker_num);
    if (threadIdx.x == 0)
        s_next = lo;
    __syncthreads();
    unsigned long long my_steps = 0;
    WalkCounts counts;
    Sampler rng;
    rng.init(L.seed);
    WalkerRun<S> run;
    uint32_t i = atomicAdd(&s_next, 1u);
    bool have = i < hi;
    if (have)
        walk_begin<S>(g, wc, L, i, run, rng);
    while (__any_sync(kFullMask, have))
    {
        if (have && !walk_trial<S>(g, wc, tc, alias, ra, L, run, rng))
        {
            L.length[i] = run.len;
            segment_done(L, i);
            my_steps += run.len - 1;
            counts.add(run);
            i = atomicAdd(&s_next, 1u);
            have = i < hi;
            if (have)
                walk_begin<S>(g, wc, L, i, run, rng);
        }
    }
    flush_steps(L.total_steps, my_steps);
    counts.flush(L.stats);
}

/* ---- batched walks --------------------------------------------------------
 * Many walk jobs of one app in one launch.  A job has its own seed, walker
 * range, length and app constants; its walkers get exactly the draws and
 * decisions of the job run alone, because every draw is keyed by the job's
 * seed and the walker's id and the job's hooks are rebuilt per walker. */

constexpr uint32_t kMaxBatchJobs = 1024;
/* resident blocks of 256 threads per SM the batch kernels are compiled for
 * (the register budget: 4 -> 64 registers a thread) */
#ifndef KK_BATCH_MINB
#define KK_BATCH_MINB 4
#endif

struct BatchJob
{
    uint64_t seed;
    uint64_t path_base;    /* first vertex slot of the job's paths */
    uint32_t walker_begin; /* first walker id */
    uint32_t walker_num;
    uint32_t first_task;   /* position of the job's first walker in the batch */
    uint32_t cap;          /* path capacity per walker, vertices */
    uint32_t walk_length;
    int32_t flag;          /* metapath: round-robin scheme assignment */
    float c[5];            /* node2vec: upperbound, lowerbound, overflow, 1/p, 1/q */
    /* the launch order: the walkers of the launch's k-th job (the jobs by
     * walk length, longest first) are the launch's walkers launch_first
     * onwards of entry k, and that job is entry launch_job of this table */
    uint32_t launch_first;
    const void *param;     /* metapath: the job's schemes (device) */
    uint32_t launch_job;
};

/* Per-job completion of a batch (serving): the walkers of job j count
 * themselves done on count[j], and the job's last walker writes flag[j] =
 * 1 + status[j] in mapped host memory, status[j] being the job's own status
 * word (its walkers' trial-limit and capacity failures), so the host hands
 * each request out as soon as it is walked, with its own outcome.
 * count == nullptr: the batch reports one status when it ends. */
struct BatchNotify
{
    uint32_t *count = nullptr;
    volatile uint32_t *flag = nullptr;
    int *status = nullptr;
};

/* Walker t of a batch: its job (binary search over the jobs' first positions
 * in shared memory), the job's hooks and launch record, the walker started. */
template <typename App>
__device__ __forceinline__ uint32_t batch_launch(const App &app, const BatchJob *jobs, const uint32_t *s_first,
                                                 uint32_t njobs, uint32_t t, const float *alias_sum, uint32_t *path,
                                                 uint32_t *length, unsigned long long *total_steps, int *status,
                                                 uint32_t trial_limit, typename App::WC &wc, typename App::TC &tc,
                                                 WalkLaunch &L, const BatchNotify &nt)
{
    /* s_first: the launch order's first walkers, then the table entry of
     * each (kMaxBatchJobs on) */
    uint32_t k = 0, hi = njobs;
    while (hi - k > 1)
    {
        const uint32_t mid = (k + hi) >> 1;
        if (s_first[mid] <= t)
            k = mid;
        else
            hi = mid;
    }
    const uint32_t lo = s_first[kMaxBatchJobs + k];
    const BatchJob job = jobs[lo];
    app.make(job, wc, tc);
    L.seed = job.seed;
    L.walker_begin = job.walker_begin;
    L.walker_num = job.walker_num;
    L.path_off = nullptr;
    L.cap = job.cap;
    L.path = path ? path + job.path_base : nullptr;
    L.length = length + job.first_task;
    L.start = nullptr;
    L.n_start = 0;
    L.total_steps = total_steps;
    L.alias_sum = alias_sum;
    L.status = status;
    L.trial_limit = trial_limit;
    L.stats = nullptr;
    if (nt.count != nullptr)
    {
        /* the job is one segment of its own */
        L.seg_count = nt.count + lo;
        L.seg_flag = nt.flag + lo;
        L.seg_shift = 31;
        L.status = nt.status + lo;
        L.seg_status = nt.status + lo;
    }
    return t - s_first[k];
}

/* Walker t of a batch started: its job, hooks and launch record, then its walk. */
template <typename S, typename App>
__device__ __forceinline__ uint32_t batch_walker_begin(const GraphView &g, const App &app, const BatchJob *jobs,
                                                       const uint32_t *s_first, uint32_t njobs, uint32_t t,
                                                       const float *alias_sum, uint32_t *path, uint32_t *length,
                                                       unsigned long long *total_steps, int *status,
                                                       uint32_t trial_limit, typename App::WC &wc,
                                                       typename App::TC &tc, WalkLaunch &L, WalkerRun<S> &run,
                                                       Sampler &rng, const BatchNotify &nt)
{
    const uint32_t i = batch_launch(app, jobs, s_first, njobs, t, alias_sum, path, length, total_steps, status,
                                    trial_limit, wc, tc, L, nt);
    rng.init(L.seed);
    walk_begin<S>(g, wc, L, i, run, rng);
    return i;
}

/* Parking of a batch launch (first-order rejection walks): the queue the
 * stragglers go to and the lane threshold; out == nullptr: none. */
struct BatchPark
{
    void *out = nullptr;
    uint32_t *count = nullptr;
    uint32_t below = 0;
};

/* One thread per walker over the concatenated walkers of all jobs.
 * App::make(job, wc, tc) builds the job's WalkerConfig / TransitionConfig. */
template <typename S, typename App, typename Bucket>
__global__ void __launch_bounds__(256, KK_BATCH_MINB) walk_batch_kernel(GraphView g, App app, const BatchJob *jobs, uint32_t njobs,
                                                         uint32_t total, const Bucket *alias,
                                                         const float *alias_sum, uint32_t *path, uint32_t *length,
                                                         unsigned long long *total_steps, int *status,
                                                         uint32_t trial_limit, unsigned long long *stats,
                                                         const uint32_t *hdr, BatchPark bp, BatchNotify nt)
{
    __shared__ uint32_t s_first[2 * kMaxBatchJobs];
    if (hdr != nullptr)
    {
        /* counts from device memory: one captured launch serves every batch */
        njobs = hdr[0];
        total = hdr[1];
    }
    for (uint32_t j = threadIdx.x; j < njobs; j += blockDim.x)
    {
        s_first[j] = jobs[j].launch_first;
        s_first[kMaxBatchJobs + j] = jobs[j].launch_job;
    }
    __syncthreads();
    unsigned long long my_steps = 0;
    WalkCounts counts;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_iter = (total + stride - 1) / stride;
    for (uint32_t it = 0; it < n_iter; it++)
    {
        const uint32_t t = (it * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        if constexpr (parks<typename App::TC>())
        {
            /* every lane takes part in walk_lanes' ballots, with the same
             * parking fields */
            typename App::WC wc;
            typename App::TC tc;
            WalkLaunch L;
            L.park = bp.out;
            L.park_count = bp.count;
            L.park_below = bp.below;
            WalkerRun<S> run;
            Sampler rng;
            const bool alive = t < total;
            uint32_t i = 0;
            if (alive)
                i = batch_walker_begin<S>(g, app, jobs, s_first, njobs, t, alias_sum, path, length, total_steps,
                                          status, trial_limit, wc, tc, L, run, rng, nt);
            L.stats = stats;
            walk_lanes<S>(g, wc, tc, alias, nullptr, L, alive, i, run, rng, my_steps, counts, t);
        }
        else if (t < total)
        {
            typename App::WC wc;
            typename App::TC tc;
            WalkLaunch L;
            WalkerRun<S> run;
            Sampler rng;
            const uint32_t i = batch_walker_begin<S>(g, app, jobs, s_first, njobs, t, alias_sum, path, length,
                                                     total_steps, status, trial_limit, wc, tc, L, run, rng, nt);
            L.stats = stats;
            while (walk_trial<S>(g, wc, tc, alias, nullptr, L, run, rng))
            {
            }
            L.length[i] = run.len;
            segment_done(L, i);
            my_steps += run.len - 1;
            counts.add(run);
        }
    }
    flush_steps(total_steps, my_steps);
    counts.flush(stats);
}

/* Resumes the batch walkers parked by the previous launch (*in_count of
 * them; a record holds the walker's position t in the batch), 32 to a warp,
 * parking again into bp (or running them to their ends when bp.out is
 * nullptr). */
template <typename S, typename App, typename Bucket>
__global__ void __launch_bounds__(256, 4) walk_batch_resume_kernel(GraphView g, App app, const BatchJob *jobs,
                                                                uint32_t njobs, const Bucket *alias,
                                                                const float *alias_sum, uint32_t *path,
                                                                uint32_t *length, unsigned long long *total_steps,
                                                                int *status, uint32_t trial_limit,
                                                                unsigned long long *stats,
                                                                const ParkedWalker<S> *in, const uint32_t *in_count,
                                                                BatchPark bp)
{
    __shared__ uint32_t s_first[2 * kMaxBatchJobs];
    for (uint32_t j = threadIdx.x; j < njobs; j += blockDim.x)
    {
        s_first[j] = jobs[j].launch_first;
        s_first[kMaxBatchJobs + j] = jobs[j].launch_job;
    }
    __syncthreads();
    unsigned long long my_steps = 0;
    WalkCounts counts;
    const uint32_t n = *in_count;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x)
    {
        const uint32_t k = b + threadIdx.x;
        typename App::WC wc;
        typename App::TC tc;
        WalkLaunch L;
        L.park = bp.out;
        L.park_count = bp.count;
        L.park_below = bp.below;
        WalkerRun<S> run;
        Sampler rng;
        const bool alive = k < n;
        uint32_t i = 0, t = 0;
        if (alive)
        {
            const ParkedWalker<S> pw = in[k];
            t = pw.i;
            i = batch_launch(app, jobs, s_first, njobs, t, alias_sum, path, length, total_steps, status, trial_limit,
                             wc, tc, L, BatchNotify{});
            rng.init(L.seed);
            resume_run<S>(L, i, pw, run);
        }
        L.stats = stats;
        walk_lanes<S>(g, wc, tc, alias, nullptr, L, alive, i, run, rng, my_steps, counts, t);
    }
    flush_steps(total_steps, my_steps);
    counts.flush(stats);
}

/* Walker pool over a batch: persistent blocks, each owning a contiguous range
 * of the concatenated walkers handed out by a shared-memory counter; a lane
 * whose walk ends takes the next walker (of whatever job) at once, so walks
 * with more rejection trials do not hold idle lanes.  Paths are those of
 * walk_batch_kernel: every walker's draws depend only on its job and id. */
template <typename S, typename App, typename Bucket>
__global__ void __launch_bounds__(256, 4) walk_batch_pool_kernel(GraphView g, App app, const BatchJob *jobs,
                                                              uint32_t njobs, uint32_t total, const Bucket *alias,
                                                              const float *alias_sum, uint32_t *path,
                                                              uint32_t *length, unsigned long long *total_steps,
                                                              int *status, uint32_t trial_limit,
                                                              unsigned long long *stats, const uint32_t *hdr,
                                                              BatchNotify nt)
{
    __shared__ uint32_t s_first[2 * kMaxBatchJobs];
    __shared__ uint32_t s_next;
    if (hdr != nullptr)
    {
        njobs = hdr[0];
        total = hdr[1];
    }
    for (uint32_t j = threadIdx.x; j < njobs; j += blockDim.x)
    {
        s_first[j] = jobs[j].launch_first;
        s_first[kMaxBatchJobs + j] = jobs[j].launch_job;
    }
    const uint32_t per = (uint32_t)(((uint64_t)total + gridDim.x - 1) / gridDim.x);
    const uint32_t lo = (uint32_t)min((uint64_t)blockIdx.x * per, (uint64_t)total);
    const uint32_t hi = (uint32_t)min((uint64_t)lo + per, (uint64_t)total);
    if (threadIdx.x == 0)
        s_next = lo;
    __syncthreads();
    unsigned long long my_steps = 0;
    WalkCounts counts;
    typename App::WC wc;
    typename App::TC tc;
    WalkLaunch L;
    WalkerRun<S> run;
    Sampler rng;
    uint32_t t = atomicAdd(&s_next, 1u), i = 0;
    bool have = t < hi;
    if (have)
        i = batch_walker_begin<S>(g, app, jobs, s_first, njobs, t, alias_sum, path, length, total_steps, status,
                                  trial_limit, wc, tc, L, run, rng, nt);
    L.stats = stats;
    while (__any_sync(kFullMask, have))
    {
        if (have && !walk_trial<S>(g, wc, tc, alias, nullptr, L, run, rng))
        {
            L.length[i] = run.len;
            segment_done(L, i);
            my_steps += run.len - 1;
            counts.add(run);
            t = atomicAdd(&s_next, 1u);
            have = t < hi;
            if (have)
                i = batch_walker_begin<S>(g, app, jobs, s_first, njobs, t, alias_sum, path, length, total_steps,
                                          status, trial_limit, wc, tc, L, run, rng, nt);
            L.stats = stats;
        }
    }
    flush_steps(total_steps, my_steps);
    counts.flush(stats);
}

/* Upper bound on each walker's path length when the extension is a constant
 * probability ext in (0,1) (PPR, src/apps/ppr.hpp:55-58): the walk cannot pass
 * the first step whose first draw (the extension draw, draw 0) says stop.
 * cap[i] = that step + 1 vertices; fails when no stop comes within max_steps.
 * A warp takes 32 walkers at a time: with check_starts, each lane first reads
 * its walker's start vertex (start list, or walker id mod V) and gives a
 * walker on an isolated or out-of-range start one vertex with no draws (its
 * walk ends there, or fails the call); the warp then tests 32 consecutive
 * steps of one live walker at a time and takes the first stop by ballot, so
 * geometric lengths leave no lane waiting on the longest walk of its warp. */
static __global__ void constant_extension_bound_kernel(GraphView g, bool check_starts, const uint32_t *start,
                                                       uint32_t n_start, uint64_t seed, walker_id_t walker_begin,
                                                       uint32_t walker_num, float ext, uint32_t max_steps,
                                                       uint64_t *cap_out, int *status)
{
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t base = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < walker_num;
         base += nwarps * 32)
    {
        const uint64_t mine = base + lane;
        bool live = mine < walker_num;
        if (live && check_starts)
        {
            const walker_id_t id = walker_begin + (uint32_t)mine;
            const uint32_t v = start != nullptr ? start[id % n_start] : (uint32_t)(id % g.V);
            live = v < g.V && g.off[v + 1] > g.off[v];
            if (!live)
                cap_out[mine] = 1;
        }
        uint32_t todo = __ballot_sync(kFullMask, live);
        while (todo != 0)
        {
            const uint32_t j = __ffs(todo) - 1;
            todo &= todo - 1;
            const walker_id_t id = walker_begin + (uint32_t)(base + j);
            uint32_t stop = max_steps;
            for (uint32_t s0 = 0; s0 < max_steps; s0 += 32)
            {
                const uint32_t s = s0 + lane;
                bool says_stop = false;
                if (s < max_steps)
                {
                    const uint4 b = philox4x32_10(make_uint4(id, s, 0, 0), k0, k1);
                    says_stop = map_gen_float(b.x, 1.0f) > ext;
                }
                const uint32_t m = __ballot_sync(kFullMask, says_stop);
                if (m != 0)
                {
                    stop = s0 + __ffs(m) - 1;
                    break;
                }
            }
            if (lane == 0)
            {
                if (stop == max_steps)
                    atomicOr(status, KK_STATUS_PATH_CAPACITY);
                cap_out[base + j] = (uint64_t)stop + 1;
            }
        }
    }
}

} // namespace kk
