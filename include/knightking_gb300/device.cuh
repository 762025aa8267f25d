/*
 * knightking_gb300 device core: graph view, walker, random stream.
 *
 * Types follow include/type.hpp:30-37 of the reference (32-bit vertex, walker
 * and step ids, 64-bit edge ids, float arithmetic).  The graph lives in HBM as
 * a structure of arrays: int64 off[V+1], uint32 nbr[E], float w[E] (optional),
 * uint8 type[E] (optional).
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace kk
{

typedef uint32_t vertex_id_t;
typedef uint64_t edge_id_t;
typedef uint32_t walker_id_t;
typedef uint32_t step_t;
typedef float real_t;

constexpr uint32_t kNone = 0xffffffffu;

/* Device view of the CSR (include/graph.hpp:49-96 replaced by SoA arrays). */
struct GraphView
{
    uint32_t V;
    uint64_t E;
    const int64_t *off;
    const uint32_t *nbr;
    const float *w;
    const uint8_t *type;
    /* cursor adjacency (optional): per edge {neighbour, 0, the neighbour's
     * vertex cursor}, so a uniform pick yields the next vertex and where its
     * adjacency lies in one 16 B read */
    const uint4 *adjc = nullptr;
};

/* An edge as the hooks see it (AdjUnit, include/graph.hpp:49-61): its
 * neighbour and its global index, through which a hook reads edge data. */
struct AdjUnit
{
    vertex_id_t neighbour;
    edge_id_t index;
    /* the edge's type when the engine already holds it (bit 8 set, type in
     * bits 0-7; an alias bucket carries its candidates' types), else 0 */
    uint32_t type_tag = 0;
};

/* A vertex's adjacency (AdjList, include/graph.hpp:63-73) as an index range. */
struct AdjList
{
    edge_id_t begin;
    edge_id_t end;
    __host__ __device__ uint32_t degree() const { return (uint32_t)(end - begin); }
};

struct EmptyData
{
};

/* Walker<S> (include/walk.hpp:31-50). */
template <typename S>
struct Walker
{
    walker_id_t id;
    step_t step;
    S data;
};

/* "No hook": the nullptr of the reference's std::function members. */
struct NoHook
{
};

template <typename T>
constexpr bool is_hook()
{
    return !std::is_same<T, NoHook>::value;
}

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------------------- */

__host__ __device__ inline uint32_t mulhi32(uint32_t a, uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ inline uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++)
    {
        if (r != 0)
        {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

/* Draw mappings replacing include/util.hpp:60-69:
 *   gen(ub)       = high 32 bits of word * ub                  in [0, ub)
 *   gen_float(ub) = ((word >> 8) * 2^-24) * ub, one rounding    in [0, ub) */
__device__ __forceinline__ uint32_t map_gen(uint32_t word, uint32_t ub)
{
    return __umulhi(word, ub);
}

__device__ __forceinline__ float map_gen_float(uint32_t word, float ub)
{
    float u = __uint2float_rn(word >> 8) * 5.9604644775390625e-8f; /* exact */
    return __fmul_rn(u, ub);
}

/* Per-walker cursor into the stream: counter = (walker, step, draw >> 2,
 * stream), word draw & 3.  draw counts the draws of one (walker, step) in
 * program order, across all rejection trials of that step. */
struct Sampler
{
    uint32_t k0, k1;
    uint32_t walker, step, stream, draw;
    uint4 buf;

    __device__ __forceinline__ void init(uint64_t seed)
    {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
    }

    __device__ __forceinline__ void enter(walker_id_t w, step_t s, uint32_t st)
    {
        walker = w;
        step = s;
        stream = st;
        draw = 0;
    }

    __device__ __forceinline__ uint32_t word()
    {
        uint32_t slot = draw & 3u;
        if (slot == 0)
        {
            buf = philox4x32_10(make_uint4(walker, step, draw >> 2, stream), k0, k1);
        }
        draw++;
        return slot == 0 ? buf.x : (slot == 1 ? buf.y : (slot == 2 ? buf.z : buf.w));
    }

    __device__ __forceinline__ uint32_t gen(uint32_t ub) { return map_gen(word(), ub); }
    __device__ __forceinline__ float gen_float(float ub) { return map_gen_float(word(), ub); }
};

/* float helpers with one rounding each and no contraction */
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float u2f(uint32_t a) { return __uint2float_rn(a); }

/* Random gathers of the walk (read-only data path). */
__device__ __forceinline__ uint32_t gather(const uint32_t *p) { return __ldg(p); }
__device__ __forceinline__ float gather(const float *p) { return __ldg(p); }
__device__ __forceinline__ uint8_t gather(const uint8_t *p) { return __ldg(p); }
__device__ __forceinline__ uint4 gather(const uint4 *p) { return __ldg(p); }
__device__ __forceinline__ int64_t gather(const int64_t *p)
{
    return (int64_t)__ldg(reinterpret_cast<const long long *>(p));
}
__device__ __forceinline__ uint64_t gather(const uint64_t *p)
{
    return (uint64_t)__ldg(reinterpret_cast<const unsigned long long *>(p));
}

} // namespace kk
