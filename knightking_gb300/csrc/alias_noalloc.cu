/*
 * kk_alias_build_noalloc: the alias-table build with no device allocation.
 *
 * Some callers cannot call cudaMalloc: a serving process that has handed all
 * device memory to its own pool, or code on a latency-critical path where an
 * allocation (and the device synchronisation cudaFree implies) is not
 * allowed.  This entry point builds the same alias tables as kk_alias_build
 * (include/walk.hpp:538-652 of the reference, index for index and bit for bit)
 * from device arrays the caller owns, into device arrays the caller owns, and
 * allocates nothing.
 *
 * Its queue scratch is the file-scope array g_alias_noalloc_scratch below:
 * 32 MiB plus a 256-byte status header, which every GPU that loads this
 * library keeps until the process exits.  Vertices of degree up to
 * kNoAllocQueue keep their queues in shared memory; vertices of degree up to
 * kNoAllocMaxDegree use one of kNoAllocSlots slices of the array; a graph with
 * a larger degree is rejected.
 */
#include <cuda_runtime.h>

#include <mutex>

#include "knightking_gb300.h"
#include "knightking_gb300/walk.cuh"

namespace
{
using namespace kk;

constexpr uint32_t kNoAllocMaxDegree = 16384; /* largest vertex degree accepted */
constexpr uint32_t kNoAllocSlots = 128;       /* warps that take vertices above kNoAllocQueue */
constexpr uint32_t kNoAllocQueue = 512;       /* shared-memory queue entries per warp */
constexpr uint32_t kNoAllocHeader = 32;       /* uint2 entries (256 B) of status words */
constexpr size_t kNoAllocSmem = (size_t)8 * 2 * kNoAllocQueue * sizeof(uint2);

/* The shared scratch: status header, then per slot a p and a q queue of
 * kNoAllocMaxDegree (index, prob) entries.  Host code never names it as a
 * device address; it uses the pointer from cudaGetSymbolAddress. */
static __device__ __align__(256) uint2 g_alias_noalloc_scratch[kNoAllocHeader + (size_t)kNoAllocSlots * 2 *
                                                                                   kNoAllocMaxDegree];

__global__ void noalloc_check_kernel(const int64_t *off, uint32_t V, unsigned int *too_large)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if ((uint64_t)(off[v + 1] - off[v]) > kNoAllocMaxDegree)
            atomicExch(too_large, 1u);
}

/* A warp per vertex: the serial sum, the stable p/q split and the batched
 * FIFO pairing of walk.cuh's alias build, writing the tables as three arrays.
 * large == 0: vertices of degree <= kNoAllocQueue, queues in shared memory;
 * large == 1: the others, queues in the warp's slice of the scratch (one
 * slice per warp: the grid has exactly kNoAllocSlots warps). */
__global__ void __launch_bounds__(256) noalloc_alias_kernel(const int64_t *off, const float *w, uint32_t V, float *p_out,
                                                            uint32_t *pi_out, uint32_t *qi_out, float *sum_out,
                                                            uint2 *scratch, int large)
{
    extern __shared__ uint2 dyn[];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t gwarp = blockIdx.x * (blockDim.x >> 5) + wib;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    uint2 *P0, *Q0;
    uint32_t cap;
    if (large)
    {
        P0 = scratch + kNoAllocHeader + (size_t)gwarp * 2 * kNoAllocMaxDegree;
        Q0 = P0 + kNoAllocMaxDegree;
        cap = kNoAllocMaxDegree;
    }
    else
    {
        P0 = dyn + (size_t)wib * 2 * kNoAllocQueue;
        Q0 = P0 + kNoAllocQueue;
        cap = kNoAllocQueue;
    }
    for (uint32_t v = gwarp; v < V; v += nwarps)
    {
        const int64_t e0 = off[v];
        const uint32_t deg = (uint32_t)(off[v + 1] - e0);
        if (deg == 0 || deg > cap || (large && deg <= kNoAllocQueue))
            continue;
        float sum = 0.0f;
        for (uint32_t base = 0; base < deg; base += 32)
        {
            const float x = base + lane < deg ? w[e0 + base + lane] : 0.0f;
#pragma unroll
            for (uint32_t j = 0; j < 32; j++)
            {
                const float y = __shfl_sync(kFullMask, x, j);
                if (base + j < deg)
                    sum = fadd(sum, y);
            }
        }
        if (lane == 0 && sum_out != nullptr)
            sum_out[v] = sum;
        const float ave = fdiv(sum, u2f(deg));
        uint32_t pt = 0, qt = 0;
        for (uint32_t base = 0; base < deg; base += 32)
        {
            const bool valid = base + lane < deg;
            const float x = valid ? w[e0 + base + lane] : 0.0f;
            const bool sm = valid && x < ave, bg = valid && !(x < ave);
            const uint32_t mp = __ballot_sync(kFullMask, sm), mq = __ballot_sync(kFullMask, bg);
            const uint2 ent = make_uint2(base + lane, __float_as_uint(x));
            if (sm)
                P0[pt + __popc(mp & lt)] = ent;
            if (bg)
                Q0[qt + __popc(mq & lt)] = ent;
            pt += __popc(mp);
            qt += __popc(mq);
        }
        __syncwarp();
        uint32_t ph = 0, qh = 0;
        while (ph < pt)
        {
            const uint32_t lp = pt - ph, lq = qt - qh;
            if (lq == 0)
            {
                for (uint32_t i = lane; i < lp; i += 32)
                {
                    p_out[e0 + ph + i] = 1.0f;
                    pi_out[e0 + ph + i] = P0[ph + i].x;
                    qi_out[e0 + ph + i] = kNone;
                }
                ph = pt;
                break;
            }
            const uint32_t b = min(min(lp, lq), 32u);
            const bool act = lane < b;
            bool conv = false;
            uint2 ne = make_uint2(0, 0);
            if (act)
            {
                const uint2 pe = P0[ph + lane], qe = Q0[qh + lane];
                const float pv = __uint_as_float(pe.y), qv = __uint_as_float(qe.y);
                p_out[e0 + ph + lane] = fdiv(pv, ave);
                pi_out[e0 + ph + lane] = pe.x;
                qi_out[e0 + ph + lane] = qe.x;
                const float r = fsub(qv, fsub(ave, pv));
                conv = r < ave;
                ne = make_uint2(qe.x, __float_as_uint(r));
            }
            const uint32_t mc = __ballot_sync(kFullMask, act && conv), ms = __ballot_sync(kFullMask, act && !conv);
            if (act)
            {
                if (conv)
                    P0[pt + __popc(mc & lt)] = ne;
                else
                    Q0[qt + __popc(ms & lt)] = ne;
            }
            __syncwarp();
            ph += b;
            qh += b;
            pt += __popc(mc);
            qt += __popc(ms);
        }
        for (uint32_t i = lane; i < qt - qh; i += 32)
        {
            p_out[e0 + pt + i] = 1.0f;
            pi_out[e0 + pt + i] = Q0[qh + i].x;
            qi_out[e0 + pt + i] = kNone;
        }
        __syncwarp();
    }
}

std::mutex g_setup_lock;
uint2 *g_scratch_ptr[128] = {};
/* cudaFuncSetAttribute applies to the current device only, so the shared-memory
 * opt-in is recorded per device like the scratch address */
bool g_smem_attr_set[128] = {};

} // namespace

extern "C" kk_status kk_alias_build_noalloc(uint32_t v_num, const int64_t *d_off, const float *d_w, float *d_p,
                                            uint32_t *d_p_idx, uint32_t *d_q_idx, float *d_sum, void *stream)
{
    if (v_num == 0 || d_off == nullptr || d_w == nullptr || d_p == nullptr || d_p_idx == nullptr ||
        d_q_idx == nullptr)
        return KK_ERR_INVALID_CONFIG;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128)
        return KK_ERR_CUDA;
    uint2 *scratch = nullptr;
    int sms = 0;
    {
        /* once per device, with that device current: the array's device address */
        std::lock_guard<std::mutex> g(g_setup_lock);
        if (g_scratch_ptr[dev] == nullptr)
        {
            if (cudaGetSymbolAddress((void **)&g_scratch_ptr[dev], g_alias_noalloc_scratch) != cudaSuccess)
            {
                g_scratch_ptr[dev] = nullptr;
                return KK_ERR_CUDA;
            }
        }
        if (!g_smem_attr_set[dev])
        {
            if (cudaFuncSetAttribute(noalloc_alias_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kNoAllocSmem) != cudaSuccess)
                return KK_ERR_CUDA;
            g_smem_attr_set[dev] = true;
        }
        scratch = g_scratch_ptr[dev];
    }
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return KK_ERR_CUDA;
    /* the status word keeps the last call's value: clear it */
    unsigned int *too_large = (unsigned int *)scratch;
    if (cudaMemsetAsync(too_large, 0, kNoAllocHeader * sizeof(uint2), st) != cudaSuccess)
        return KK_ERR_CUDA;
    unsigned int blocks = (v_num + 255) / 256 < 8u * sms ? (v_num + 255) / 256 : 8u * sms;
    noalloc_check_kernel<<<blocks, 256, 0, st>>>(d_off, v_num, too_large);
    unsigned int h_too_large = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&h_too_large, too_large, sizeof(h_too_large), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return KK_ERR_CUDA;
    if (h_too_large)
        return KK_ERR_INVALID_CONFIG; /* a vertex degree exceeds kNoAllocMaxDegree (16384) */
    unsigned int warp_blocks = (v_num + 7) / 8 < 3u * sms ? (v_num + 7) / 8 : 3u * sms;
    noalloc_alias_kernel<<<warp_blocks, 256, kNoAllocSmem, st>>>(d_off, d_w, v_num, d_p, d_p_idx, d_q_idx, d_sum,
                                                                 scratch, 0);
    /* the large-degree pass keeps its queues in the scratch slices: no shared memory */
    noalloc_alias_kernel<<<kNoAllocSlots / 8, 256, 0, st>>>(d_off, d_w, v_num, d_p, d_p_idx, d_q_idx, d_sum, scratch,
                                                            1);
    if (cudaGetLastError() != cudaSuccess)
        return KK_ERR_CUDA;
    return KK_OK;
}
