// plain.cu -- the one-launch-per-request BFS form, kept as the measured baseline
// and as the PLAIN variant.
//
// It keeps the reference's structure (one CTA per source, the int32 distance
// row itself as the visited set claimed with atomicCAS, level queues in global
// memory, a CTA barrier per level; multi_search/shuffle_based.cuh:81-286 with
// the atomicCAS visit of multi_search/linear_with_atomics.cu:130) written with
// sm_103a warp intrinsics: warp per frontier vertex with a dynamic warp queue,
// warp-aggregated queue appends.  No batching, no bitmaps, no bottom-up.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <climits>

namespace gu {

constexpr int PLAIN_THREADS = 512;

__global__ void __launch_bounds__(PLAIN_THREADS) plain_bfs_kernel(const int32_t *__restrict__ R,
                                                                  const int32_t *__restrict__ C, int32_t n,
                                                                  const int32_t *__restrict__ sources, int32_t k,
                                                                  int32_t *dist, int64_t ld, int32_t *qbuf)
{
    __shared__ int s_qlen, s_q2len, s_next;
    int32_t *Q = qbuf + (int64_t)blockIdx.x * 2 * n;
    int32_t *Q2 = Q + n;
    const int lane = lane_id();
    const int nwarps = blockDim.x >> 5;
    for (int si = blockIdx.x; si < k; si += gridDim.x) {
        int32_t *d = dist + (int64_t)si * ld;
        const int32_t src = __ldg(sources + si);
        for (int32_t v = threadIdx.x; v < n; v += blockDim.x) d[v] = (v == src) ? 0 : INT_MAX;
        if (threadIdx.x == 0) {
            Q[0] = src;
            s_qlen = 1;
            s_q2len = 0;
        }
        __syncthreads();
        for (int32_t level = 0; s_qlen > 0; ++level) {
            if (threadIdx.x == 0) s_next = nwarps;
            __syncthreads();
            const int qlen = s_qlen;
            int kq = warp_in_block();
            while (kq < qlen) {
                const int32_t v = Q[kq];
                const int32_t e1 = __ldg(R + v + 1);
                for (int32_t e = __ldg(R + v) + lane; e < e1; e += 32) {
                    const int32_t w = __ldg(C + e);
                    if (atomicCAS(&d[w], INT_MAX, level + 1) == INT_MAX) {
                        const unsigned mask = __activemask();
                        const int leader = __ffs(mask) - 1;
                        int base = 0;
                        if (lane == leader) base = atomicAdd(&s_q2len, __popc(mask));
                        base = __shfl_sync(mask, base, leader);
                        Q2[base + __popc(mask & ((1u << lane) - 1u))] = w;
                    }
                }
                int nk = 0;
                if (lane == 0) nk = atomicAdd(&s_next, 1);
                kq = __shfl_sync(FULL_MASK, nk, 0);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                s_qlen = s_q2len;
                s_q2len = 0;
            }
            int32_t *t = Q;
            Q = Q2;
            Q2 = t;
            __syncthreads();
        }
        // the queues of this CTA are reused by its next source
        Q = qbuf + (int64_t)blockIdx.x * 2 * n;
        Q2 = Q + n;
        __syncthreads();
    }
}

void launch_plain_bfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                      cudaStream_t stream)
{
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, plain_bfs_kernel, PLAIN_THREADS, 0));
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    int grid = g.sm_count * blocks_per_sm;
    if (grid > k) grid = k;
    if (grid < 1) grid = 1;
    const size_t need = (size_t)grid * 2 * (size_t)g.n * sizeof(int32_t) + WS_CONTROL_BYTES;
    char *ws = (char *)g.ws.get(need);
    int32_t *qbuf = reinterpret_cast<int32_t *>(ws + WS_CONTROL_BYTES);
    // no level statistics or timeline for this form
    GU_CUDA_CHECK(cudaMemsetAsync(ws, 0, WS_CONTROL_BYTES, stream));
    g.mark_start(stream);
    plain_bfs_kernel<<<grid, PLAIN_THREADS, 0, stream>>>(g.R, g.C, g.n, sources, k, dist, ld, qbuf);
    GU_CUDA_CHECK(cudaGetLastError());
    g.mark_stop(stream);
}

}  // namespace gu
