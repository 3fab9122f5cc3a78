// lbs.cu -- load-balanced search and warp race-and-resolve on sm_103a.
//
// Load-balanced search (load_balanced_search.cu:123-192, example lbs.cu:18-31):
// given per-item work counts, scanned = exclusive prefix sum (int32), total =
// sum, and result[i] for every work slot i < total = the item owning it
// (upper_bound(scanned, i) - 1).  The reference runs it in ONE CTA whose threads
// each walk the scanned array from the start (quadratic in the item count);
// here:
//   1. scan: CTAs reduce tiles of 4096 counts (int64, warp shuffles), one CTA
//      scans the tile sums, CTAs rescan their tiles with the tile offset;
//   2. search: merge-path partition (the merge of slot keys 0..total-1 with the
//      scanned offsets, ties to the offsets) into equal diagonals of 4096; the
//      tiles' path endpoints are found by binary search in one pass (a thread
//      per endpoint), then each search CTA takes tiles in turn, stages their
//      offsets in shared memory, every thread merges 16 steps from its own
//      diagonal, and the CTA writes its run of owners contiguously.
//   The scan of the tile sums also checks the call (negative counts, int32
//   overflow, result capacity) on the device, so all kernels are queued at once
//   and the host waits once, at the end.
// race_and_resolve (race_and_resolve.cuh:13-25) is exposed as a warp-level
// kernel over an array of predicates for testing the device primitive.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>

namespace gu {

constexpr int LBS_THREADS = 512;
constexpr int LBS_ITEMS = 8;
constexpr int LBS_TILE = LBS_THREADS * LBS_ITEMS;  // counts per scan tile / diagonals per search tile
constexpr int LBS_STHREADS = 256;                  // search CTA: fewer threads, more CTAs resident per SM
constexpr int LBS_SITEMS = LBS_TILE / LBS_STHREADS;  // merge steps per search thread

__device__ __forceinline__ long long block_reduce_ll(long long x, long long *s_warp)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL_MASK, x, o);
    if (lane_id() == 0) s_warp[warp_in_block()] = x;
    __syncthreads();
    long long t = 0;
    if (warp_in_block() == 0) {
        t = lane_id() < (int)(blockDim.x >> 5) ? s_warp[lane_id()] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULL_MASK, t, o);
    }
    __syncthreads();
    return t;  // valid in warp 0
}

// exclusive scan of one value per thread across the CTA (warp shuffles)
__device__ __forceinline__ long long block_exscan_ll(long long x, long long *s_warp, long long *total)
{
    const int lane = lane_id(), wid = warp_in_block(), nw = blockDim.x >> 5;
    long long incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const long long t = lane < nw ? s_warp[lane] : 0;
        long long ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(FULL_MASK, ti, o);
            if (lane >= o) ti += y;
        }
        if (lane < nw) s_warp[lane] = ti - t;
        if (lane == 31) s_warp[32] = ti;
    }
    __syncthreads();
    const long long r = s_warp[wid] + incl - x;
    *total = s_warp[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(LBS_THREADS) lbs_tile_sums(const int32_t *__restrict__ counts, int32_t N,
                                                             long long *__restrict__ tile_sum, int *negative)
{
    __shared__ long long s_warp[33];
    const long long base = (long long)blockIdx.x * LBS_TILE;
    long long s = 0;
    bool neg = false;
#pragma unroll
    for (int t = 0; t < LBS_ITEMS; ++t) {
        const long long i = base + (long long)t * LBS_THREADS + threadIdx.x;
        if (i < N) {
            const int32_t c = counts[i];
            neg |= c < 0;
            s += c;
        }
    }
    if (__any_sync(FULL_MASK, neg) && lane_id() == 0) atomicOr(negative, 1);
    const long long tot = block_reduce_ll(s, s_warp);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// one CTA: exclusive scan of the tile sums in chunks of blockDim; last entry = total.
// It also decides on the device whether the search may run (no negative count,
// total within int32 and within the result capacity, a result buffer when the
// total is positive) -- the later kernels read the verdict, so the call needs no
// host round trip before them -- and writes the int32 total when it may.
__global__ void __launch_bounds__(LBS_THREADS) lbs_scan_tiles(long long *__restrict__ tile_sum, int32_t ntiles,
                                                              long long *__restrict__ total, const int *neg,
                                                              long long capacity, int has_result, int *ok,
                                                              int32_t *total_out)
{
    __shared__ long long s_warp[33];
    long long carry = 0;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const long long x = i < ntiles ? tile_sum[i] : 0;
        long long tot;
        const long long ex = block_exscan_ll(x, s_warp, &tot);
        if (i < ntiles) tile_sum[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        *total = carry;
        const bool good = *neg == 0 && carry <= INT32_MAX && carry <= capacity && (carry == 0 || has_result);
        *ok = good ? 1 : 0;
        if (good && total_out) *total_out = (int32_t)carry;
    }
}

// rescan each tile with its offset; counts are read in blocked order (thread t
// owns LBS_ITEMS consecutive counts) so the scan order is the array order
__global__ void __launch_bounds__(LBS_THREADS) lbs_scan_write(const int32_t *__restrict__ counts, int32_t N,
                                                              const long long *__restrict__ tile_off,
                                                              int32_t *__restrict__ scanned)
{
    __shared__ long long s_warp[33];
    const long long base = (long long)blockIdx.x * LBS_TILE + (long long)threadIdx.x * LBS_ITEMS;
    int32_t v[LBS_ITEMS];
    long long s = 0;
#pragma unroll
    for (int t = 0; t < LBS_ITEMS; ++t) {
        v[t] = base + t < N ? counts[base + t] : 0;
        s += v[t];
    }
    long long tot;
    long long run = tile_off[blockIdx.x] + block_exscan_ll(s, s_warp, &tot);
#pragma unroll
    for (int t = 0; t < LBS_ITEMS; ++t) {
        if (base + t < N) scanned[base + t] = (int32_t)run;
        run += v[t];
    }
}

// Merge-path split of diagonal d between slot keys A[i] = i (i < total) and
// offsets B[k] = scanned[k] (k < N), ties to B: returns the number of offsets
// among the first d merged elements.
__device__ __forceinline__ int32_t merge_path(const int32_t *B, int32_t N, long long total, long long d)
{
    long long lo = d > total ? d - total : 0;
    long long hi = d < N ? d : N;
    while (lo < hi) {
        const long long k = (lo + hi) >> 1;  // candidate: k offsets consumed
        // B[k] belongs before A[d-k-1]  <=>  B[k] <= d-k-1
        if ((long long)B[k] <= d - k - 1) lo = k + 1;
        else hi = k;
    }
    return (int32_t)lo;
}

// Path endpoints of every search tile, all in parallel: one thread per tile
// boundary d = t * LBS_TILE (the last one at total + N).  Done inside each
// search CTA, the 20-odd dependent global loads of the binary search were most
// of the kernel's time.
__global__ void lbs_partition(const int32_t *__restrict__ scanned, int32_t N, const long long *total_p,
                              const int *ok, int32_t *__restrict__ kpart)
{
    if (!*ok) return;
    const long long total = *total_p;
    if (total == 0) return;
    const long long ntile = (total + N + LBS_TILE - 1) / LBS_TILE;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t <= ntile;
         t += (long long)gridDim.x * blockDim.x)
        kpart[t] = merge_path(scanned, N, total, min(t * LBS_TILE, total + N));
}

__global__ void __launch_bounds__(LBS_STHREADS) lbs_search(const int32_t *__restrict__ scanned, int32_t N,
                                                           const long long *total_p, const int *ok,
                                                           const int32_t *__restrict__ kpart,
                                                           int32_t *__restrict__ result)
{
    __shared__ int32_t s_b[LBS_TILE + 1];
    // owners by slot, one padding word per 32: thread t writes slots 16t.. (a stride of
    // 16 words across the warp), which unpadded would hit 2 banks
    __shared__ int32_t s_out[LBS_TILE + LBS_TILE / 32];
    if (!*ok) return;
    const long long total = *total_p;
    if (total == 0) return;  // no slots; the path endpoints were not written
    const long long ntile = (total + N + LBS_TILE - 1) / LBS_TILE;
    for (long long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {  // block-uniform
        const long long d0 = tile * LBS_TILE;
        const long long d1 = min(d0 + LBS_TILE, total + N);
        const int32_t k0 = __ldg(kpart + tile), k1 = __ldg(kpart + tile + 1);
        const long long i0 = d0 - k0, i1 = d1 - k1;  // slots [i0, i1) of this tile
        const int nb = k1 - k0;
        for (int t = threadIdx.x; t < nb; t += blockDim.x) s_b[t] = scanned[k0 + t];
        __syncthreads();
        // this thread's diagonal, then LBS_SITEMS merge steps
        const long long dt = min(d0 + (long long)threadIdx.x * LBS_SITEMS, d1) - d0;
        long long lo = dt > (i1 - i0) ? dt - (i1 - i0) : 0, hi = dt < nb ? dt : nb;
        while (lo < hi) {
            const long long k = (lo + hi) >> 1;
            if ((long long)s_b[k] <= i0 + (dt - k) - 1) lo = k + 1;
            else hi = k;
        }
        int kk = (int)lo;
        long long ii = i0 + (dt - lo);
        for (int step = 0; step < LBS_SITEMS && (ii - i0) + kk < (i1 - i0) + nb; ++step) {
            const bool take_slot = kk >= nb || ii < (long long)s_b[kk];
            if (take_slot) {
                if (ii >= i1) break;
                const int o = (int)(ii - i0);
                s_out[o + (o >> 5)] = k0 + kk - 1;
                ++ii;
            } else {
                ++kk;
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < (int)(i1 - i0); i += blockDim.x) result[i0 + i] = s_out[i + (i >> 5)];
        __syncthreads();  // s_b and s_out are reused by the next tile
    }
}

// Winner lane per warp of 32 predicates (race_and_resolve_warp).
__global__ void race_and_resolve_kernel(const int32_t *__restrict__ pred, int32_t nwarps, int32_t *__restrict__ winner)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((i >> 5) >= nwarps) return;  // whole warps only (blockDim is a multiple of 32)
    winner[i] = race_and_resolve_warp(pred[i] != 0);
}

// Scan tile sums and flags, then the search tiles' path endpoints (as many as a
// total of result_capacity slots can need).
size_t lbs_scratch_bytes(int32_t N, int64_t result_capacity)
{
    const long long n = N > 0 ? N : 0;
    const size_t ntiles = (size_t)((n + LBS_TILE - 1) / LBS_TILE);
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    const size_t nsearch = (size_t)((cap + n + LBS_TILE - 1) / LBS_TILE);
    return (ntiles + 2) * sizeof(long long) + 256 + (nsearch + 2) * sizeof(int32_t);
}

void launch_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result, int64_t result_capacity,
                int32_t *total_dev, int64_t *total_host, void *scratch_ptr, size_t scratch_bytes, cudaStream_t st)
{
    if (N < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "N must be >= 0");
    if (N > 0 && (!counts || !scanned)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null counts or scanned");
    const int32_t ntiles = (int32_t)(((long long)N + LBS_TILE - 1) / LBS_TILE);
    if (scratch_bytes < lbs_scratch_bytes(N, result_capacity)) throw gu_error(GU_ERR_INTERNAL, "lbs scratch too small");
    long long *tile = reinterpret_cast<long long *>(scratch_ptr);
    long long *tot_d = tile + ntiles;
    int *neg_d = reinterpret_cast<int *>(tot_d + 1);
    int *ok_d = neg_d + 1;
    int32_t *kpart = reinterpret_cast<int32_t *>(reinterpret_cast<char *>(tile) + (ntiles + 2) * sizeof(long long) + 256);
    // every kernel is queued at once; the scan-of-tile-sums kernel decides whether
    // the search may run, and the host checks the same conditions after one wait
    long long tot = 0;
    int neg = 0;
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    if (N > 0) {
        GU_CUDA_CHECK(cudaMemsetAsync(neg_d, 0, sizeof(int), st));
        lbs_tile_sums<<<ntiles, LBS_THREADS, 0, st>>>(counts, N, tile, neg_d);
        lbs_scan_tiles<<<1, LBS_THREADS, 0, st>>>(tile, ntiles, tot_d, neg_d, result_capacity, result ? 1 : 0, ok_d,
                                                  total_dev);
        lbs_scan_write<<<ntiles, LBS_THREADS, 0, st>>>(counts, N, tile, scanned);
        // grids sized by the capacity bound, capped; both loop over the tiles the total needs
        const long long nsearch_max = (cap + N + LBS_TILE - 1) / LBS_TILE;
        const int gpart = (int)std::min<long long>((nsearch_max + 1 + 255) / 256, 1024);
        const int gsearch = (int)std::min<long long>(std::max<long long>(nsearch_max, 1), 4096);
        lbs_partition<<<gpart, 256, 0, st>>>(scanned, N, tot_d, ok_d, kpart);
        lbs_search<<<gsearch, LBS_STHREADS, 0, st>>>(scanned, N, tot_d, ok_d, kpart, result);
        GU_CUDA_CHECK(cudaGetLastError());
        GU_CUDA_CHECK(cudaMemcpyAsync(&tot, tot_d, sizeof(long long), cudaMemcpyDeviceToHost, st));
        GU_CUDA_CHECK(cudaMemcpyAsync(&neg, neg_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    } else if (total_dev) {
        GU_CUDA_CHECK(cudaMemsetAsync(total_dev, 0, sizeof(int32_t), st));
    }
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    if (total_host) *total_host = tot;
    if (neg) throw gu_error(GU_ERR_INVALID_ARGUMENT, "work counts must be >= 0");
    if (tot > INT32_MAX) throw gu_error(GU_ERR_OVERFLOW, "total work exceeds INT32_MAX (int32 scanned offsets)");
    if (tot > result_capacity)
        throw gu_error(GU_ERR_CAPACITY, "result buffer holds " + std::to_string(result_capacity) + " slots, need " +
                                            std::to_string(tot));
    if (tot > 0 && !result) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null result");
}

void launch_race_and_resolve(const int32_t *pred, int32_t nwarps, int32_t *winner, cudaStream_t st)
{
    if (nwarps <= 0) return;
    const long long threads = (long long)nwarps * 32;
    race_and_resolve_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(pred, nwarps, winner);
    GU_CUDA_CHECK(cudaGetLastError());
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
}

}  // namespace gu
