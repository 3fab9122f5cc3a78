// lbs.cu -- load-balanced search and warp race-and-resolve on sm_103a.
//
// Load-balanced search (load_balanced_search.cu:123-192, example lbs.cu:18-31):
// given per-item work counts, scanned = exclusive prefix sum (int32), total =
// sum, and result[i] for every work slot i < total = the item owning it
// (upper_bound(scanned, i) - 1).  The reference runs it in ONE CTA whose threads
// each walk the scanned array from the start (quadratic in the item count);
// here three kernels:
//   1. lbs_tile_sums: the sum of every tile of 8192 counts (and a flag for a
//      negative count).
//   2. lbs_scan_apply: each tile adds the sums of the tiles before it (all final,
//      so no tile waits on another), scans its counts again from L2, writes its
//      part of scanned and the merge-path endpoints of the search tiles whose
//      first diagonal lies in its own stretch of the merge; the tile holding the
//      last counts knows the total and decides whether the call may write
//      results (no negative count, total within int32 and within the result
//      capacity, a result buffer when the total is positive).  A single-pass
//      scan with decoupled look-back took longer: with 512 tiles in flight a
//      published tile sum reached the tiles polling for it only microseconds
//      later, however the polling was arranged.
//   3. lbs_search: persistent CTAs (eight per SM) take search tiles of 4092
//      diagonals; the items a tile consumes mark their first slots in shared
//      memory and a block-wide running maximum turns the marks into owners,
//      written 16 bytes at a time.  A CTA loads its next tile's path endpoints
//      and first offsets before working on the current tile.
//   Kernels 2 and 3 are launched as programmatic dependents of their
//   predecessor, so that their launch overlaps its tail; the host waits once,
//   at the end.
// race_and_resolve (race_and_resolve.cuh:13-25) is exposed as a warp-level
// kernel over an array of predicates for testing the device primitive.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>

namespace gu {

constexpr int LBS_THREADS = 512;
constexpr int LBS_ITEMS = 16;
constexpr int LBS_SCAN_TILE = LBS_THREADS * LBS_ITEMS;  // counts per scan tile (8192: one wave for 4 M items)
// diagonals per search tile: its slots, counted from the 16-byte boundary at or
// below the first, span at most 4092 + 3 < 4096 positions (16 per search thread)
constexpr int LBS_TILE = 4092;
constexpr int LBS_STHREADS = 256;
constexpr int LBS_SPAN = LBS_STHREADS * 16;  // slot positions per search tile

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

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may start while its predecessor is still running; it waits
// here for the predecessor's completion (and its memory) before reading its
// results.  A kernel lets its successor start launching once all of its own
// CTAs have started (every CTA calls launch_dependents first): the successor's
// CTAs then only take SM room that this kernel's CTAs no longer need.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// Pass 1: the sum of each tile of LBS_SCAN_TILE counts, and the negative-count
// flag.  The counts are read with the default caching so that they are still in
// L2 for pass 2.
__global__ void __launch_bounds__(LBS_THREADS) lbs_tile_sums(const int32_t *__restrict__ counts, int32_t N,
                                                            long long *__restrict__ sums, int *neg)
{
    griddep_launch_dependents();
    __shared__ long long s_part[LBS_THREADS / 32];
    const long long k0 = (long long)blockIdx.x * LBS_SCAN_TILE;
    const int nk = (int)min((long long)LBS_SCAN_TILE, (long long)N - k0);
    long long sum = 0;
    bool bad = false;
#pragma unroll
    for (int r = 0; r < LBS_ITEMS; ++r) {
        const int i = threadIdx.x + r * LBS_THREADS;
        const int32_t c = i < nk ? __ldg(counts + k0 + i) : 0;
        bad |= c < 0;
        sum += c;
    }
    if (__any_sync(FULL_MASK, bad) && lane_id() == 0) atomicOr(neg, 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL_MASK, sum, o);
    if (lane_id() == 0) s_part[warp_in_block()] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
#pragma unroll
        for (int w = 0; w < LBS_THREADS / 32; ++w) t += s_part[w];
        sums[blockIdx.x] = t;
    }
}

// Pass 2: each tile adds up the sums of the tiles before it (all of them are
// final: pass 1 has completed), scans its counts again (from L2), writes its part
// of scanned and the merge-path endpoints of the search tiles whose first
// diagonal lies in its own stretch of the merge (the merge of slot keys
// 0..total-1 with the offsets, ties to the offsets; the stretch of items
// [k0, k1) is diagonals [k0 + P, k1 + P + A), P its prefix and A its sum, and
// depends on nothing else).  The tile holding the last counts knows the total
// and decides whether the call may write results (no negative count, total
// within int32 and within the result capacity, a result buffer when the total
// is positive).
// kpart[t] = offsets consumed at diagonal t * LBS_TILE (t < kpart_len).
__global__ void __launch_bounds__(LBS_THREADS) lbs_scan_apply(
    const int32_t *__restrict__ counts, int32_t N, int32_t ntiles, const long long *__restrict__ sums,
    int32_t *__restrict__ scanned, const int *neg, long long *total_p, int *ok, int32_t *total_out, long long capacity,
    int has_result, int32_t *__restrict__ kpart, long long kpart_len)
{
    griddep_launch_dependents();
    griddep_wait();
    // the tile's counts, then (in place) its offsets relative to the tile's prefix
    // (int32: a tile sum beyond INT32_MAX fails the call anyway); element i at
    // i + i / 16, so that a thread's 16 consecutive elements (stride 17 across the
    // warp) and the striped global accesses are both free of bank conflicts
    __shared__ int32_t s_val[LBS_SCAN_TILE + LBS_SCAN_TILE / 16 + 1];
    __shared__ long long s_warp[33];
    __shared__ long long s_part[LBS_THREADS / 32];
    auto at = [](int i) { return i + (i >> 4); };
    const int t = blockIdx.x;
    const long long k0 = (long long)t * LBS_SCAN_TILE;
    const int nk = (int)min((long long)LBS_SCAN_TILE, (long long)N - k0);
    long long x = 0;  // the sums of tiles 0 .. t-1
    for (int i = threadIdx.x; i < t; i += LBS_THREADS) x += __ldcg(sums + i);
#pragma unroll
    for (int r = 0; r < LBS_ITEMS; ++r) {
        const int i = threadIdx.x + r * LBS_THREADS;
        s_val[at(i)] = i < nk ? __ldg(counts + k0 + i) : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL_MASK, x, o);
    if (lane_id() == 0) s_part[warp_in_block()] = x;
    __syncthreads();
    long long P = 0;
#pragma unroll
    for (int w = 0; w < LBS_THREADS / 32; ++w) P += s_part[w];
    const int base = threadIdx.x * (LBS_ITEMS + 1);  // at(LBS_ITEMS * threadIdx.x)
    long long sum = 0;
#pragma unroll
    for (int i = 0; i < LBS_ITEMS; ++i) sum += s_val[base + i];
    long long agg;
    long long run = block_exscan_ll(sum, s_warp, &agg);
#pragma unroll
    for (int i = 0; i < LBS_ITEMS; ++i) {
        const int32_t c = s_val[base + i];
        s_val[base + i] = (int32_t)run;
        run += c;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nk; i += LBS_THREADS) scanned[k0 + i] = (int32_t)(P + s_val[at(i)]);
    // merge-path endpoints of the search tiles starting in diagonals [k0 + P, k1 + P + agg)
    const long long k1 = k0 + nk;
    const long long d0 = k0 + P, d1 = k1 + P + agg;
    const bool last = t == ntiles - 1;
    const long long first = (d0 + LBS_TILE - 1) / LBS_TILE;
    for (long long tt = first + threadIdx.x; tt * LBS_TILE < d1 && tt < kpart_len; tt += LBS_THREADS) {
        const long long d = tt * LBS_TILE;
        long long lo = max(0ll, d - P - agg - k0), hi = min((long long)nk, d - P - k0);  // items of the tile consumed
        while (lo < hi) {
            const long long k = (lo + hi) >> 1;
            if (P + s_val[at((int)k)] <= d - (k0 + k) - 1) lo = k + 1;
            else hi = k;
        }
        kpart[tt] = (int32_t)(k0 + lo);
    }
    if (last && threadIdx.x == 0) {
        const long long total = P + agg;
        const long long end = (total + N + LBS_TILE - 1) / LBS_TILE;  // the final endpoint, at diagonal total + N
        if (end < kpart_len) kpart[end] = N;
        *total_p = total;
        const bool good = *neg == 0 && total <= INT32_MAX && total <= capacity && (total == 0 || has_result);
        *ok = good ? 1 : 0;
        if (good && total_out) *total_out = (int32_t)total;
    }
}

// Owners of one search tile's slots: every item the tile consumes marks the
// position of its first slot with its id (shared-memory atomicMax: of several
// items starting at one slot, the last owns it), and a block-wide running
// maximum from k0 - 1 gives each slot its owner (upper_bound(scanned, i) - 1).
// Positions count from the 16-byte boundary at or below the tile's first slot;
// thread t holds positions 16 t .. 16 t + 15 and writes them with four 16-byte
// stores (scalar ones at the tile's two ends).  Shared element p sits at
// p + p / 16, so a thread's 16 consecutive elements (stride 17 across a warp)
// meet no bank conflict; a thread reads them twice (its maximum, then its
// owners) rather than holding 16 in registers, so that 8 CTAs fit on an SM.
__global__ void __launch_bounds__(LBS_STHREADS, 8) lbs_search(const int32_t *__restrict__ scanned, int32_t N,
                                                           const long long *total_p, const int *ok,
                                                           const int32_t *__restrict__ kpart,
                                                           int32_t *__restrict__ result)
{
    __shared__ int32_t s_mark[LBS_SPAN + LBS_SPAN / 16];
    __shared__ int32_t s_wmax[LBS_STHREADS / 32];
    griddep_wait();
    if (!*ok) return;
    const long long total = *total_p;
    if (total == 0) return;  // no slots; the path endpoints were not written
    const long long ntile = (total + N + LBS_TILE - 1) / LBS_TILE;
    const int ra = (int)(((uintptr_t)result >> 2) & 3);  // result's element offset from a 16-byte boundary
    const int lane = lane_id(), warp = warp_in_block();
    const int base = threadIdx.x * 17;  // position 16 t in the padded array
    // software pipeline over the CTA's tiles: the next tile's path endpoints and
    // its first 4 * LBS_STHREADS offsets (four per thread, in registers) are
    // loaded before the current tile is worked on
    constexpr int PRE = 4;
    long long tile = blockIdx.x;
    int32_t k0 = 0, k1 = 0;
    int32_t pre[PRE];
    if (tile < ntile) {
        k0 = __ldg(kpart + tile);
        k1 = __ldg(kpart + tile + 1);
#pragma unroll
        for (int r = 0; r < PRE; ++r) {
            const int t = threadIdx.x + r * LBS_STHREADS;
            pre[r] = t < k1 - k0 ? __ldg(scanned + k0 + t) : 0;
        }
    }
    for (; tile < ntile; tile += gridDim.x) {  // block-uniform
        const long long d0 = tile * LBS_TILE;
        const long long d1 = min(d0 + LBS_TILE, total + N);
        const long long nt = tile + gridDim.x;
        int32_t k0n = 0, k1n = 0, pren[PRE];
        if (nt < ntile) {
            k0n = __ldg(kpart + nt);
            k1n = __ldg(kpart + nt + 1);
        }
        const int32_t i0 = (int32_t)(d0 - k0);  // first slot of the tile (total <= INT32_MAX)
        const int nb = k1 - k0, ns = (int)(d1 - d0) - nb;
        const int32_t a = i0 - ((i0 + ra) & 3);  // 16-byte aligned base slot
        const int sh = i0 - a;                    // the tile's slots are positions [sh, sh + ns)
#pragma unroll
        for (int i = 0; i < 16; ++i) s_mark[base + i] = INT_MIN;
#pragma unroll
        for (int r = 0; r < PRE; ++r) {  // the next tile's offsets (its endpoints are in flight)
            const int t = threadIdx.x + r * LBS_STHREADS;
            pren[r] = (nt < ntile && t < k1n - k0n) ? __ldg(scanned + k0n + t) : 0;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PRE; ++r) {
            const int t = threadIdx.x + r * LBS_STHREADS;
            if (t < nb) {
                const int p = pre[r] - a;  // in [sh, sh + ns]
                if (p < LBS_SPAN) atomicMax(&s_mark[p + (p >> 4)], k0 + t);
            }
        }
        for (int t = threadIdx.x + PRE * LBS_STHREADS; t < nb; t += LBS_STHREADS) {
            const int p = __ldg(scanned + k0 + t) - a;
            if (p < LBS_SPAN) atomicMax(&s_mark[p + (p >> 4)], k0 + t);
        }
        __syncthreads();
        int run = INT_MIN;  // this thread's maximum mark; the owners are formed in a second pass
#pragma unroll
        for (int i = 0; i < 16; ++i) run = max(run, s_mark[base + i]);
        int incl = run;  // block-wide running maximum over the threads' positions
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl = max(incl, y);
        }
        if (lane == 31) s_wmax[warp] = incl;
        int carry = __shfl_up_sync(FULL_MASK, incl, 1);
        if (lane == 0) carry = INT_MIN;
        __syncthreads();
        carry = max(carry, k0 - 1);
        for (int w = 0; w < warp; ++w) carry = max(carry, s_wmax[w]);
        const int lo = 16 * (int)threadIdx.x;
        const int vlo = max(lo, sh), vhi = min(lo + 16, sh + ns);
        int32_t *dst = result + ((long long)a + lo);
        if (vlo == lo && vhi == lo + 16) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int4 o;
                o.x = carry = max(carry, s_mark[base + 4 * q]);
                o.y = carry = max(carry, s_mark[base + 4 * q + 1]);
                o.z = carry = max(carry, s_mark[base + 4 * q + 2]);
                o.w = carry = max(carry, s_mark[base + 4 * q + 3]);
                reinterpret_cast<int4 *>(dst)[q] = o;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                carry = max(carry, s_mark[base + i]);
                if (lo + i >= vlo && lo + i < vhi) dst[i] = carry;
            }
        }
        __syncthreads();  // s_mark and s_wmax are reused by the next tile
        k0 = k0n;
        k1 = k1n;
#pragma unroll
        for (int r = 0; r < PRE; ++r) pre[r] = pren[r];
    }
}

// Winner lane per warp of 32 predicates (race_and_resolve_warp).
__global__ void race_and_resolve_kernel(const int32_t *__restrict__ pred, int32_t nwarps, int32_t *__restrict__ winner)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((i >> 5) >= nwarps) return;  // whole warps only (blockDim is a multiple of 32)
    winner[i] = race_and_resolve_warp(pred[i] != 0);
}

// Scratch: the total, the flags, one sum per scan tile, then the search tiles'
// path endpoints (as many as a total of result_capacity slots can need).
constexpr size_t LBS_HEAD = 64;
size_t lbs_scratch_bytes(int32_t N, int64_t result_capacity)
{
    const long long n = N > 0 ? N : 0;
    const size_t ntiles = (size_t)((n + LBS_SCAN_TILE - 1) / LBS_SCAN_TILE);
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    const size_t nsearch = (size_t)((cap + n + LBS_TILE - 1) / LBS_TILE);
    return LBS_HEAD + ntiles * sizeof(unsigned long long) + (nsearch + 2) * sizeof(int32_t);
}

// Device time of the last call on each device: from before the flags are
// cleared to after the search, CUDA events on the call's stream (the three
// kernels overlap, so their sum would overstate it).  Calls are serialised by
// the caller (one scratch area per device).
static cudaEvent_t g_lbs_ev[128][2];
static double g_lbs_last_ms[128];

double lbs_last_ms(int device) { return device >= 0 && device < 128 ? g_lbs_last_ms[device] : 0.0; }

void launch_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result, int64_t result_capacity,
                int32_t *total_dev, int64_t *total_host, void *scratch_ptr, size_t scratch_bytes, cudaStream_t st)
{
    if (N < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "N must be >= 0");
    if (N > 0 && (!counts || !scanned)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null counts or scanned");
    const int32_t ntiles = (int32_t)(((long long)N + LBS_SCAN_TILE - 1) / LBS_SCAN_TILE);
    if (scratch_bytes < lbs_scratch_bytes(N, result_capacity)) throw gu_error(GU_ERR_INTERNAL, "lbs scratch too small");
    char *base = reinterpret_cast<char *>(scratch_ptr);
    long long *tot_d = reinterpret_cast<long long *>(base);
    int *flags = reinterpret_cast<int *>(base + 8);  // neg, ok
    long long *sums = reinterpret_cast<long long *>(base + LBS_HEAD);
    int32_t *kpart = reinterpret_cast<int32_t *>(sums + ntiles);
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    const long long nsearch_max = (cap + N + LBS_TILE - 1) / LBS_TILE;
    // both kernels are queued at once; the scan decides on the device whether the
    // search may run, and the host checks the same conditions after one wait
    long long tot = 0;
    int hflags[3] = {0, 0, 0};
    int dev = 0;
    GU_CUDA_CHECK(cudaGetDevice(&dev));
    cudaEvent_t *ev = dev >= 0 && dev < 128 ? g_lbs_ev[dev] : nullptr;
    if (ev && !ev[0]) {
        GU_CUDA_CHECK(cudaEventCreate(&ev[0]));
        GU_CUDA_CHECK(cudaEventCreate(&ev[1]));
    }
    if (N > 0) {
        if (ev) GU_CUDA_CHECK(cudaEventRecord(ev[0], st));
        GU_CUDA_CHECK(cudaMemsetAsync(flags, 0, LBS_HEAD - 8, st));
        lbs_tile_sums<<<ntiles, LBS_THREADS, 0, st>>>(counts, N, sums, flags);
        cudaLaunchAttribute pdl[1];
        pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        pdl[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ntiles);
        cfg.blockDim = dim3(LBS_THREADS);
        cfg.stream = st;
        cfg.attrs = pdl;
        cfg.numAttrs = 1;
        GU_CUDA_CHECK(cudaLaunchKernelEx(&cfg, lbs_scan_apply, counts, N, ntiles, (const long long *)sums, scanned,
                                         (const int *)flags, tot_d, flags + 1, total_dev, (long long)result_capacity,
                                         result ? 1 : 0, kpart, nsearch_max + 2));
        static int sms_of[128];  // persistent search CTAs: eight per SM, each pipelining its tiles
        int &sms = sms_of[dev >= 0 && dev < 128 ? dev : 0];
        if (!sms) GU_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int gsearch = (int)std::min<long long>(std::max<long long>(nsearch_max, 1), (long long)sms * 8);
        cfg.gridDim = dim3((unsigned)gsearch);
        cfg.blockDim = dim3(LBS_STHREADS);
        GU_CUDA_CHECK(cudaLaunchKernelEx(&cfg, lbs_search, (const int32_t *)scanned, N, (const long long *)tot_d,
                                         (const int *)(flags + 1), (const int32_t *)kpart, result));
        GU_CUDA_CHECK(cudaGetLastError());
        if (ev) GU_CUDA_CHECK(cudaEventRecord(ev[1], st));
        GU_CUDA_CHECK(cudaMemcpyAsync(&tot, tot_d, sizeof(long long), cudaMemcpyDeviceToHost, st));
        GU_CUDA_CHECK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    } else if (total_dev) {
        GU_CUDA_CHECK(cudaMemsetAsync(total_dev, 0, sizeof(int32_t), st));
    }
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    if (ev && N > 0) {
        float ms = 0.f;
        GU_CUDA_CHECK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        g_lbs_last_ms[dev] = ms;
    }
    if (total_host) *total_host = tot;
    if (hflags[0]) throw gu_error(GU_ERR_INVALID_ARGUMENT, "work counts must be >= 0");
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
