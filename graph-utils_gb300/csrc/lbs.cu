// lbs.cu -- load-balanced search and warp race-and-resolve on sm_103a.
//
// Load-balanced search (load_balanced_search.cu:123-192, example lbs.cu:18-31):
// given per-item work counts, scanned = exclusive prefix sum (int32), total =
// sum, and result[i] for every work slot i < total = the item owning it
// (upper_bound(scanned, i) - 1).  The reference runs it in ONE CTA whose threads
// each walk the scanned array from the start (quadratic in the item count);
// here two kernels:
//   1. lbs_scan_single: a single-pass scan with decoupled look-back.  A CTA
//      takes the next tile of 8192 counts (a ticket, so it only ever waits on
//      tiles already taken), scans it in shared memory, publishes the tile's sum
//      and then -- after looking back over its predecessors' published sums --
//      its inclusive prefix; it writes its part of scanned and the merge-path
//      endpoints of the search tiles whose first diagonal lies in its own
//      stretch of the merge (the merge of slot keys 0..total-1 with the offsets,
//      ties to the offsets; the stretch of items [k0, k1) is diagonals
//      [k0 + P, k1 + P + A), P its prefix and A its sum, and depends on nothing
//      else).  The tile holding the last counts knows the total and decides
//      whether the call may write results (no negative count, total within
//      int32 and within the result capacity, a result buffer when the total is
//      positive).  Every wait is bounded.
//   2. lbs_search: each CTA takes search tiles of 4092 diagonals; the items a
//      tile consumes mark their first slots in shared memory and a block-wide
//      running maximum turns the marks into owners, written 16 bytes at a time.
//   Both are queued at once; the host waits once, at the end.
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

// Tile status word of the look-back: flag in bits 62-63 (1: the tile's sum, 2:
// its inclusive prefix), value in bits 0-61 (sums of int32 counts over at most
// 2^31 items fit).
constexpr unsigned long long LB_FLAG_SUM = 1ull << 62, LB_FLAG_PREFIX = 2ull << 62;
constexpr unsigned long long LB_VALUE = (1ull << 62) - 1ull;

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Scan, merge-path endpoints and verdict in one pass (see the file comment).
// kpart[t] = offsets consumed at diagonal t * LBS_TILE (t < kpart_len).
__global__ void __launch_bounds__(LBS_THREADS) lbs_scan_single(
    const int32_t *__restrict__ counts, int32_t N, int32_t ntiles, int32_t *__restrict__ scanned,
    unsigned long long *status, int *ticket, int *neg, long long *total_p, int *ok, int *err, int32_t *total_out,
    long long capacity, int has_result, int32_t *__restrict__ kpart, long long kpart_len, unsigned long long limit_ns)
{
    // the tile's counts, then (in place) its offsets relative to the tile's prefix
    // (int32: a tile sum beyond INT32_MAX fails the call anyway); element i at
    // i + i / 16, so that a thread's 16 consecutive elements (stride 17 across the
    // warp) and the striped global accesses are both free of bank conflicts
    __shared__ int32_t s_val[LBS_SCAN_TILE + LBS_SCAN_TILE / 16 + 1];
    __shared__ long long s_warp[33];
    __shared__ int s_tile;
    __shared__ long long s_prefix;
    auto at = [](int i) { return i + (i >> 4); };
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1);
    __syncthreads();
    const int t = s_tile;
    const long long k0 = (long long)t * LBS_SCAN_TILE;
    const int nk = (int)min((long long)LBS_SCAN_TILE, (long long)N - k0);
    // counts in, coalesced; each thread then sums its LBS_ITEMS consecutive ones
    bool bad = false;
#pragma unroll 4
    for (int i = threadIdx.x; i < LBS_SCAN_TILE; i += LBS_THREADS) {
        const int32_t c = i < nk ? __ldcs(counts + k0 + i) : 0;
        bad |= c < 0;
        s_val[at(i)] = c;
    }
    if (__any_sync(FULL_MASK, bad) && lane_id() == 0) {
        atomicOr(neg, 1);
        __threadfence();
    }
    __syncthreads();
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
    // look-back: warp 0 publishes the sum, then reads 128 predecessors at a time
    // (four per lane, loads issued together) until it meets one that has published
    // its inclusive prefix, and publishes its own.  In the first wave the
    // published prefixes advance about one tile per L2 round trip, so a window
    // of 32 left late tiles a dozen rounds behind.
    constexpr int LB_WIN = 4;
    if (threadIdx.x < 32) {
        const int lane = lane_id();
        long long prefix = 0;
        if (t == 0) {
            if (lane == 0) st_release_u64(status, LB_FLAG_PREFIX | ((unsigned long long)agg & LB_VALUE));
        } else {
            if (lane == 0) st_release_u64(status + t, LB_FLAG_SUM | ((unsigned long long)agg & LB_VALUE));
            long long j = t - 1;  // the nearest predecessor of this round
            const unsigned long long t0 = global_timer_ns();
            bool timed_out = false;
            while (true) {
                unsigned long long v[LB_WIN];
#pragma unroll
                for (int r = 0; r < LB_WIN; ++r) {  // element e = 32 r + lane is tile j - e
                    const long long idx = j - (32 * r + lane);
                    v[r] = idx >= 0 ? ld_acquire_u64(status + idx) : LB_FLAG_PREFIX;
                }
                unsigned spins = 0;
                while (true) {
                    bool waiting = false;
#pragma unroll
                    for (int r = 0; r < LB_WIN; ++r) waiting |= (v[r] >> 62) == 0;
                    if (!__any_sync(FULL_MASK, waiting)) break;
#pragma unroll
                    for (int r = 0; r < LB_WIN; ++r)  // a predecessor has not published yet
                        if ((v[r] >> 62) == 0) v[r] = ld_acquire_u64(status + (j - (32 * r + lane)));
                    if ((++spins & 63u) == 0) {
                        const bool late = global_timer_ns() - t0 > limit_ns || ld_volatile_i32(err) != 0;
                        if (__any_sync(FULL_MASK, late)) {
                            timed_out = true;
                            break;
                        }
                    }
                }
                if (timed_out) break;
                int stop = 32 * LB_WIN;  // the nearest element holding a prefix (none: the whole window)
#pragma unroll
                for (int r = LB_WIN - 1; r >= 0; --r) {
                    const unsigned done = __ballot_sync(FULL_MASK, (v[r] >> 62) == 2);
                    if (done) stop = 32 * r + __ffs(done) - 1;
                }
                long long x = 0;
#pragma unroll
                for (int r = 0; r < LB_WIN; ++r)
                    if (32 * r + lane <= stop) x += (long long)(v[r] & LB_VALUE);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL_MASK, x, o);
                prefix += x;
                if (stop < 32 * LB_WIN) break;
                j -= 32 * LB_WIN;
            }
            if (timed_out) {
                if (lane == 0) atomicCAS(err, 0, 1);
                prefix = 0;
            }
            // published even after a timeout, so that no successor waits on this tile
            if (lane == 0) st_release_u64(status + t, LB_FLAG_PREFIX | ((unsigned long long)(prefix + agg) & LB_VALUE));
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    const long long P = s_prefix;
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
        __threadfence();
        const bool good = ld_volatile_i32(neg) == 0 && ld_volatile_i32(err) == 0 && total <= INT32_MAX &&
                          total <= capacity && (total == 0 || has_result);
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
    if (!*ok) return;
    const long long total = *total_p;
    if (total == 0) return;  // no slots; the path endpoints were not written
    const long long ntile = (total + N + LBS_TILE - 1) / LBS_TILE;
    const int ra = (int)(((uintptr_t)result >> 2) & 3);  // result's element offset from a 16-byte boundary
    const int lane = lane_id(), warp = warp_in_block();
    const int base = threadIdx.x * 17;  // position 16 t in the padded array
    for (long long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {  // block-uniform
        const long long d0 = tile * LBS_TILE;
        const long long d1 = min(d0 + LBS_TILE, total + N);
        const int32_t k0 = __ldg(kpart + tile), k1 = __ldg(kpart + tile + 1);
        const int32_t i0 = (int32_t)(d0 - k0);  // first slot of the tile (total <= INT32_MAX)
        const int nb = k1 - k0, ns = (int)(d1 - d0) - nb;
        const int32_t a = i0 - ((i0 + ra) & 3);  // 16-byte aligned base slot
        const int sh = i0 - a;                    // the tile's slots are positions [sh, sh + ns)
#pragma unroll
        for (int i = 0; i < 16; ++i) s_mark[base + i] = INT_MIN;
        __syncthreads();
        for (int t = threadIdx.x; t < nb; t += LBS_STHREADS) {
            const int p = __ldg(scanned + k0 + t) - a;  // in [sh, sh + ns]
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
    }
}

// Winner lane per warp of 32 predicates (race_and_resolve_warp).
__global__ void race_and_resolve_kernel(const int32_t *__restrict__ pred, int32_t nwarps, int32_t *__restrict__ winner)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((i >> 5) >= nwarps) return;  // whole warps only (blockDim is a multiple of 32)
    winner[i] = race_and_resolve_warp(pred[i] != 0);
}

// Scratch: the total, the flags, the ticket, one look-back status word per scan
// tile, then the search tiles' path endpoints (as many as a total of
// result_capacity slots can need).
constexpr size_t LBS_HEAD = 64;
size_t lbs_scratch_bytes(int32_t N, int64_t result_capacity)
{
    const long long n = N > 0 ? N : 0;
    const size_t ntiles = (size_t)((n + LBS_SCAN_TILE - 1) / LBS_SCAN_TILE);
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    const size_t nsearch = (size_t)((cap + n + LBS_TILE - 1) / LBS_TILE);
    return LBS_HEAD + ntiles * sizeof(unsigned long long) + (nsearch + 2) * sizeof(int32_t);
}

void launch_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result, int64_t result_capacity,
                int32_t *total_dev, int64_t *total_host, void *scratch_ptr, size_t scratch_bytes, cudaStream_t st)
{
    if (N < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "N must be >= 0");
    if (N > 0 && (!counts || !scanned)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null counts or scanned");
    const int32_t ntiles = (int32_t)(((long long)N + LBS_SCAN_TILE - 1) / LBS_SCAN_TILE);
    if (scratch_bytes < lbs_scratch_bytes(N, result_capacity)) throw gu_error(GU_ERR_INTERNAL, "lbs scratch too small");
    char *base = reinterpret_cast<char *>(scratch_ptr);
    long long *tot_d = reinterpret_cast<long long *>(base);
    int *flags = reinterpret_cast<int *>(base + 8);  // neg, ok, err, ticket
    unsigned long long *status = reinterpret_cast<unsigned long long *>(base + LBS_HEAD);
    int32_t *kpart = reinterpret_cast<int32_t *>(status + ntiles);
    const long long cap = result_capacity < 0 ? 0 : (result_capacity > INT32_MAX ? INT32_MAX : result_capacity);
    const long long nsearch_max = (cap + N + LBS_TILE - 1) / LBS_TILE;
    // both kernels are queued at once; the scan decides on the device whether the
    // search may run, and the host checks the same conditions after one wait
    long long tot = 0;
    int hflags[3] = {0, 0, 0};
    if (N > 0) {
        GU_CUDA_CHECK(cudaMemsetAsync(flags, 0, (LBS_HEAD - 8) + (size_t)ntiles * sizeof(unsigned long long), st));
        lbs_scan_single<<<ntiles, LBS_THREADS, 0, st>>>(counts, N, ntiles, scanned, status, flags + 3, flags, tot_d,
                                                        flags + 1, flags + 2, total_dev, result_capacity,
                                                        result ? 1 : 0, kpart, nsearch_max + 2, wait_limit_ns());
        const int gsearch = (int)std::min<long long>(std::max<long long>(nsearch_max, 1), 4096);
        lbs_search<<<gsearch, LBS_STHREADS, 0, st>>>(scanned, N, tot_d, flags + 1, kpart, result);
        GU_CUDA_CHECK(cudaGetLastError());
        GU_CUDA_CHECK(cudaMemcpyAsync(&tot, tot_d, sizeof(long long), cudaMemcpyDeviceToHost, st));
        GU_CUDA_CHECK(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    } else if (total_dev) {
        GU_CUDA_CHECK(cudaMemsetAsync(total_dev, 0, sizeof(int32_t), st));
    }
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    if (hflags[2]) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit (scan look-back)");
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
