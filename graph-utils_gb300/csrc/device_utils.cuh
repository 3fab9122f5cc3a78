// device_utils.cuh -- warp / CTA / grid primitives for sm_103a.
//
// Replaces graph-utils/kernel_utils.cuh:8-35 (lane/warp id, bit extract/insert)
// and graph-utils/race_and_resolve.cuh:13-25 with the *_sync warp intrinsics
// (the reference's __ballot/__shfl forms are pre-Volta and no longer compile),
// and adds the bounded grid barrier and warp-aggregated queue append the
// persistent kernels are built on.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gu_internal.h"

namespace gu {

typedef unsigned long long u64;

constexpr unsigned FULL_MASK = 0xffffffffu;

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_in_block() { return threadIdx.x >> 5; }

// Bit extract / insert (kernel_utils.cuh:21-35 getBit / setBit).
__device__ __forceinline__ int get_bit(unsigned val, int pos) { return (val >> pos) & 1u; }
__device__ __forceinline__ unsigned set_bit(unsigned val, unsigned bit, int pos)
{
    return (val & ~(1u << pos)) | ((bit & 1u) << pos);
}

// Warp leader election: the highest lane whose predicate is true; a lane's own
// id when no lane votes (race_and_resolve.cuh:13-25).  All lanes of `mask` call.
__device__ __forceinline__ int race_and_resolve_warp(int predicate, unsigned mask = FULL_MASK)
{
    unsigned vote = __ballot_sync(mask, predicate);
    int winner = lane_id();
    if (vote) winner = 31 - __clz(vote);
    return winner;
}

__device__ __forceinline__ u64 global_timer_ns()
{
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ u64 ld_acquire_u64(const u64 *p)
{
    u64 v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned *p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile_i32(const int *p) { return *(const volatile int *)p; }
__device__ __forceinline__ u64 ld_volatile_u64(const u64 *p) { return *(const volatile u64 *)p; }

// Grid-wide barrier for a cooperative launch (all CTAs co-resident).  `bar` is a
// monotonically increasing arrival counter zeroed before the launch; `epoch`
// counts this CTA's barriers.  Returns false if any CTA reported an error.
// Thread 0 alone reads the global words every thread needs after the barrier
// (the error flag, and n 64-bit words from src into the shared dst): one
// request per CTA instead of one per warp, all at the same address.
//
// nblocks: the CTAs that meet at the barrier (0: the whole grid; a CTA group of a
// work-queue launch passes its own size and its own counter).
//
// The wait is bounded by limit_ns (a launch argument, gu_set_wait_limit; 4 s by
// default): a wait that runs out records DEV_ERR_BARRIER_TIMEOUT in *err and
// returns false; every block then leaves the kernel and the host reports
// GU_ERR_TIMEOUT.  No wait is unbounded.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err, unsigned &epoch, u64 limit_ns,
                                             const u64 *src = nullptr, u64 *dst = nullptr, int n = 0,
                                             unsigned nblocks = 0)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x < 32) {
        if (threadIdx.x == 0) {
            epoch += 1;
            const unsigned target = epoch * (nblocks ? nblocks : gridDim.x);
            __threadfence();
            red_release_add_u32(bar, 1u);
            u64 t0 = 0;
            unsigned spins = 0;
            while (true) {
                unsigned v = ld_acquire_u32(bar);
                if ((int)(v - target) >= 0) break;
                if (ld_volatile_i32(err) != 0) break;
                if ((++spins & 63u) == 0) {
                    u64 now = global_timer_ns();
                    if (t0 == 0) t0 = now;
                    else if (now - t0 > limit_ns) {
                        atomicCAS(err, 0, (int)DEV_ERR_BARRIER_TIMEOUT);
                        break;
                    }
                }
                __nanosleep(32);
            }
            __threadfence();
            s_ok = ld_volatile_i32(err) == 0;
        }
        // the words every thread needs after the barrier, read by the lanes of
        // warp 0 at once (one request) instead of one after another by thread 0
        // (a barrier in 2.2 us instead of 4.4 us at 304 CTAs of 512 threads)
        __syncwarp();
        for (int i = threadIdx.x; i < n; i += 32) dst[i] = ld_acquire_u64(src + i);
    }
    __syncthreads();
    return s_ok != 0;
}

// Lanes of `mask` append one value each to q at a reserved, contiguous range.
// The counter is bumped once per warp; `weight` (e.g. a degree) is summed into
// *wsum by the same leader.
__device__ __forceinline__ void warp_append(int32_t value, int32_t *q, int *qlen, u64 *wsum, unsigned weight)
{
    const unsigned mask = __activemask();
    const int lane = lane_id();
    const int leader = __ffs(mask) - 1;
    const int rank = __popc(mask & ((1u << lane) - 1u));
    const unsigned wtot = __reduce_add_sync(mask, weight);
    int base = 0;
    if (lane == leader) {
        base = atomicAdd(qlen, __popc(mask));
        atomicAdd(wsum, (u64)wtot);
    }
    base = __shfl_sync(mask, base, leader);
    q[base + rank] = value;
}

__device__ __forceinline__ u64 warp_or_u64(unsigned mask, u64 x)
{
    unsigned lo = __reduce_or_sync(mask, (unsigned)x);
    unsigned hi = __reduce_or_sync(mask, (unsigned)(x >> 32));
    return ((u64)hi << 32) | lo;
}

}  // namespace gu
