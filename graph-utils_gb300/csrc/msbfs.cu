// msbfs.cu -- batched multi-source BFS on sm_103a.
//
// One persistent, cooperatively launched kernel runs every batch of sources and
// every level of each batch; levels are separated by a bounded grid barrier
// (device_utils.cuh), so a whole multi-source search is a single launch.
//
// A batch holds 64*W sources (W 64-bit words, W in {1,2,4}).  Bit i of word q
// of every per-vertex record stands for source row0 + 64q + i.  State, in SoA
// layout with the W words of one vertex contiguous (16/32-byte vector access):
//   seen[n][W]      sources that reached the vertex in an earlier level
//   f[3][n][W]      frontier bitmaps F_j, rotating over three levels
//   plane[P][n][W]  bit b of the BFS level of every (source, vertex) pair
//   stamp[n]        last level that appended the vertex to a queue (W > 1)
//   q[3], qoff[3]   frontier queues; qoff[i] = out-edges of q[0..i) (an
//                   exclusive prefix sum reserved together with the slot, so
//                   the next level splits the frontier's edges evenly)
// For n = 2^20 and W = 4 one bitmap array is 32 MiB, so the arrays touched at
// random during a level stay in the 126 MiB L2.  Distances are not written
// during the search: the level bit-planes are transposed into the int32
// distance rows once per batch, each row segment written whole and coalesced.
//
// Phase j of a batch (one grid barrier per level; bottom-up levels add one or
// two, see the bottom-up section):
//   * finalise F_{j-1}: set the level bits of j-1 in the planes (seen took the
//     bits when they were discovered)
//   * clear F_{j-2}
//   * discover F_j top-down (gather the adjacency of the F_{j-1} queue and claim
//     the bits missing from seen with 64-bit OR reductions into seen and F_j; on
//     an expansion over more edges than the graph has vertices, OR the frontier
//     words into F_j unread and let one scan after the level drop the bits seen
//     before, update seen and build the queue) or bottom-up (each vertex still
//     missing some active source ORs its in-neighbours' F_{j-1} words, stopping
//     as soon as every missing active source is found).
// A source is active while its frontier is non-empty; the active mask of F_j is
// OR-reduced per CTA in shared memory during phase j.  Direction: top-down ->
// bottom-up when the frontier's out-edges exceed m / alpha, back when it holds
// fewer than n / beta vertices (after Beamer, Asanovic, Patterson, SC'12) or
// its out-edges are fewer than n / gamma (a wide frontier of low-degree
// vertices: expanding it costs less than one sweep over all vertices).
//
// Top-down gather strategies restate the reference kernels' neighbour gathering
// (file:line in include/gu.h); AUTO uses the edge-balanced merge-path gather.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdlib>
#include <vector>

namespace gu {

constexpr int MS_THREADS = 512;
constexpr int MS_MIN_BLOCKS = 2;  // <= 64 registers: 2 CTAs (1024 threads) per SM
constexpr int MAXW = 4;
constexpr int MAX_PLANES = 31;              // levels < 2^31
constexpr int EAGER_PLANES = 4;             // zeroed with the batch (levels < 16)
constexpr int CTA_DEGREE_THRESHOLD = 2048;  // CTA_warp.cu:44
constexpr int QPACK_SHIFT = 38;             // qpack = (count << 38) | edges
constexpr u64 QPACK_EDGES = (1ull << QPACK_SHIFT) - 1ull;

struct __align__(128) MsCtl {
    unsigned bar;
    int err;
    int td_levels;
    int bu_levels;
    int max_level;
    int nblocks;  // grid size of the launch (profiling)
    int item;     // work-queue launch: the item the group works on (set by its first CTA)
    int pad0;
    u64 qpack[4];
    int work[4];
    u64 rpack;  // bottom-up level: rare-source frontier list, (count << 38) | edges
    int wo_next;  // distance write-out: next tile to take (zeroed with the batch)
    int pad1;
    u64 active[4][MAXW];
};
static_assert(sizeof(MsCtl) <= 256, "control block must fit its reserved space");

// Per-phase timeline (profiling hook).  Every CTA's thread 0 stamps the end of
// its share of phase i (atomicMax of the global timer, so t_last_ns is the
// slowest CTA); thread 0 of the grid also records what the phase was.
constexpr int TIMELINE_MAX = 1024;
struct MsEvent {
    u64 t_last_ns;
    int32_t batch, level;
    int32_t bottom_up, qlen;
    long long qedges;
    u64 idle_ns;  // summed over CTAs: time spent waiting at the grid barriers of this phase
};
// Per-source coverage of each level's discoveries: cover[j & 3][s] counts the
// CTAs that discovered source s in F_j (a source with a frontier of a few dozen
// vertices is seen by a few dozen CTAs, an empty frontier by none).
constexpr size_t COVER_OFF = (256 + sizeof(MsEvent) * TIMELINE_MAX + sizeof(int) * 4 + 15) & ~size_t(15);
constexpr int COVER_SLOT = 64 * MAXW;
constexpr size_t CTL_REGION = COVER_OFF + sizeof(int) * 4 * COVER_SLOT;

__device__ __forceinline__ void record_event(MsCtl *ctl, int i, bool describe, int batch, int level, int bu,
                                             int qlen, long long qedges)
{
    MsEvent *ev = reinterpret_cast<MsEvent *>(reinterpret_cast<char *>(ctl) + 256);
    if (i >= TIMELINE_MAX) return;
    atomicMax(&ev[i].t_last_ns, global_timer_ns());
    if (describe) {
        ev[i].batch = batch;
        ev[i].level = level;
        ev[i].bottom_up = bu;
        ev[i].qlen = qlen;
        ev[i].qedges = qedges;
        *reinterpret_cast<int *>(ev + TIMELINE_MAX) = i + 1;
    }
}

struct MsArgs {
    const int32_t *__restrict__ R;
    const int32_t *__restrict__ C;
    const int32_t *__restrict__ RT;
    const int32_t *__restrict__ CT;
    const int32_t *__restrict__ F;
    const int32_t *__restrict__ light;  // bottom-up degree classes (ascending vertex lists)
    const int32_t *__restrict__ mid;
    const int32_t *__restrict__ wide;
    const int32_t *__restrict__ heavy;
    int32_t n;
    int32_t nlight, nmid, nwide, nheavy;
    int64_t m;
    const int32_t *sources;
    int32_t k;
    int32_t *dist;
    unsigned long long *reach;  // per-source reachable-vertex counts (null: none)
    int64_t ld;
    u64 *seen;
    u64 *fr[3];
    u64 *plane;  // [nplanes][n][W]
    int nplanes;
    int32_t *stamp;
    int32_t *q[3];
    int32_t *qoff[3];
    MsCtl *ctl;
    int *cover;  // [4][COVER_SLOT]
    float alpha, beta, gamma;
    float rare_frac;  // bottom-up levels leave a source covered by fewer CTAs to top-down
    int degbits;
    unsigned long long wait_ns;  // bound of every grid-barrier wait (gu_set_wait_limit)
};

struct Lvl {
    int cur, nxt, prv, slot;
    int qlen, qlen_prev;
    long long qedges;
    const int32_t *qcur;
    const int32_t *qcur_off;
    int32_t *qnxt;
    int32_t *qnxt_off;
    const int32_t *qprev;
    const u64 *fcur;
    u64 *fnxt;
    u64 *fprv;
    u64 *sact;    // shared-memory active-source accumulator of this CTA
    int32_t lev;  // BFS level of F_{j-1}
    int32_t tag;  // stamp of level j (j + 1)
    u64 active[MAXW];  // bottom-up levels: without the rare sources
    bool rare_td;      // bottom-up level with rare sources expanded top-down
    bool scanq;        // top-down level whose next queue is built by a scan of F_j afterwards
};

struct GridG {
    __device__ static long long rank() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ static long long size() { return (long long)gridDim.x * blockDim.x; }
    __device__ static int blk() { return blockIdx.x; }
    __device__ static int nblk() { return gridDim.x; }
};

// One CTA group of a work-queue launch (ms_queue_kernel): CTAs [base, base + nblk)
// of the grid, set by each CTA at the start of the launch.
__shared__ int s_grp_base, s_grp_nblk;
struct GroupG {
    __device__ static long long rank() { return (long long)(blockIdx.x - s_grp_base) * blockDim.x + threadIdx.x; }
    __device__ static long long size() { return (long long)s_grp_nblk * blockDim.x; }
    __device__ static int blk() { return blockIdx.x - s_grp_base; }
    __device__ static int nblk() { return s_grp_nblk; }
};

// One shared-memory buffer per CTA for the phases' staging (merge-path owners
// and discovered vertices, distance-row tiles); phases never overlap in a CTA.
constexpr int MS_SMEM_BYTES = 32768;
__device__ __forceinline__ unsigned char *ms_smem()
{
    __shared__ __align__(16) unsigned char buf[MS_SMEM_BYTES];
    return buf;
}

// ---- W-word helpers -----------------------------------------------------------
// Four words (one 256-source group, 32-byte aligned) move as one 256-bit
// access: one L1 wavefront per lane instead of two.
template <int W>
__device__ __forceinline__ void ldw(const u64 *p, u64 (&x)[W])
{
    if constexpr (W == 1) {
        x[0] = __ldcg(p);
    } else if constexpr (W == 4) {
        asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];"
                     : "=l"(x[0]), "=l"(x[1]), "=l"(x[2]), "=l"(x[3]) : "l"(p) : "memory");
    } else {
#pragma unroll
        for (int i = 0; i < W / 2; ++i) {
            const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(p) + i);
            x[2 * i] = v.x;
            x[2 * i + 1] = v.y;
        }
    }
}

// L1-allocating load of words that no thread changes in a way that matters
// within the current phase (the frontier being expanded, seen | frontier):
// hub vertices' words are re-read by many warps of an SM.  The grid barrier's
// acquire fence invalidates L1, so no line survives from an earlier phase.
template <int W>
__device__ __forceinline__ void ldw_l1(const u64 *p, u64 (&x)[W])
{
    if constexpr (W == 1) {
        x[0] = __ldca(p);
    } else if constexpr (W == 4) {
        asm volatile("ld.global.ca.v4.u64 {%0, %1, %2, %3}, [%4];"
                     : "=l"(x[0]), "=l"(x[1]), "=l"(x[2]), "=l"(x[3]) : "l"(p) : "memory");
    } else {
#pragma unroll
        for (int i = 0; i < W / 2; ++i) {
            const ulonglong2 v = __ldca(reinterpret_cast<const ulonglong2 *>(p) + i);
            x[2 * i] = v.x;
            x[2 * i + 1] = v.y;
        }
    }
}

template <int W>
__device__ __forceinline__ void stw(u64 *p, const u64 (&x)[W])
{
    if constexpr (W == 1) {
        p[0] = x[0];
    } else if constexpr (W == 4) {
        asm volatile("st.global.v4.u64 [%0], {%1, %2, %3, %4};"
                     :: "l"(p), "l"(x[0]), "l"(x[1]), "l"(x[2]), "l"(x[3]) : "memory");
    } else {
#pragma unroll
        for (int i = 0; i < W / 2; ++i)
            reinterpret_cast<ulonglong2 *>(p)[i] = make_ulonglong2(x[2 * i], x[2 * i + 1]);
    }
}

template <int W>
__device__ __forceinline__ void zerow(u64 *p)
{
    const u64 z[W] = {};
    stw<W>(p, z);
}

template <int W>
__device__ __forceinline__ bool anyw(const u64 (&x)[W])
{
    u64 o = 0;
#pragma unroll
    for (int q = 0; q < W; ++q) o |= x[q];
    return o != 0;
}

__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// ---- frontier queue append ------------------------------------------------------
// Lanes of the calling (possibly partial) warp append their vertices; one
// 64-bit atomicAdd reserves both the queue slots and the range of their
// out-edges.  The exclusive prefix of the degrees over the active lanes is a
// bit-sliced ballot sum (works for any active mask).
__device__ __forceinline__ void append_to(const MsArgs &a, u64 *pack, int32_t *qnxt, int32_t *qnxt_off, int32_t w)
{
    const unsigned deg = (unsigned)(__ldg(a.R + w + 1) - __ldg(a.R + w));
    const unsigned mask = __activemask();
    const int lane = lane_id();
    const int leader = __ffs(mask) - 1;
    const unsigned lt = lanemask_lt();
    u64 excl = 0, tot = 0;
    for (int b = 0; b < a.degbits; ++b) {
        const unsigned v = __ballot_sync(mask, (deg >> b) & 1u);
        excl += (u64)__popc(v & lt) << b;
        tot += (u64)__popc(v) << b;
    }
    u64 old = 0;
    if (lane == leader) old = atomicAdd(pack, ((u64)__popc(mask) << QPACK_SHIFT) | tot);
    old = __shfl_sync(mask, old, leader);
    const int pos = (int)(old >> QPACK_SHIFT) + __popc(mask & lt);
    qnxt[pos] = w;
    qnxt_off[pos] = (int32_t)((old & QPACK_EDGES) + excl);
}

__device__ __forceinline__ void append_vertex(const MsArgs &a, int slot, int32_t *qnxt, int32_t *qnxt_off,
                                              int32_t w)
{
    append_to(a, &a.ctl->qpack[slot], qnxt, qnxt_off, w);
}

// ---- where a top-down visit puts the vertices it discovers first --------------------
struct GlobalQ {  // straight into the level's queue, one 64-bit atomic per warp
    __device__ __forceinline__ void push(const MsArgs &a, const Lvl &L, int32_t w) const
    {
        append_vertex(a, L.slot, L.qnxt, L.qnxt_off, w);
    }
};

// Per-CTA collection in shared memory, appended to the level's queue by
// cta_flush with one 64-bit atomic per 2048 vertices: the queue counter is a
// single address, and one atomic per warp from every warp of the GPU
// serialises there when a level discovers 10^5..10^6 vertices.  Pushes beyond
// the capacity go to the queue directly.
constexpr int CQ_PER_THREAD = 4;
struct CtaQ {
    int32_t *v;  // [cap] shared
    int *n;      // shared: pushes since the last flush (the excess over cap went direct)
    int cap;
    __device__ __forceinline__ void push(const MsArgs &a, const Lvl &L, int32_t w) const
    {
        const unsigned mask = __activemask();
        const int leader = __ffs(mask) - 1;
        int base = 0;
        if (lane_id() == leader) base = atomicAdd(n, __popc(mask));
        base = __shfl_sync(mask, base, leader);
        const int pos = base + __popc(mask & lanemask_lt());
        if (pos < cap) v[pos] = w;
        else append_vertex(a, L.slot, L.qnxt, L.qnxt_off, w);
    }
};

// The CTA's queue counter and flush scratch (zeroed at kernel start; every
// flush leaves the counter at zero).
__device__ __forceinline__ int *cq_count()
{
    __shared__ int n;
    return &n;
}
__device__ __forceinline__ u64 *cq_scan()
{
    __shared__ u64 scan[33];
    return scan;
}

// Append the CTA's collected vertices to the level's queue: degrees scanned
// across the CTA, one atomic reserves the slots and the edge range.  Every
// thread of the CTA calls it after a __syncthreads (the count is then uniform).
__device__ void cta_flush(const MsArgs &a, const Lvl &L, const CtaQ &cq)
{
    u64 *s_scan = cq_scan();
    const int cnt = min(*cq.n, cq.cap);
    const int lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int per_round = blockDim.x * CQ_PER_THREAD;
    for (int r0 = 0; r0 < cnt; r0 += per_round) {
        const int i0 = r0 + threadIdx.x * CQ_PER_THREAD;
        int32_t v[CQ_PER_THREAD];
        unsigned d[CQ_PER_THREAD];
        u64 sum = 0;
#pragma unroll
        for (int t = 0; t < CQ_PER_THREAD; ++t) {
            v[t] = i0 + t < cnt ? cq.v[i0 + t] : -1;
            d[t] = v[t] >= 0 ? (unsigned)(__ldg(a.R + v[t] + 1) - __ldg(a.R + v[t])) : 0u;
            sum += d[t];
        }
        u64 inc = sum;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const u64 y = __shfl_up_sync(FULL_MASK, inc, off);
            if (lane >= off) inc += y;
        }
        if (lane == 31) s_scan[warp] = inc;
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 run = 0;
            for (int k = 0; k < nw; ++k) {
                const u64 t = s_scan[k];
                s_scan[k] = run;
                run += t;
            }
            const int rc = min(cnt - r0, per_round);
            s_scan[32] = atomicAdd(&a.ctl->qpack[L.slot], ((u64)rc << QPACK_SHIFT) | run);
        }
        __syncthreads();
        const u64 old = s_scan[32];
        const long long slot0 = (long long)(old >> QPACK_SHIFT) + (i0 - r0);
        u64 e = (old & QPACK_EDGES) + s_scan[warp] + (inc - sum);
#pragma unroll
        for (int t = 0; t < CQ_PER_THREAD; ++t) {
            if (v[t] >= 0) {
                L.qnxt[slot0 + t] = v[t];
                L.qnxt_off[slot0 + t] = (int32_t)e;
            }
            e += d[t];
        }
        __syncthreads();  // s_scan is reused by the next round
    }
    if (threadIdx.x == 0) *cq.n = 0;
    __syncthreads();
}

// ---- top-down visit: frontier bits f arrive at vertex w over one edge ----------------
// seen(w) holds every source that has reached w, this level's finds included:
// a visit claims the bits f & ~seen with fire-and-forget OR reductions into
// seen and into the next frontier.  A stale read (a bit another visit set a
// moment ago) only repeats an idempotent reduction; "first" (the one append of
// w to the next queue) is decided by the level stamp (W > 1) or by the
// frontier word having been zero (W = 1).
__device__ __forceinline__ void red_or(u64 *p, u64 v)
{
    // volatile: kept in order with the grid barrier's own (volatile) fences
    asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v));
}

template <int W>
__device__ __forceinline__ bool claim(const MsArgs &a, const Lvl &L, size_t o, const u64 (&nb)[W], bool &first)
{
    bool found = false;
#pragma unroll
    for (int q = 0; q < W; ++q) {
        if (nb[q]) {
            red_or(a.seen + o + q, nb[q]);
            if (W == 1) {
                if (atomicOr(L.fnxt + o + q, nb[q]) == 0) first = true;
            } else {
                red_or(L.fnxt + o + q, nb[q]);
            }
            found = true;
        }
    }
    return found;
}

template <int W, class Q = GlobalQ>
__device__ __forceinline__ void td_visit(const MsArgs &a, const Lvl &L, const u64 (&f)[W], int32_t w,
                                         const Q &qu = Q())
{
    const size_t o = (size_t)w * W;
    if (L.scanq) {  // OR every frontier bit into F_j; the scan after the level removes the known ones
#pragma unroll
        for (int q = 0; q < W; ++q)
            if (f[q]) red_or(L.fnxt + o + q, f[q]);
        return;
    }
    u64 s[W], nb[W];
    ldw<W>(a.seen + o, s);
#pragma unroll
    for (int q = 0; q < W; ++q) nb[q] = f[q] & ~s[q];
    bool first = false;
    const bool found = claim<W>(a, L, o, nb, first);
    if (W > 1 && found) first = atomicMax(a.stamp + w, L.tag) < L.tag;
    if (first) qu.push(a, L, w);
}

// Two visits with their state loads issued together (w2 < 0: none).
template <int W, class Q = GlobalQ>
__device__ __forceinline__ void td_visit2(const MsArgs &a, const Lvl &L, const u64 (&f)[W], int32_t w,
                                          const u64 (&f2)[W], int32_t w2, const Q &qu = Q())
{
    const size_t o = (size_t)w * W, o2 = (size_t)(w2 < 0 ? w : w2) * W;
    if (L.scanq) {
#pragma unroll
        for (int q = 0; q < W; ++q) {
            if (f[q]) red_or(L.fnxt + o + q, f[q]);
            if (w2 >= 0 && f2[q]) red_or(L.fnxt + o2 + q, f2[q]);
        }
        return;
    }
    u64 s[W], s2[W];
    ldw<W>(a.seen + o, s);
    ldw<W>(a.seen + o2, s2);
    u64 nb[W], nb2[W];
#pragma unroll
    for (int q = 0; q < W; ++q) {
        nb[q] = f[q] & ~s[q];
        nb2[q] = w2 < 0 ? 0ull : (f2[q] & ~s2[q]);
    }
    bool first = false, first2 = false;
    const bool found = claim<W>(a, L, o, nb, first);
    const bool found2 = claim<W>(a, L, o2, nb2, first2);
    if (W > 1) {
        if (found) first = atomicMax(a.stamp + w, L.tag) < L.tag;
        if (found2) first2 = atomicMax(a.stamp + w2, L.tag) < L.tag;
    }
    if (first) qu.push(a, L, w);
    if (first2) qu.push(a, L, w2);
}

// Finalise F_{j-1} bits of one vertex: the level bit-planes (seen took them at
// discovery).  Only the thread that owns the vertex in this phase calls it.
template <int W>
__device__ __forceinline__ void finalise(const MsArgs &a, int32_t lev, size_t o, const u64 (&f)[W])
{
    const size_t pstride = (size_t)a.n * W;
    for (int b = 0; (lev >> b) != 0; ++b) {
        if (!((lev >> b) & 1)) continue;
        u64 *pp = a.plane + (size_t)b * pstride + o;
        u64 pv[W];
        ldw<W>(pp, pv);
#pragma unroll
        for (int q = 0; q < W; ++q) pv[q] |= f[q];
        stw<W>(pp, pv);
    }
}

// Sources with a non-empty F_{j-1}: OR of the finalised words, reduced per warp
// and per CTA (shared), then once per CTA into the phase's control slot.  Read
// at the start of phase j+1 it is a superset of the sources active in F_j,
// which is all the bottom-up early exit needs.
template <int W>
__device__ __forceinline__ void flush_active(const Lvl &L, const u64 (&act)[W])
{
#pragma unroll
    for (int q = 0; q < W; ++q) {
        const u64 r = warp_or_u64(FULL_MASK, act[q]);
        if (lane_id() == 0 && r) atomicOr(L.sact + q, r);
    }
}

// Finalise F_{j-1} in queue order and clear F_{j-2}.
template <int W, class G>
__device__ void td_update(const MsArgs &a, const Lvl &L)
{
    const long long rank = G::rank(), size = G::size();
    u64 act[W] = {};
    for (long long i = rank; i < L.qlen; i += size) {
        const int32_t v = __ldcg(L.qcur + i);
        const size_t o = (size_t)v * W;
        u64 f[W];
        ldw<W>(L.fcur + o, f);
        finalise<W>(a, L.lev, o, f);
#pragma unroll
        for (int q = 0; q < W; ++q) act[q] |= f[q];
    }
    flush_active<W>(L, act);
    for (long long i = rank; i < L.qlen_prev; i += size) zerow<W>(L.fprv + (size_t)__ldcg(L.qprev + i) * W);
}

template <int W>
__device__ __forceinline__ void load_front(const Lvl &L, int32_t v, u64 (&f)[W])
{
    ldw_l1<W>(L.fcur + (size_t)v * W, f);
}

// Frontier words of v restricted to the sources in fmask (shared) when MASKED.
template <int W, bool MASKED>
__device__ __forceinline__ void load_front_m(const Lvl &L, int32_t v, u64 (&f)[W], const u64 *fmask)
{
    ldw_l1<W>(L.fcur + (size_t)v * W, f);
    if (MASKED) {
#pragma unroll
        for (int q = 0; q < W; ++q) f[q] &= fmask[q];
    }
}

// LINEAR: thread per frontier vertex, serial adjacency (linear_with_atomics.cu:122-135).
template <int W, class G>
__device__ void gather_linear(const MsArgs &a, const Lvl &L)
{
    for (long long i = G::rank(); i < L.qlen; i += G::size()) {
        const int32_t v = __ldcg(L.qcur + i);
        u64 f[W];
        load_front<W>(L, v, f);
        const int32_t e1 = __ldg(a.R + v + 1);
        for (int32_t e = __ldg(a.R + v); e < e1; ++e) td_visit<W>(a, L, f, __ldg(a.C + e));
    }
}

// EDGE: every CSR entry every level, source vertex from the COO array
// (edge_parallel.cu:77-88); one sweep serves every source of the batch.
template <int W, class G>
__device__ void gather_edge(const MsArgs &a, const Lvl &L)
{
    for (long long e = G::rank(); e < a.m; e += G::size()) {
        const int32_t u = __ldg(a.F + e);
        u64 f[W];
        load_front<W>(L, u, f);
        if (anyw<W>(f)) td_visit<W>(a, L, f, __ldg(a.C + e));
    }
}

// SHUFFLE: warp per frontier vertex; warps take the next vertex from a shared
// counter when done (shuffle_based.cuh:192-223).
template <int W, class G>
__device__ void gather_shuffle(const MsArgs &a, const Lvl &L)
{
    const int lane = lane_id();
    const long long nw = G::size() >> 5;
    long long kq = G::rank() >> 5;
    while (kq < L.qlen) {
        const int32_t v = __ldcg(L.qcur + kq);
        u64 f[W];
        load_front<W>(L, v, f);
        const int32_t e1 = __ldg(a.R + v + 1);
        for (int32_t e = __ldg(a.R + v) + lane; e < e1; e += 32) td_visit<W>(a, L, f, __ldg(a.C + e));
        int nk = 0;
        if (lane == 0) nk = atomicAdd(&a.ctl->work[L.slot], 1);
        kq = nw + __shfl_sync(FULL_MASK, nk, 0);
    }
}

// Warp strip-mining: each lane holds one frontier vertex; the warp elects the
// highest lane with adjacency left (race_and_resolve) and gathers its list
// together (warp_based.cu:109-145).
template <int W>
__device__ __forceinline__ void warp_stripmine(const MsArgs &a, const Lvl &L, int32_t r, int32_t r_end, int32_t v)
{
    const int lane = lane_id();
    while (__any_sync(FULL_MASK, r < r_end)) {
        const int winner = race_and_resolve_warp(r < r_end);
        const int32_t rw = __shfl_sync(FULL_MASK, r, winner);
        const int32_t re = __shfl_sync(FULL_MASK, r_end, winner);
        const int32_t vw = __shfl_sync(FULL_MASK, v, winner);
        if (lane == winner) r = r_end;  // a lane cannot win twice
        u64 f[W];
        load_front<W>(L, vw, f);
        for (int32_t e = rw + lane; e < re; e += 32) td_visit<W>(a, L, f, __ldg(a.C + e));
    }
}

template <int W, class G>
__device__ void gather_warp(const MsArgs &a, const Lvl &L)
{
    const int lane = lane_id();
    const long long nw = G::size() >> 5;
    for (long long base = (G::rank() >> 5) * 32; base < L.qlen; base += nw * 32) {
        const long long i = base + lane;
        int32_t r = 0, r_end = 0, v = 0;
        if (i < L.qlen) {
            v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            r_end = __ldg(a.R + v + 1);
        }
        warp_stripmine<W>(a, L, r, r_end, v);
    }
}

// CTA_WARP: lists longer than 2048 are gathered by the whole CTA, one at a
// time (highest thread first), the rest by warp strip-mining (CTA_warp.cu:62-265).
template <int W, class G>
__device__ void gather_cta_warp(const MsArgs &a, const Lvl &L)
{
    __shared__ int s_winner;
    __shared__ int32_t s_r, s_re, s_v;
    const int BD = blockDim.x;
    for (long long base = (long long)G::blk() * BD; base < L.qlen; base += (long long)G::nblk() * BD) {
        const long long i = base + threadIdx.x;
        int32_t r = 0, r_end = 0, v = 0;
        if (i < L.qlen) {
            v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            r_end = __ldg(a.R + v + 1);
        }
        while (true) {
            if (threadIdx.x == 0) s_winner = -1;
            __syncthreads();
            if (r_end - r > CTA_DEGREE_THRESHOLD) atomicMax(&s_winner, (int)threadIdx.x);
            __syncthreads();
            const int wt = s_winner;
            if (wt < 0) break;
            if ((int)threadIdx.x == wt) {
                s_r = r;
                s_re = r_end;
                s_v = v;
                r = r_end;
            }
            __syncthreads();
            const int32_t re = s_re;
            u64 f[W];
            load_front<W>(L, s_v, f);
            for (int32_t e = s_r + threadIdx.x; e < re; e += BD) td_visit<W>(a, L, f, __ldg(a.C + e));
            __syncthreads();
        }
        warp_stripmine<W>(a, L, r, r_end, v);
        __syncthreads();
    }
}

// Block-wide exclusive scan of one int per thread (warp shuffles + shared).
__device__ __forceinline__ int block_exclusive_scan(int x, int *total, int *s_warp)
{
    const int lane = lane_id(), wid = warp_in_block(), nw = blockDim.x >> 5;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int t = lane < nw ? s_warp[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, ti, o);
            if (lane >= o) ti += y;
        }
        if (lane < nw) s_warp[lane] = ti - t;
        if (lane == 31) s_warp[32] = ti;
    }
    __syncthreads();
    const int res = s_warp[wid] + incl - x;
    *total = s_warp[32];
    __syncthreads();
    return res;
}

// SCAN: the CTA ranks the adjacency lists of blockDim frontier vertices with an
// exclusive scan, then threads take consecutive edge slots and find the owning
// vertex by binary search over the scanned offsets (scan_based.cu:107-149).
template <int W, class G>
__device__ void gather_scan(const MsArgs &a, const Lvl &L)
{
    __shared__ int s_off[MS_THREADS];
    __shared__ int32_t s_r[MS_THREADS];
    __shared__ int32_t s_v[MS_THREADS];
    __shared__ int s_warp[33];
    const int BD = blockDim.x;
    for (long long base = (long long)G::blk() * BD; base < L.qlen; base += (long long)G::nblk() * BD) {
        const long long i = base + threadIdx.x;
        int32_t r = 0, v = 0;
        int deg = 0;
        if (i < L.qlen) {
            v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            deg = __ldg(a.R + v + 1) - r;
        }
        int total;
        const int off = block_exclusive_scan(deg, &total, s_warp);
        s_off[threadIdx.x] = off;
        s_r[threadIdx.x] = r;
        s_v[threadIdx.x] = v;
        __syncthreads();
        for (int e = threadIdx.x; e < total; e += BD) {
            int lo = 0, hi = BD - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= e) lo = mid;
                else hi = mid - 1;
            }
            u64 f[W];
            load_front<W>(L, s_v[lo], f);
            td_visit<W>(a, L, f, __ldg(a.C + s_r[lo] + (e - s_off[lo])));
        }
        __syncthreads();
    }
}

// Merge-path gather (AUTO): the frontier's out-edges, ranked by the edge
// offsets reserved at append time, are cut into equal tasks, and the owner of
// every edge slot is found by binary search over those offsets (the
// load-balanced search of load_balanced_search.cu:123-192, grid-wide).
// Warp-wide 32-ary search: the largest idx in [lo, hi] with off[idx] <= e
// (off non-decreasing, off[lo] <= e).  Each round the lanes probe 32 evenly
// spaced positions and the ballot of "off <= e" (a prefix of the lanes)
// narrows the range 32-fold: three dependent loads for 10^4 owners instead of
// fourteen.  Every lane of the warp calls it and gets the result.
__device__ __forceinline__ int owner_search_warp(const int32_t *off, int lo, int hi, long long e)
{
    const int lane = lane_id();
    while (lo < hi) {
        const long long span = hi - lo;
        const int p = lo + (int)((span * (lane + 1) + 31) / 32);  // lo < p <= hi, p(31) = hi
        const unsigned le = __ballot_sync(FULL_MASK, (long long)__ldcg(off + p) <= e);
        const int cnt = __popc(le);
        const int plo = __shfl_sync(FULL_MASK, p, cnt > 0 ? cnt - 1 : 0);
        const int phi = __shfl_sync(FULL_MASK, p, cnt < 32 ? cnt : 31);
        if (cnt > 0) lo = plo;
        hi = cnt < 32 ? phi - 1 : hi;
    }
    return lo;
}

// A CTA takes a task of consecutive edge slots (MP_TASK, or fewer when the
// frontier is small so that every CTA gets work); two warps bracket the owners
// [k0, k1] by 32-ary search in global memory, the CTA stages the owners' ids,
// offsets and CSR starts in shared memory, and every thread then resolves its
// edge slots by binary search in shared memory.  Tasks whose bracket exceeds
// the shared capacity (many tiny lists) are walked owner by owner.
constexpr int MP_TASK = MS_THREADS * 8;
constexpr int MP_STAGE = 1024;
constexpr int MP_QUEUE = 2048;  // discovered-vertex queue after the staging
static_assert(3 * MP_STAGE * 4 + MP_QUEUE * 4 <= MS_SMEM_BYTES, "merge-path staging exceeds the shared buffer");

template <int W, class G, bool MASKED = false>
__device__ void gather_mp(const MsArgs &a, const Lvl &L, const u64 *fmask = nullptr)
{
    int32_t *s_off = reinterpret_cast<int32_t *>(ms_smem());
    int32_t *s_v = s_off + MP_STAGE;
    int32_t *s_r = s_v + MP_STAGE;
    __shared__ int s_k[2];
    const long long E = L.qedges;
    if (E == 0) return;
    const CtaQ cq{s_r + MP_STAGE, cq_count(), MP_QUEUE};
    const long long per_blk = (E + G::nblk() - 1) / G::nblk();
    const long long task = min((long long)MP_TASK, max(32ll, (per_blk + 31) & ~31ll));
    const long long ntask = (E + task - 1) / task;
    for (long long t = G::blk(); t < ntask; t += G::nblk()) {
        const long long e0 = t * task;
        const long long e1 = min(E, e0 + task);
        const int warp = threadIdx.x >> 5;
        if (warp < 2) {
            const int k = owner_search_warp(L.qcur_off, 0, L.qlen - 1, warp == 0 ? e0 : e1 - 1);
            if (lane_id() == 0) s_k[warp] = k;
        }
        __syncthreads();
        const int k0 = s_k[0], nk = s_k[1] - k0 + 1;
        if (nk <= MP_STAGE) {
            for (int i = threadIdx.x; i < nk; i += blockDim.x) {
                const int32_t v = __ldcg(L.qcur + k0 + i);
                s_v[i] = v;
                s_off[i] = __ldcg(L.qcur_off + k0 + i);
                s_r[i] = __ldg(a.R + v);
            }
            __syncthreads();
            // two edge slots per trip: both visits' loads are issued before either claims
            for (long long e = e0 + threadIdx.x; e < e1; e += 2 * (long long)blockDim.x) {
                const long long e2 = e + blockDim.x;
                int lo = 0, hi = nk - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if ((long long)s_off[mid] <= e) lo = mid;
                    else hi = mid - 1;
                }
                int lo2 = lo, hi2 = nk - 1;
                while (lo2 < hi2) {
                    const int mid = (lo2 + hi2 + 1) >> 1;
                    if ((long long)s_off[mid] <= e2) lo2 = mid;
                    else hi2 = mid - 1;
                }
                const bool has2 = e2 < e1;
                u64 f[W];
                load_front_m<W, MASKED>(L, s_v[lo], f, fmask);
                const int32_t w = __ldg(a.C + s_r[lo] + (int32_t)(e - s_off[lo]));
                const int32_t w2 = has2 ? __ldg(a.C + s_r[lo2] + (int32_t)(e2 - s_off[lo2])) : -1;
                if (!has2 || lo2 == lo) {
                    // both slots in one adjacency list (the common case: frontier
                    // hubs): one frontier word group, both visits' loads together
                    td_visit2<W>(a, L, f, w, f, w2, cq);
                } else {
                    td_visit<W>(a, L, f, w, cq);
                    u64 f2[W];
                    load_front_m<W, MASKED>(L, s_v[lo2], f2, fmask);
                    td_visit<W>(a, L, f2, w2, cq);
                }
            }
        } else {
            for (int i = threadIdx.x; i < nk; i += blockDim.x) {
                const int32_t v = __ldcg(L.qcur + k0 + i);
                const long long off = __ldcg(L.qcur_off + k0 + i);
                const int32_t r = __ldg(a.R + v), deg = __ldg(a.R + v + 1) - r;
                const long long lo_e = max(off, e0), hi_e = min(off + deg, e1);
                if (lo_e >= hi_e) continue;
                u64 f[W];
                load_front_m<W, MASKED>(L, v, f, fmask);
                for (long long e = lo_e; e < hi_e; ++e) td_visit<W>(a, L, f, __ldg(a.C + r + (int32_t)(e - off)), cq);
            }
        }
        __syncthreads();
        if (*cq.n > cq.cap / 2) cta_flush(a, L, cq);
    }
    __syncthreads();
    if (*cq.n > 0) cta_flush(a, L, cq);
}

// Bottom-up level, in up to three grid-synchronised parts.
//  A  Every vertex with in-edges (the light, mid, wide and heavy class lists;
//     vertices without in-edges are never discovered after level 0) finalises
//     its F_{j-1} bits and clears its F_{j-2} words.  The OR of the F_{j-1}
//     words a CTA finalised marks the sources it saw; the count of CTAs that saw
//     a source is its coverage (a source with a frontier of a few dozen vertices
//     is seen by a few dozen CTAs, a source whose search ended by none).
//  B  Sources seen by at least rare_frac of the CTAs are searched bottom-up:
//     each vertex still missing one ORs its in-neighbours' F_{j-1} words, the
//     light, mid and wide passes in at most two rounds of loads issued together
//     (no loop: lanes of a warp never diverge over trip counts), the heavy pass
//     stepping through the in-edges; mid, wide and heavy stop once every
//     missing source is found.  Frontier vertices holding a rare source (seen,
//     but by fewer CTAs) are listed.
//  C  Only with rare sources: the listed vertices are expanded top-down, with
//     their rare bits only, by the merge-path gather.  Searched bottom-up, a
//     rare source would keep every vertex it has not reached scanning all its
//     in-edges, since the early exit waits for every missing source.
template <int W>
__device__ __forceinline__ bool covers(const u64 (&acc)[W], const u64 (&need)[W])
{
    bool ok = true;
#pragma unroll
    for (int q = 0; q < W; ++q) ok &= (acc[q] & need[q]) == need[q];
    return ok;
}

template <int W>
__device__ __forceinline__ void or_front(const Lvl &L, int32_t v, u64 (&acc)[W])
{
    u64 x[W];
    ldw_l1<W>(L.fcur + (size_t)v * W, x);
#pragma unroll
    for (int q = 0; q < W; ++q) acc[q] |= x[q];
}

// Part A for one vertex.
template <int W>
__device__ __forceinline__ void bu_finalise(const MsArgs &a, const Lvl &L, int32_t w, u64 (&act)[W])
{
    const size_t o = (size_t)w * W;
    u64 f[W];
    ldw<W>(L.fcur + o, f);
    if (anyw<W>(f)) {
        finalise<W>(a, L.lev, o, f);
#pragma unroll
        for (int q = 0; q < W; ++q) act[q] |= f[q];
    }
    zerow<W>(L.fprv + o);
}

template <int W, class G>
__device__ void bu_finalise_all(const MsArgs &a, const Lvl &L)
{
    u64 act[W] = {};
    const long long rank = G::rank(), size = G::size();
    for (long long i = rank; i < a.nlight; i += size) bu_finalise<W>(a, L, __ldg(a.light + i), act);
    for (long long i = rank; i < a.nmid; i += size) bu_finalise<W>(a, L, __ldg(a.mid + i), act);
    for (long long i = rank; i < a.nwide; i += size) bu_finalise<W>(a, L, __ldg(a.wide + i), act);
    for (long long i = rank; i < a.nheavy; i += size) bu_finalise<W>(a, L, __ldg(a.heavy + i), act);
    flush_active<W>(L, act);
}

// Sources of part B a vertex still misses (seen holds F_{j-1} after part A).
template <int W>
__device__ __forceinline__ void bu_need(const MsArgs &a, const Lvl &L, int32_t w, u64 (&need)[W])
{
    u64 s[W];
    ldw<W>(a.seen + (size_t)w * W, s);
#pragma unroll
    for (int q = 0; q < W; ++q) need[q] = L.active[q] & ~s[q];
}

template <int W>
__device__ __forceinline__ void bu_found(const MsArgs &a, const Lvl &L, const CtaQ &cq, int32_t w,
                                         const u64 (&acc)[W], const u64 (&need)[W])
{
    u64 nb[W];
#pragma unroll
    for (int q = 0; q < W; ++q) nb[q] = acc[q] & need[q];
    if (!anyw<W>(nb)) return;
    stw<W>(L.fnxt + (size_t)w * W, nb);  // the vertex's only writer in part B
#pragma unroll
    for (int q = 0; q < W; ++q)
        if (nb[q]) red_or(a.seen + (size_t)w * W + q, nb[q]);
    if (W > 1 && L.rare_td) a.stamp[w] = L.tag;  // part C's visits must not append w again
    cq.push(a, L, w);
}

// Vertices of a class per warp step: the class spread over every warp, at most
// one per lane.  Each lane reads the missing set of one vertex; the warp then
// scans only the vertices that still miss a source.
__device__ __forceinline__ long long class_chunk(long long count, long long nwarps)
{
    return max(1ll, min(32ll, (count + nwarps - 1) / nwarps));
}

template <int W>
__device__ __forceinline__ void shfl_words(const u64 (&x)[W], u64 (&y)[W], int src)
{
#pragma unroll
    for (int q = 0; q < W; ++q) y[q] = __shfl_sync(FULL_MASK, x[q], src);
}

// Light: one thread per vertex, up to BU_LIGHT_DEGREE loads in flight.
template <int W, class G>
__device__ void bu_light(const MsArgs &a, const Lvl &L, const CtaQ &cq)
{
    const long long size = G::size();
    for (long long i = G::rank(); i < a.nlight; i += size) {
        const int32_t w = __ldg(a.light + i);
        u64 need[W];
        bu_need<W>(a, L, w, need);
        if (!anyw<W>(need)) continue;
        const int32_t e0 = __ldg(a.RT + w), e1 = __ldg(a.RT + w + 1);
        int32_t c[BU_LIGHT_DEGREE];
#pragma unroll
        for (int t = 0; t < BU_LIGHT_DEGREE; ++t) c[t] = e0 + t < e1 ? __ldg(a.CT + e0 + t) : -1;
        u64 acc[W] = {};
#pragma unroll
        for (int t = 0; t < BU_LIGHT_DEGREE; ++t)
            if (c[t] >= 0) or_front<W>(L, c[t], acc);
        bu_found<W>(a, L, cq, w, acc, need);
    }
}

// Mid: eight lanes per needy vertex (four at a time).  First the eight
// highest-degree in-neighbours (one load per lane), which at the later levels
// usually cover every missing source; then, only where they do not, the rest
// (up to three more loads per lane, in flight together).  The group's words
// are OR-ed with xor shuffles inside the group.
template <int W>
__device__ __forceinline__ void group8_or(u64 (&x)[W])
{
#pragma unroll
    for (int q = 0; q < W; ++q) {
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) x[q] |= __shfl_xor_sync(FULL_MASK, x[q], off);
    }
}

template <int W, class G>
__device__ void bu_mid(const MsArgs &a, const Lvl &L, const CtaQ &cq)
{
    static_assert(BU_LIGHT_DEGREE >= 7, "mid class: the first round gives every lane an in-edge");
    static_assert(BU_MID_DEGREE <= 8 * 4, "mid class: at most four in-edges per lane");
    const int lane = lane_id(), sub = lane & 7, grp = lane >> 3;
    const long long nw = G::size() >> 5, chunk = class_chunk(a.nmid, nw);
    for (long long base = (G::rank() >> 5) * chunk; base < a.nmid; base += nw * chunk) {  // warp-uniform
        const bool valid = lane < chunk && base + lane < a.nmid;
        const int32_t mine = valid ? __ldg(a.mid + base + lane) : 0;
        u64 need_l[W] = {};
        if (valid) bu_need<W>(a, L, mine, need_l);
        unsigned todo = __ballot_sync(FULL_MASK, anyw<W>(need_l));
        while (todo) {  // warp-uniform
            unsigned t = todo;
            for (int k = 0; k < grp && t; ++k) t &= t - 1;  // this group's needy lane: the grp-th set bit
            const int src = t ? __ffs(t) - 1 : 0;
            const bool has = t != 0;
            for (int k = 0; k < 4 && todo; ++k) todo &= todo - 1;
            const int32_t w = __shfl_sync(FULL_MASK, mine, src);
            u64 need[W];
            shfl_words<W>(need_l, need, src);
            u64 acc[W] = {};
            int32_t e0 = 0, e1 = 0;
            if (has) {
                e0 = __ldg(a.RT + w);
                e1 = __ldg(a.RT + w + 1);
                or_front<W>(L, __ldg(a.CT + e0 + sub), acc);  // in-degree > 8: every lane has one
            }
            group8_or<W>(acc);
            const bool more = has && !covers<W>(acc, need);
            if (__any_sync(FULL_MASK, more)) {
                u64 x[W] = {};
                if (more) {
                    int32_t c[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        c[r] = e0 + 8 * (r + 1) + sub < e1 ? __ldg(a.CT + e0 + 8 * (r + 1) + sub) : -1;
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        if (c[r] >= 0) or_front<W>(L, c[r], x);
                }
                group8_or<W>(x);
#pragma unroll
                for (int q = 0; q < W; ++q) acc[q] |= x[q];
            }
            if (has && sub == 0) bu_found<W>(a, L, cq, w, acc, need);
        }
    }
}

// Wide: a warp per needy vertex: the 32 highest-degree in-neighbours first,
// then, only if they leave a missing source uncovered, the rest (up to three
// more loads per lane, in flight together).
template <int W, class G>
__device__ void bu_wide(const MsArgs &a, const Lvl &L, const CtaQ &cq)
{
    static_assert(BU_MID_DEGREE >= 31, "wide class: the first round gives every lane an in-edge");
    static_assert(BU_HEAVY_DEGREE <= 32 * 4, "wide class: at most four in-edges per lane");
    const int lane = lane_id();
    const long long nw = G::size() >> 5, chunk = class_chunk(a.nwide, nw);
    for (long long base = (G::rank() >> 5) * chunk; base < a.nwide; base += nw * chunk) {  // warp-uniform
        const bool valid = lane < chunk && base + lane < a.nwide;
        const int32_t mine = valid ? __ldg(a.wide + base + lane) : 0;
        u64 need_l[W] = {};
        if (valid) bu_need<W>(a, L, mine, need_l);
        unsigned todo = __ballot_sync(FULL_MASK, anyw<W>(need_l));
        while (todo) {  // warp-uniform
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int32_t w = __shfl_sync(FULL_MASK, mine, src);
            u64 need[W];
            shfl_words<W>(need_l, need, src);
            const int32_t e0 = __ldg(a.RT + w), e1 = __ldg(a.RT + w + 1);
            u64 acc[W] = {};
            or_front<W>(L, __ldg(a.CT + e0 + lane), acc);  // in-degree > 32: every lane has one
#pragma unroll
            for (int q = 0; q < W; ++q) acc[q] = warp_or_u64(FULL_MASK, acc[q]);
            if (!covers<W>(acc, need)) {
                int32_t c[3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    c[r] = e0 + 32 * (r + 1) + lane < e1 ? __ldg(a.CT + e0 + 32 * (r + 1) + lane) : -1;
                u64 x[W] = {};
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    if (c[r] >= 0) or_front<W>(L, c[r], x);
#pragma unroll
                for (int q = 0; q < W; ++q) acc[q] |= warp_or_u64(FULL_MASK, x[q]);
            }
            if (lane == 0) bu_found<W>(a, L, cq, w, acc, need);
        }
    }
}

// Heavy (in-degree > BU_HEAVY_DEGREE): a warp per needy vertex ORs 128
// in-neighbours per step (four loads in flight per lane), the 32
// highest-degree ones first, and stops once every missing source is found.
template <int W, class G>
__device__ void bu_heavy(const MsArgs &a, const Lvl &L, const CtaQ &cq)
{
    const int lane = lane_id();
    const long long nw = G::size() >> 5, chunk = class_chunk(a.nheavy, nw);
    for (long long base = (G::rank() >> 5) * chunk; base < a.nheavy; base += nw * chunk) {  // warp-uniform
        const bool valid = lane < chunk && base + lane < a.nheavy;
        const int32_t mine = valid ? __ldg(a.heavy + base + lane) : 0;
        u64 need_l[W] = {};
        if (valid) bu_need<W>(a, L, mine, need_l);
        unsigned todo = __ballot_sync(FULL_MASK, anyw<W>(need_l));
        while (todo) {  // warp-uniform
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int32_t w = __shfl_sync(FULL_MASK, mine, src);
            u64 need[W];
            shfl_words<W>(need_l, need, src);
            const int32_t e0 = __ldg(a.RT + w), e1 = __ldg(a.RT + w + 1);
            u64 acc[W] = {};
            {  // first step: the 32 highest-degree in-neighbours
                u64 x[W] = {};
                or_front<W>(L, __ldg(a.CT + e0 + lane), x);  // in-degree > 128
#pragma unroll
                for (int q = 0; q < W; ++q) acc[q] |= warp_or_u64(FULL_MASK, x[q]);
            }
            for (int32_t eb = e0 + 32; eb < e1 && !covers<W>(acc, need); eb += 128) {  // then 128 per step
                u64 x[W] = {};
                int32_t c[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) c[r] = eb + 32 * r + lane < e1 ? __ldg(a.CT + eb + 32 * r + lane) : -1;
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (c[r] >= 0) or_front<W>(L, c[r], x);
#pragma unroll
                for (int q = 0; q < W; ++q) acc[q] |= warp_or_u64(FULL_MASK, x[q]);
            }
            if (lane == 0) bu_found<W>(a, L, cq, w, acc, need);
        }
    }
}

// Part B's list of the frontier vertices that hold a rare source, with their
// out-edge offsets, in F_{j-2}'s queue arrays (free during a bottom-up level).
template <int W, class G>
__device__ void bu_rare_list(const MsArgs &a, const Lvl &L, const u64 *s_rare)
{
    u64 r[W];
#pragma unroll
    for (int q = 0; q < W; ++q) r[q] = s_rare[q];
    for (long long i = G::rank(); i < L.qlen; i += G::size()) {
        const int32_t u = __ldcg(L.qcur + i);
        u64 f[W];
        ldw<W>(L.fcur + (size_t)u * W, f);
        bool any = false;
#pragma unroll
        for (int q = 0; q < W; ++q) any |= (f[q] & r[q]) != 0;
        if (any) append_to(a, &a.ctl->rpack, a.q[L.prv], a.qoff[L.prv], u);
    }
}

// Distance rows of one batch from seen and the level bit-planes.
//
// Fast path (levels < 256, 16-byte aligned rows): a CTA takes a tile of
// blockDim / W consecutive vertices and all W words of each, thread (vertex,
// word) reading its seen and plane words coalesced (consecutive threads,
// consecutive words); the next tile's words are loaded while this one is
// written.  Each thread decodes 16 rows of its word per round into a shared
// [16 W][blockDim / W] tile (columns rotated by word so a warp's stores hit 32
// distinct banks), and the CTA writes each row's segment (512 bytes for W = 4)
// with contiguous int4 stores.  Otherwise lanes hold consecutive vertices and
// store one int each.
constexpr int WD_ROWS = 16;
static_assert(WD_ROWS * MS_THREADS * 4 <= MS_SMEM_BYTES, "distance tile exceeds the shared buffer");

// Transpose of an 8x8 bit matrix held row-major in a u64 (bit 8r+c -> bit
// 8c+r): three rounds of masked swaps of the off-diagonal blocks, the method of
// Warren, "Hacker's Delight", section 7-3.
__device__ __forceinline__ u64 transpose8x8(u64 x)
{
    u64 t;
    t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
    x = x ^ t ^ (t << 7);
    t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
    x = x ^ t ^ (t << 14);
    t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
    x = x ^ t ^ (t << 28);
    return x;
}

// 8x8 bit-matrix transpose on two 32-bit words: rows 0-3 are the bytes of x,
// rows 4-7 those of y; afterwards byte c (of x for c < 4, of y for c >= 4)
// holds column c.  The three stages of transpose8x8, the first two inside
// each word and the third exchanging nibbles between the words.
__device__ __forceinline__ void transpose8x8_32(uint32_t &x, uint32_t &y)
{
    uint32_t t;
    t = (x ^ (x >> 7)) & 0x00AA00AAu;
    x ^= t ^ (t << 7);
    t = (y ^ (y >> 7)) & 0x00AA00AAu;
    y ^= t ^ (t << 7);
    t = (x ^ (x >> 14)) & 0x0000CCCCu;
    x ^= t ^ (t << 14);
    t = (y ^ (y >> 14)) & 0x0000CCCCu;
    y ^= t ^ (t << 14);
    t = (x ^ (y << 4)) & 0xF0F0F0F0u;
    x ^= t;
    y ^= t >> 4;
}

// Distance rows of a batch whose levels fit in four planes (levels < 16, the
// common case).  Tiles of 256 / W consecutive vertices (all W words each) go
// through a double-buffered shared byte tile: while the upper half of the CTA
// writes tile i-1 to the rows, the lower half decodes tile i, so the row
// stores stream without waiting for the decode.  A decoding thread (vertex,
// word q) reads its seen and plane words coalesced (the next tile's words are
// loaded while this one is decoded); for each group of eight sources it
// gathers byte g of the four planes into x and byte g of ~seen, four times,
// into y, and after the bit transpose byte c holds the source's level in the
// low nibble and 0xF in the high nibble if the source never reached the
// vertex.  The bytes fill a [64 W rows][256 / W] tile (columns rotated by word
// so a warp's stores hit distinct banks); the writing half widens four bytes
// at a time (unreached -> INT_MAX) into int4 streaming stores.
template <int W, class G>
__device__ void write_distances_nibble(const MsArgs &a, int row0, int nb)
{
    constexpr int HALF = MS_THREADS / 2;
    constexpr int TV = HALF / W;  // vertices per tile
    constexpr int ROWS = 64 * W;
    constexpr int TILE = ROWS * TV;
    constexpr int SWZ = 32 / W;   // byte rotation per word
    static_assert(2 * TILE <= MS_SMEM_BYTES, "byte tiles exceed the shared buffer");
    // Tiles are taken from a counter (ctl->wo_next) rather than by a fixed
    // stride, so that CTAs whose stores drain faster take more of them (a fixed
    // split left a fifth of the CTA time idle).  Tile of iteration i: s_tile[i & 3],
    // taken by thread 0 two iterations ahead (the decoders prefetch the next one).
    __shared__ int s_tile[4];
    unsigned char *tiles = ms_smem();
    const size_t pstride = (size_t)a.n * W;
    const bool decoder = threadIdx.x < HALF;
    const int tid = decoder ? threadIdx.x : threadIdx.x - HALF;
    const int q = tid % W, vl = tid / W;
    const int nq = (nb + 63) / 64;
    const int ntile = (int)(((long long)a.n + TV - 1) / TV);
    const int col = (vl + SWZ * q) % TV;
    int *next = &a.ctl->wo_next;
    auto load = [&](int t, u64 &s, u64 (&pl)[4]) {
        const int32_t v = t * TV + vl;
        const bool valid = decoder && t < ntile && v < a.n && q < nq;
        const size_t o = (size_t)v * W + q;
        s = valid ? __ldcs(a.seen + o) : 0ull;
#pragma unroll
        for (int b = 0; b < 4; ++b) pl[b] = (b < a.nplanes && valid) ? __ldcs(a.plane + b * pstride + o) : 0ull;
    };
    if (threadIdx.x == 0) {
        s_tile[0] = atomicAdd(next, 1);
        s_tile[1] = atomicAdd(next, 1);
    }
    __syncthreads();
    u64 s, pl[4];
    load(s_tile[0], s, pl);
    for (int i = 0;; ++i) {  // block-uniform
        const int td = s_tile[i & 3], ts = i > 0 ? s_tile[(i - 1) & 3] : ntile, tn = s_tile[(i + 1) & 3];
        if (td >= ntile && ts >= ntile) break;
        if (threadIdx.x == 0) s_tile[(i + 2) & 3] = td < ntile ? atomicAdd(next, 1) : ntile;
        if (decoder) {
            if (td < ntile) {
                u64 s_n, pl_n[4];
                load(tn, s_n, pl_n);
                unsigned char *tile = tiles + (i & 1) * TILE;
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    const int bi = g & 3;
                    const uint32_t h0 = (uint32_t)(pl[0] >> (g < 4 ? 0 : 32)), h1 = (uint32_t)(pl[1] >> (g < 4 ? 0 : 32));
                    const uint32_t h2 = (uint32_t)(pl[2] >> (g < 4 ? 0 : 32)), h3 = (uint32_t)(pl[3] >> (g < 4 ? 0 : 32));
                    const uint32_t ns = ~(uint32_t)(s >> (g < 4 ? 0 : 32));
                    const uint32_t t01 = __byte_perm(h0, h1, bi | ((4 + bi) << 4));
                    const uint32_t t23 = __byte_perm(h2, h3, bi | ((4 + bi) << 4));
                    uint32_t x = __byte_perm(t01, t23, 0x5410);
                    uint32_t y = __byte_perm(ns, 0u, bi * 0x1111);
                    transpose8x8_32(x, y);
                    unsigned char *dst = tile + (64 * q + 8 * g) * TV + col;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        dst[c * TV] = (unsigned char)(x >> (8 * c));
                        dst[(c + 4) * TV] = (unsigned char)(y >> (8 * c));
                    }
                }
                s = s_n;
#pragma unroll
                for (int b = 0; b < 4; ++b) pl[b] = pl_n[b];
            }
        } else if (ts < ntile) {
            const unsigned char *tile = tiles + ((i - 1) & 1) * TILE;
            const int32_t vbase = ts * TV;
            const int nv = min(TV, a.n - vbase), nv4 = nv >> 2;
            for (int k = tid; k < ROWS * (TV / 4); k += HALF) {
                const int row = k / (TV / 4), c4 = k - row * (TV / 4);
                if (row >= nb) continue;
                const int sh = SWZ * (row >> 6);
                const unsigned char *trow = tile + row * TV;
                int32_t *drow = a.dist + (int64_t)(row0 + row) * a.ld + vbase;
                if (c4 < nv4) {
                    uint32_t w4 = *reinterpret_cast<const uint32_t *>(trow + (4 * c4 + sh) % TV);
                    w4 |= (w4 >> 4) & 0x0F0F0F0Fu;  // unreached bytes 0xF0 -> 0xFF
                    int4 o;
                    o.x = (int32_t)(int8_t)(w4) & INT_MAX;
                    o.y = (int32_t)(int8_t)(w4 >> 8) & INT_MAX;
                    o.z = (int32_t)(int8_t)(w4 >> 16) & INT_MAX;
                    o.w = (int32_t)(int8_t)(w4 >> 24) & INT_MAX;
                    // streaming store: the rows are not read again by this kernel
                    __stcs(reinterpret_cast<int4 *>(drow) + c4, o);
                } else if (c4 == nv4) {
                    for (int x = 4 * c4; x < nv; ++x) {
                        const unsigned b = trow[(x + sh) % TV];
                        drow[x] = (b & 0xF0u) ? INT_MAX : (int32_t)b;
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <int W, class G>
__device__ void write_distances(const MsArgs &a, int row0, int nb, int nplanes_used)
{
    if (nplanes_used <= 4 && (a.ld & 3) == 0 && (((uintptr_t)a.dist) & 15) == 0 && blockDim.x == MS_THREADS) {
        write_distances_nibble<W, G>(a, row0, nb);
        return;
    }
    if (nplanes_used <= 8 && (a.ld & 3) == 0 && (((uintptr_t)a.dist) & 15) == 0 && blockDim.x == MS_THREADS) {
        constexpr int TV = MS_THREADS / W;  // vertices per tile
        constexpr int SWZ = 32 / W;         // column rotation per word
        int32_t *tile = reinterpret_cast<int32_t *>(ms_smem());  // [WD_ROWS * W][TV]
        const size_t pstride = (size_t)a.n * W;
        const int q = threadIdx.x % W, vl = threadIdx.x / W;
        const int nq = (nb + 63) / 64;
        const long long ntile = ((long long)a.n + TV - 1) / TV;
        const int col = (vl + SWZ * q) % TV;
        auto load = [&](long long t, u64 &s, u64 (&pl)[8]) {
            const int32_t v = (int32_t)(t * TV) + vl;
            const bool valid = t < ntile && v < a.n && q < nq;
            const size_t o = (size_t)v * W + q;
            s = valid ? __ldcs(a.seen + o) : 0ull;
#pragma unroll
            for (int b = 0; b < 8; ++b) pl[b] = (b < nplanes_used && valid) ? __ldcs(a.plane + b * pstride + o) : 0ull;
        };
        u64 s, pl[8];
        load(G::blk(), s, pl);
        for (long long t = G::blk(); t < ntile; t += G::nblk()) {
            u64 s_n, pl_n[8];
            load(t + G::nblk(), s_n, pl_n);  // next tile's words in flight during this one
            const int32_t vbase = (int32_t)(t * TV);
            const int nv = min(TV, a.n - vbase);
            for (int r0 = 0; r0 < 64; r0 += WD_ROWS) {
#pragma unroll
                for (int h = 0; h < WD_ROWS / 8; ++h) {
                    // sources 8g..8g+7 of word q: byte b of M = byte g of plane b; after
                    // an 8x8 bit-matrix transpose byte c of M is the level of source 8g+c
                    const int g8 = (r0 >> 3) + h;
                    u64 M = 0;
#pragma unroll
                    for (int b = 0; b < 8; ++b) M |= ((pl[b] >> (8 * g8)) & 0xFFull) << (8 * b);
                    M = transpose8x8(M);
                    const unsigned sb = (unsigned)(s >> (8 * g8)) & 0xFFu;
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        tile[(WD_ROWS * q + 8 * h + c) * TV + col] =
                            ((sb >> c) & 1u) ? (int32_t)((M >> (8 * c)) & 0xFFull) : INT_MAX;
                }
                __syncthreads();
                const int nv4 = nv >> 2;
                for (int k = threadIdx.x; k < WD_ROWS * W * (TV / 4); k += MS_THREADS) {
                    const int rr = k / (TV / 4), c4 = k - rr * (TV / 4);
                    const int wq = rr / WD_ROWS, row = 64 * wq + r0 + (rr - wq * WD_ROWS);
                    if (row >= nb) continue;
                    int32_t *drow = a.dist + (int64_t)(row0 + row) * a.ld + vbase;
                    const int32_t *trow = tile + rr * TV;
                    const int sh = SWZ * wq;
                    if (c4 < nv4) {
                        // streaming store: the rows are not read again by this kernel
                        __stcs(reinterpret_cast<int4 *>(drow) + c4,
                               *reinterpret_cast<const int4 *>(trow + (4 * c4 + sh) % TV));
                    } else if (c4 == nv4) {
                        for (int x = 4 * c4; x < nv; ++x) drow[x] = trow[(x + sh) % TV];
                    }
                }
                __syncthreads();
            }
            s = s_n;
#pragma unroll
            for (int b = 0; b < 8; ++b) pl[b] = pl_n[b];
        }
        return;
    }
    const int lane = lane_id();
    const long long size = G::size();
    const size_t pstride = (size_t)a.n * W;
    for (long long base = G::rank() - lane; base < a.n; base += size) {
        const int32_t v = (int32_t)(base + lane);
        const bool valid = v < a.n;
        for (int q = 0; q < W && 64 * q < nb; ++q) {
            const size_t o = (size_t)v * W + q;
            const u64 s = valid ? __ldcg(a.seen + o) : 0ull;
            const int rows = min(64, nb - 64 * q);
            int32_t *drow = a.dist + (int64_t)(row0 + 64 * q) * a.ld + v;
            if (nplanes_used <= 8) {  // levels < 256: all planes in registers
                u64 pl[8];
#pragma unroll
                for (int b = 0; b < 8; ++b)
                    pl[b] = (b < nplanes_used && valid) ? __ldcg(a.plane + b * pstride + o) : 0ull;
                for (int i = 0; i < rows; ++i) {
                    int32_t lvl = 0;
#pragma unroll
                    for (int b = 0; b < 8; ++b) lvl |= (int32_t)((pl[b] >> i) & 1ull) << b;
                    if (valid) drow[(int64_t)i * a.ld] = ((s >> i) & 1ull) ? lvl : INT_MAX;
                }
            } else {  // deep searches: 8 rows at a time, planes streamed
                for (int i0 = 0; i0 < rows; i0 += 8) {
                    int32_t lvl[8] = {};
                    for (int b = 0; b < nplanes_used; ++b) {
                        const u64 w8 = valid ? (__ldcg(a.plane + b * pstride + o) >> i0) : 0ull;
#pragma unroll
                        for (int t = 0; t < 8; ++t) lvl[t] |= (int32_t)((w8 >> t) & 1ull) << b;
                    }
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                        if (valid && i0 + t < rows)
                            drow[(int64_t)(i0 + t) * a.ld] = ((s >> (i0 + t)) & 1ull) ? lvl[t] : INT_MAX;
                }
            }
        }
    }
}

// Reachable-vertex count of every source of the batch (the source itself
// included, reachability.cu:11-33), from seen at the end of the batch: a warp
// takes 32 vertices, and for each of a word's 64 sources one ballot over the
// lanes' seen words counts the 32 vertices at once; lane b keeps sources b and
// b + 32.  Per-CTA sums in shared memory, one global atomic per source per CTA.
template <int W, class G>
__device__ void count_reached(const MsArgs &a, int row0, int nb)
{
    __shared__ unsigned long long s_cnt[64 * MAXW];
    for (int i = threadIdx.x; i < 64 * W; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
    const int lane = lane_id();
    const long long nw = G::size() >> 5;
    for (int q = 0; q < W; ++q) {  // one source word at a time: few live registers
        unsigned c0 = 0, c1 = 0;
        for (long long base = (G::rank() >> 5) * 32; base < a.n; base += nw * 32) {  // warp-uniform
            const long long v = base + lane;
            const u64 sw = v < a.n ? __ldcg(a.seen + (size_t)v * W + q) : 0ull;
            for (int b = 0; b < 32; ++b) {
                const unsigned lo = __ballot_sync(FULL_MASK, (sw >> b) & 1ull);
                const unsigned hi = __ballot_sync(FULL_MASK, (sw >> (b + 32)) & 1ull);
                if (lane == b) {
                    c0 += __popc(lo);
                    c1 += __popc(hi);
                }
            }
        }
        if (c0) atomicAdd(&s_cnt[64 * q + lane], (unsigned long long)c0);
        if (c1) atomicAdd(&s_cnt[64 * q + 32 + lane], (unsigned long long)c1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (s_cnt[i]) atomicAdd(a.reach + row0 + i, s_cnt[i]);
    __syncthreads();
}

// The batched search of one launch (G = the whole grid) or of one item of a
// work-queue launch (G = the item's CTA group, whose barrier counter lives in the
// item's control block).  epoch counts this CTA's barriers on that counter.
template <int VARIANT, int W, class G>
__device__ __forceinline__ void ms_search(const MsArgs &a, unsigned &epoch)
{
    __shared__ u64 s_act[MAXW];
    // copy of the control block taken by each CTA's thread 0 after every barrier
    __shared__ MsCtl s_ctl;
    __shared__ u64 s_rare[MAXW];  // bottom-up level: rare sources expanded top-down
    __shared__ u64 s_excl[MAXW];  // ... and the sources it searches bottom-up
    int ev_idx = 0;
    MsCtl *ctl = a.ctl;
    // slot: the timeline entry whose phase the barrier ends (or is inside of); each
    // CTA adds its wait there (profiling hook: idle CTA time per phase)
    auto barrier = [&](int slot) {
        const u64 t_arrive = threadIdx.x == 0 ? global_timer_ns() : 0ull;
        const bool ok = grid_barrier(&ctl->bar, &ctl->err, epoch, a.wait_ns, reinterpret_cast<const u64 *>(ctl),
                                     reinterpret_cast<u64 *>(&s_ctl), (int)(sizeof(MsCtl) / sizeof(u64)),
                                     (unsigned)G::nblk());
        if (threadIdx.x == 0 && slot < TIMELINE_MAX)
            atomicAdd(&reinterpret_cast<MsEvent *>(reinterpret_cast<char *>(ctl) + 256)[slot].idle_ns,
                      global_timer_ns() - t_arrive);
        return ok;
    };
    const long long rank = G::rank(), size = G::size();
    const size_t pstride = (size_t)a.n * W;
    if (threadIdx.x < MAXW) s_act[threadIdx.x] = 0;
    if (threadIdx.x == 0) *cq_count() = 0;
    if (rank == 0) ctl->nblocks = G::nblk();
    const int bsz = 64 * W;
    const int nbatch = (a.k + bsz - 1) / bsz;
    // First-discovery stamps carry level tags that grow across the launch's batches
    // (a batch's tags start above every tag of the batches before it), so the
    // stamps are cleared once per launch, not per batch.
    int tag_base = 0;
    for (int b = 0; b < nbatch; ++b) {
        const int row0 = b * bsz;
        const int nb = min(bsz, a.k - row0);
        const int eager = min(EAGER_PLANES, a.nplanes);
        if (tag_base > INT_MAX / 2) tag_base = 0;  // (then the stamps are cleared again below)
        {
            // seen, f[0..2] and the eager planes are one contiguous region (256-byte
            // aligned start), cleared with consecutive 16-byte stores.  After the
            // first batch the frontier arrays are already clear (each batch clears
            // its last frontier through its queue), so only seen and the planes are.
            const ulonglong2 z2 = make_ulonglong2(0ull, 0ull);
            auto clear = [&](u64 *p0, size_t cnt) {
                ulonglong2 *v2 = reinterpret_cast<ulonglong2 *>(p0);
                for (long long i = rank; i < (long long)(cnt >> 1); i += size) v2[i] = z2;
                if ((cnt & 1) && rank == 0) p0[cnt - 1] = 0ull;
            };
            if (b == 0) {
                clear(a.seen, (size_t)((a.plane + eager * pstride) - a.seen));
            } else {
                clear(a.seen, (size_t)(a.fr[0] - a.seen));
                clear(a.plane, (size_t)eager * pstride);
            }
            if (W > 1 && tag_base == 0)
                for (long long w = rank; w < a.n; w += size) a.stamp[w] = 0;
        }
        if (rank == 0) ctl->wo_next = 0;
        if (rank < 4) {
            ctl->qpack[rank] = 0;
            ctl->work[rank] = 0;
#pragma unroll
            for (int q = 0; q < MAXW; ++q) ctl->active[rank][q] = 0;
        }
        if (rank < 4 * COVER_SLOT) a.cover[rank] = 0;
        if (!barrier(ev_idx)) return;
        if (rank < nb) {
            const int32_t s = __ldg(a.sources + row0 + rank);
            if ((unsigned)s >= (unsigned)a.n) {  // reported by the call; its row is never seeded
                atomicCAS(&ctl->err, 0, (int)DEV_ERR_BAD_SOURCE);
                goto seeded;
            }
            const int q = (int)rank >> 6;
            const u64 bit = 1ull << (rank & 63);
            const u64 old = atomicOr(a.fr[0] + (size_t)s * W + q, bit);
            red_or(a.seen + (size_t)s * W + q, bit);
            atomicOr(&ctl->active[0][q], bit);
            bool first;
            if (W == 1) first = old == 0;
            else first = atomicMax(a.stamp + s, tag_base + 1) < tag_base + 1;
            if (first) append_vertex(a, 0, a.q[0], a.qoff[0], s);
        }
    seeded:
        if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, 0, 4, nb, 0);  // batch initialised, seeded
        ++ev_idx;
        if (!barrier(ev_idx - 1)) return;

        bool prev_bu = false;
        int j = 1;
        for (;; ++j) {
            Lvl L;
            const int sc = (j - 1) & 3, sp = (j - 2) & 3;
            const u64 pk = s_ctl.qpack[sc];
            L.qlen = (int)(pk >> QPACK_SHIFT);
            if (L.qlen == 0) break;
            L.qedges = (long long)(pk & QPACK_EDGES);
            L.qlen_prev = j >= 2 ? (int)(s_ctl.qpack[sp] >> QPACK_SHIFT) : 0;
#pragma unroll
            for (int q = 0; q < MAXW; ++q) L.active[q] = q < W ? s_ctl.active[sc][q] : 0ull;
            L.slot = j & 3;
            L.cur = (j - 1) % 3;
            L.nxt = j % 3;
            L.prv = (j + 1) % 3;
            L.qcur = a.q[L.cur];
            L.qcur_off = a.qoff[L.cur];
            L.qnxt = a.q[L.nxt];
            L.qnxt_off = a.qoff[L.nxt];
            L.qprev = a.q[L.prv];
            L.fcur = a.fr[L.cur];
            L.fnxt = a.fr[L.nxt];
            L.fprv = a.fr[L.prv];
            L.sact = s_act;
            L.lev = j - 1;
            L.tag = tag_base + j + 1;
            if (rank == 0) {
                const int z = (j + 1) & 3;
                ctl->qpack[z] = 0;
                ctl->work[z] = 0;
#pragma unroll
                for (int q = 0; q < MAXW; ++q) ctl->active[z][q] = 0;
            }
            if (rank < COVER_SLOT) a.cover[((j + 1) & 3) * COVER_SLOT + rank] = 0;
            L.rare_td = false;
            L.scanq = false;
            // plane b is first written in phase 2^b + 1; clear it one phase earlier
            if ((j & (j - 1)) == 0) {
                const int pb = __ffs(j) - 1;
                if (pb >= EAGER_PLANES && pb < a.nplanes)
                    for (long long w = rank; w < a.n; w += size) zerow<W>(a.plane + pb * pstride + (size_t)w * W);
            }
            bool bu = false;
            if (VARIANT == GU_BFS_BOTTOM_UP) {
                bu = j > 1;
            } else if (VARIANT == GU_BFS_AUTO) {
                if (!prev_bu) bu = j > 1 && (double)L.qedges * (double)a.alpha > (double)a.m;
                else bu = (double)L.qlen * (double)a.beta > (double)a.n &&
                          (double)L.qedges * (double)a.gamma > (double)a.n;
            }
            if (bu) {
                // part A; F_0 may hold sources without in-edges, which no class list has
                if (j == 2 && rank < nb) {
                    const int32_t s0 = __ldg(a.sources + row0 + rank);
                    if ((unsigned)s0 < (unsigned)a.n) zerow<W>(L.fprv + (size_t)s0 * W);
                }
                if (rank == 0) ctl->rpack = 0;
                bu_finalise_all<W, G>(a, L);
                __syncthreads();
                if (threadIdx.x < 64 * W && ((s_act[threadIdx.x >> 6] >> (threadIdx.x & 63)) & 1ull))
                    atomicAdd(&a.cover[L.slot * COVER_SLOT + threadIdx.x], 1);
                // timeline kinds 5-7: parts A and B, and the light class within B
                if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, j, 5, L.qlen, L.qedges);
                ++ev_idx;
                if (!barrier(ev_idx - 1)) return;
                // part B: sources searched bottom-up and rare ones, from the coverage
                if (threadIdx.x < 64 * W) {
                    const float c = (float)ld_volatile_i32(&a.cover[L.slot * COVER_SLOT + threadIdx.x]);
                    const float thr = fmaxf(1.f, a.rare_frac * (float)G::nblk());
                    const unsigned cb = __ballot_sync(FULL_MASK, c >= thr);
                    const unsigned rb = __ballot_sync(FULL_MASK, c >= 1.f && c < thr);
                    if ((threadIdx.x & 31) == 0) {  // 32-bit halves of the 64-bit words
                        reinterpret_cast<unsigned *>(s_excl)[threadIdx.x >> 5] = cb;
                        reinterpret_cast<unsigned *>(s_rare)[threadIdx.x >> 5] = rb;
                    }
                }
                __syncthreads();
                u64 any_rare = 0;
#pragma unroll
                for (int q = 0; q < W; ++q) {
                    L.active[q] = s_excl[q];
                    any_rare |= s_rare[q];
                }
                L.rare_td = any_rare != 0;
                // discovered vertices collect in the CTA's shared queue (the whole
                // staging buffer), flushed to the level's queue at the end of part B
                const CtaQ cq{reinterpret_cast<int32_t *>(ms_smem()), cq_count(), MS_SMEM_BYTES / 4};
                bu_light<W, G>(a, L, cq);
                if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, j, 6, L.qlen, L.qedges);
                ++ev_idx;
                bu_mid<W, G>(a, L, cq);
                bu_wide<W, G>(a, L, cq);
                bu_heavy<W, G>(a, L, cq);
                if (L.rare_td) bu_rare_list<W, G>(a, L, s_rare);
                __syncthreads();
                if (*cq.n > 0) cta_flush(a, L, cq);
                if (L.rare_td) {  // part C
                    if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, j, 7, L.qlen, L.qedges);
                    ++ev_idx;
                    if (!barrier(ev_idx - 1)) return;
                    const u64 rp = s_ctl.rpack;
                    Lvl LC = L;
                    LC.qcur = a.q[L.prv];
                    LC.qcur_off = a.qoff[L.prv];
                    LC.qlen = (int)(rp >> QPACK_SHIFT);
                    LC.qedges = (long long)(rp & QPACK_EDGES);
                    gather_mp<W, G, true>(a, LC, s_rare);
                }
            } else {
                // A top-down expansion over more edges than the graph has vertices
                // discovers a large F_j, most vertices many times: then a visit is
                // only an OR of the frontier word into F_j (no read of seen, no
                // first-discovery stamp), and one scan after the level keeps the
                // bits not seen before, updates seen and builds the next queue.
                L.scanq = VARIANT == GU_BFS_AUTO && (double)L.qedges > (double)a.n;
                td_update<W, G>(a, L);
                if (VARIANT == GU_BFS_EDGE) gather_edge<W, G>(a, L);
                else if (VARIANT == GU_BFS_WARP) gather_warp<W, G>(a, L);
                else if (VARIANT == GU_BFS_CTA_WARP) gather_cta_warp<W, G>(a, L);
                else if (VARIANT == GU_BFS_SCAN) gather_scan<W, G>(a, L);
                else if (VARIANT == GU_BFS_SHUFFLE) gather_shuffle<W, G>(a, L);
                else if (VARIANT == GU_BFS_LINEAR) gather_linear<W, G>(a, L);
                else gather_mp<W, G>(a, L);  // AUTO, BOTTOM_UP level 1
                if (L.scanq) {
                    if (!barrier(ev_idx)) return;  // every claim of the level is in F_j
                    const CtaQ cq{reinterpret_cast<int32_t *>(ms_smem()), cq_count(), MS_SMEM_BYTES / 4};
                    for (long long v = rank; v < a.n; v += size) {
                        const size_t o = (size_t)v * W;
                        u64 f[W];
                        ldw<W>(L.fnxt + o, f);
                        if (!anyw<W>(f)) continue;
                        u64 sn[W], nb[W];
                        ldw<W>(a.seen + o, sn);
#pragma unroll
                        for (int q = 0; q < W; ++q) {
                            nb[q] = f[q] & ~sn[q];
                            sn[q] |= nb[q];
                        }
                        stw<W>(L.fnxt + o, nb);  // F_j: the new bits only (zero if none)
                        if (anyw<W>(nb)) {
                            stw<W>(a.seen + o, sn);
                            cq.push(a, L, (int32_t)v);
                        }
                    }
                    __syncthreads();
                    if (*cq.n > 0) cta_flush(a, L, cq);
                }
            }
            __syncthreads();
            if (threadIdx.x < W) {
                const u64 r = s_act[threadIdx.x];
                if (r) atomicOr(&ctl->active[L.slot][threadIdx.x], r);
                s_act[threadIdx.x] = 0;
            }
            if (rank == 0) {
                if (bu) ctl->bu_levels++;
                else ctl->td_levels++;
                if (j - 1 > ctl->max_level) ctl->max_level = j - 1;
            }
            if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, j, bu ? 1 : 0, L.qlen, L.qedges);
            ++ev_idx;
            prev_bu = bu;
            if (!barrier(ev_idx - 1)) return;
        }
        // F_{j-1} is empty: levels of this batch are 0..j-2.  F_{j-2} is the only
        // frontier array with bits left: clear it through its queue, so that the
        // next batch starts from clear frontier arrays.
        {
            const int nq = (int)(s_ctl.qpack[(j - 2) & 3] >> QPACK_SHIFT);
            const int32_t *qq = a.q[(j - 2) % 3];
            u64 *ff = a.fr[(j - 2) % 3];
            for (long long i = rank; i < nq; i += size) zerow<W>(ff + (size_t)__ldcg(qq + i) * W);
        }
        tag_base += j + 1;
        int used = 0;
        while (used < 31 && ((j - 2) >> used) != 0) ++used;
        if (a.dist) write_distances<W, G>(a, row0, nb, used);  // no rows: diameter, reach queries
        if (a.reach) count_reached<W, G>(a, row0, nb);
        if (threadIdx.x == 0) record_event(ctl, ev_idx, rank == 0, b, j, 2, 0, 0);  // distance rows written
        ++ev_idx;
        if (!barrier(ev_idx - 1)) return;
    }
}

template <int VARIANT, int W>
__global__ void __launch_bounds__(MS_THREADS, MS_MIN_BLOCKS) ms_grid_kernel(MsArgs a)
{
    unsigned epoch = 0;
    ms_search<VARIANT, W, GridG>(a, epoch);
}

// Workspace layout of one batched search over n vertices with W words per vertex:
// control region, seen, three frontier arrays, the level planes, stamps, three
// queues with their offsets (each array 256-byte aligned).
__host__ __device__ inline size_t ms_up256(size_t b) { return ((b + 255) / 256) * 256; }
__host__ __device__ inline int ms_planes(size_t n)
{
    // every BFS level is at most n - 1: bit-length of n - 1 planes suffice
    int nplanes = 1;
    while (nplanes < MAX_PLANES && ((int64_t)(n > 0 ? n - 1 : 0) >> nplanes) != 0) ++nplanes;
    return nplanes;
}
__host__ __device__ inline size_t ms_layout_bytes(size_t n, int W)
{
    return WS_CONTROL_BYTES + (4 + (size_t)ms_planes(n)) * ms_up256(n * W * sizeof(u64)) +
           7 * ms_up256(n * sizeof(int32_t));
}
__host__ __device__ inline void ms_layout(char *ws, size_t n, int W, MsArgs &a)
{
    const size_t words_bytes = ms_up256(n * W * sizeof(u64));
    const size_t i32_bytes = ms_up256(n * sizeof(int32_t));
    char *p = ws;
    a.ctl = reinterpret_cast<MsCtl *>(p);
    a.cover = reinterpret_cast<int *>(p + COVER_OFF);
    p += WS_CONTROL_BYTES;
    a.seen = reinterpret_cast<u64 *>(p);
    p += words_bytes;
    for (int i = 0; i < 3; ++i) {
        a.fr[i] = reinterpret_cast<u64 *>(p);
        p += words_bytes;
    }
    a.plane = reinterpret_cast<u64 *>(p);
    a.nplanes = ms_planes(n);
    p += (size_t)a.nplanes * words_bytes;
    a.stamp = reinterpret_cast<int32_t *>(p);
    p += i32_bytes;
    for (int i = 0; i < 3; ++i) {
        a.q[i] = reinterpret_cast<int32_t *>(p);
        p += i32_bytes;
        a.qoff[i] = reinterpret_cast<int32_t *>(p);
        p += i32_bytes;
    }
}

// ---- work-queue launch: many graphs and source blocks in one persistent grid ----
// The grid is cut into groups of group_size consecutive CTAs.  A group's first CTA
// takes the next item from a device counter and the group barrier hands it to the
// group's other CTAs; the group then runs the batched search of that item (one
// graph, up to 64 W sources) in its own slice of the workspace, with barriers over
// its own CTAs only, and takes the next item until none is left.  Items of
// different graphs and sizes run side by side on different groups.
struct MqItem {
    const int32_t *R, *C, *RT, *CT;
    const int32_t *light, *mid, *wide, *heavy;
    int32_t n, nlight, nmid, nwide, nheavy;
    int32_t degbits;
    int64_t m;
    const int32_t *sources;
    int32_t k;
    int32_t *dist;              // k x ld rows, or null
    int64_t ld;
    unsigned long long *reach;  // k reachable counts (zeroed before the launch), or null
};

struct MqArgs {
    const MqItem *items;
    int nitems;
    int *next;           // item counter, zeroed before the launch
    char *ws;            // group g's slice at ws + g * ws_stride
    size_t ws_stride;
    int group_size;
    float alpha, beta, gamma, rare_frac;
    unsigned long long wait_ns;
};

template <int W>
__global__ void __launch_bounds__(MS_THREADS, MS_MIN_BLOCKS) ms_queue_kernel(MqArgs q)
{
    __shared__ int s_item;
    __shared__ MsArgs s_args;
    const int grp = blockIdx.x / q.group_size;
    if (threadIdx.x == 0) {
        s_grp_base = grp * q.group_size;
        s_grp_nblk = min(q.group_size, (int)gridDim.x - grp * q.group_size);
    }
    __syncthreads();
    char *ws = q.ws + (size_t)grp * q.ws_stride;
    MsCtl *ctl = reinterpret_cast<MsCtl *>(ws);
    unsigned epoch = 0;
    while (true) {
        if (GroupG::rank() == 0) ctl->item = atomicAdd(q.next, 1);
        if (!grid_barrier(&ctl->bar, &ctl->err, epoch, q.wait_ns, nullptr, nullptr, 0, (unsigned)GroupG::nblk())) return;
        if (threadIdx.x == 0) s_item = ld_volatile_i32(&ctl->item);
        __syncthreads();
        const int it = s_item;
        if (it >= q.nitems) return;
        if (threadIdx.x == 0) {  // the item's arguments, in shared memory for the whole CTA
            const MqItem m = q.items[it];
            MsArgs &a = s_args;
            a.R = m.R;
            a.C = m.C;
            a.RT = m.RT;
            a.CT = m.CT;
            a.F = nullptr;  // AUTO never sweeps the COO array
            a.light = m.light;
            a.mid = m.mid;
            a.wide = m.wide;
            a.heavy = m.heavy;
            a.n = m.n;
            a.nlight = m.nlight;
            a.nmid = m.nmid;
            a.nwide = m.nwide;
            a.nheavy = m.nheavy;
            a.m = m.m;
            a.sources = m.sources;
            a.k = m.k;
            a.dist = m.dist;
            a.reach = m.reach;
            a.ld = m.ld;
            ms_layout(ws, (size_t)m.n, W, a);
            a.alpha = q.alpha;
            a.beta = q.beta;
            a.gamma = q.gamma;
            a.rare_frac = q.rare_frac;
            a.degbits = m.degbits;
            a.wait_ns = q.wait_ns;
        }
        __syncthreads();
        ms_search<GU_BFS_AUTO, W, GroupG>(s_args, epoch);
        if (ld_volatile_i32(&ctl->err) != 0) return;  // every CTA of the group sees it at its next barrier
    }
}

// ---- host side ---------------------------------------------------------------------
template <int V, int W>
static void launch_one(const MsArgs &a, int sms, cudaStream_t stream, int max_blocks = 0)
{
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, ms_grid_kernel<V, W>, MS_THREADS, 0));
        if (blocks_per_sm < 1) throw gu_error(GU_ERR_INTERNAL, "msbfs kernel cannot be resident");
    }
    int nblocks = sms * blocks_per_sm;
    if (max_blocks > 0 && nblocks > max_blocks) nblocks = max_blocks;
    dim3 grid(nblocks), block(MS_THREADS);
    MsArgs args = a;
    void *params[] = {&args};
    GU_CUDA_CHECK(cudaLaunchCooperativeKernel((const void *)ms_grid_kernel<V, W>, grid, block, params, 0, stream));
}

template <int V>
static void launch_words(const MsArgs &a, int W, int sms, cudaStream_t stream, int max_blocks)
{
    if (W == 1) launch_one<V, 1>(a, sms, stream, max_blocks);
    else if (W == 2) launch_one<V, 2>(a, sms, stream, max_blocks);
    else launch_one<V, 4>(a, sms, stream, max_blocks);
}

static float env_float(const char *name, float dflt)
{
    const char *s = std::getenv(name);
    if (!s || !*s) return dflt;
    return std::strtof(s, nullptr);
}

int msbfs_words_for(int32_t k)
{
    const char *s = std::getenv("GU_MS_WORDS");
    if (s && *s) {
        const int w = std::atoi(s);
        if (w == 1 || w == 2 || w == 4) return w;
    }
    if (k <= 64) return 1;
    if (k <= 128) return 2;
    return 4;
}

size_t msbfs_workspace_bytes(const DeviceGraph &g, int32_t k)
{
    return ms_layout_bytes((size_t)g.n, msbfs_words_for(k));
}

void launch_msbfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                  const MsOptions &opt, cudaStream_t stream, int *dev_err_out)
{
    (void)dev_err_out;
    if (opt.variant == GU_BFS_EDGE) ensure_coo(g, stream);
    const int W = (opt.batch_words == 1 || opt.batch_words == 2 || opt.batch_words == 4) ? opt.batch_words
                                                                                         : msbfs_words_for(k);
    const size_t n = (size_t)g.n;
    static_assert(CTL_REGION <= WS_CONTROL_BYTES, "timeline must fit the control region");
    Workspace &wsp = opt.ws ? *opt.ws : g.ws;
    char *ws = (char *)wsp.get(ms_layout_bytes(n, W));
    MsArgs a;
    a.R = g.R;
    a.C = g.C;
    a.RT = g.RT;
    a.CT = g.CT;
    a.F = g.F;
    a.light = g.light;
    a.mid = g.mid;
    a.wide = g.wide;
    a.heavy = g.heavy;
    a.n = g.n;
    a.nlight = g.nlight;
    a.nmid = g.nmid;
    a.nwide = g.nwide;
    a.nheavy = g.nheavy;
    a.m = g.m;
    a.sources = sources;
    a.k = k;
    a.dist = dist;
    a.reach = opt.reach;
    a.ld = ld;
    ms_layout(ws, n, W, a);
    a.alpha = opt.tuned ? opt.alpha : env_float("GU_MS_ALPHA", opt.alpha);
    a.beta = opt.tuned ? opt.beta : env_float("GU_MS_BETA", opt.beta);
    a.gamma = env_float("GU_MS_GAMMA", opt.gamma);
    a.rare_frac = opt.tuned ? opt.rare_frac : env_float("GU_MS_RARE", opt.rare_frac);
    int degbits = 1;
    while (degbits < 31 && (1ll << degbits) <= (long long)g.max_degree) ++degbits;
    a.degbits = degbits;
    a.wait_ns = wait_limit_ns();
    GU_CUDA_CHECK(cudaMemsetAsync(a.ctl, 0, CTL_REGION, stream));
    const int sms = g.sm_count;
    const int mb = opt.max_blocks;
    g.timeline = 0;
    if (opt.timed) g.mark_start(stream);
    switch (opt.variant) {
    case GU_BFS_AUTO: launch_words<GU_BFS_AUTO>(a, W, sms, stream, mb); break;
    case GU_BFS_LINEAR: launch_words<GU_BFS_LINEAR>(a, W, sms, stream, mb); break;
    case GU_BFS_EDGE: launch_words<GU_BFS_EDGE>(a, W, sms, stream, mb); break;
    case GU_BFS_WARP: launch_words<GU_BFS_WARP>(a, W, sms, stream, mb); break;
    case GU_BFS_CTA_WARP: launch_words<GU_BFS_CTA_WARP>(a, W, sms, stream, mb); break;
    case GU_BFS_SCAN: launch_words<GU_BFS_SCAN>(a, W, sms, stream, mb); break;
    case GU_BFS_SHUFFLE: launch_words<GU_BFS_SHUFFLE>(a, W, sms, stream, mb); break;
    case GU_BFS_BOTTOM_UP: launch_words<GU_BFS_BOTTOM_UP>(a, W, sms, stream, mb); break;
    default: throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown BFS variant");
    }
    if (opt.timed) g.mark_stop(stream);
    if (&wsp == &g.ws) {  // the control block comes back with the launch: one round trip per call
        if (!g.ctl_host) GU_CUDA_CHECK(pinned_alloc(&g.ctl_host, sizeof(MsCtl)));
        GU_CUDA_CHECK(cudaMemcpyAsync(g.ctl_host, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, stream));
    }
}

// ---- work-queue launch (host) ----------------------------------------------------
template <int W>
static int queue_blocks_per_sm()
{
    static int b = -1;
    if (b < 0) {
        GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ms_queue_kernel<W>, MS_THREADS, 0));
        if (b < 1) throw gu_error(GU_ERR_INTERNAL, "work-queue kernel cannot be resident");
    }
    return b;
}

// Words per vertex, groups and workspace of a work-queue launch over reqs.
MsQueueLaunch msbfs_queue_plan(const std::vector<MsQueueRequest> &reqs, int sms, int max_blocks)
{
    int32_t maxk = 0;
    size_t maxn = 0;
    for (const MsQueueRequest &r : reqs) {
        if (!r.g || r.k < 0 || (r.k > 0 && (!r.sources || (!r.dist && !r.reach))))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad work-queue request");
        if (r.dist && r.ld < r.g->n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
        if (r.k == 0) continue;
        maxk = std::max(maxk, r.k);
        maxn = std::max(maxn, (size_t)r.g->n);
    }
    MsQueueLaunch L;
    if (maxk == 0) return L;
    L.W = msbfs_words_for(std::min(maxk, 64 * MAXW));
    const int per_item = 64 * L.W;
    for (const MsQueueRequest &r : reqs) L.items += (r.k + per_item - 1) / per_item;
    const int bps = L.W == 1 ? queue_blocks_per_sm<1>() : L.W == 2 ? queue_blocks_per_sm<2>() : queue_blocks_per_sm<4>();
    int blocks = sms * bps;
    if (max_blocks > 0) blocks = std::min(blocks, max_blocks);
    // group size: about 16 K vertices per CTA of a group, larger while there are
    // fewer items than groups, so that the grid is used
    int gs = (int)std::min<size_t>((maxn + 16383) / 16384, (size_t)blocks);
    gs = std::max(gs, std::max(1, blocks / L.items));
    L.group_size = std::max(1, std::min(gs, blocks));
    L.ngroups = blocks / L.group_size;
    L.stride = ms_up256(ms_layout_bytes(maxn, L.W));
    L.items_off = (size_t)L.ngroups * L.stride;
    L.cnt_off = L.items_off + ms_up256(sizeof(MqItem) * (size_t)L.items);
    L.bytes = L.cnt_off + 256;
    return L;
}

MsQueueLaunch launch_msbfs_queue(const std::vector<MsQueueRequest> &reqs, Workspace &wsp, int sms, int max_blocks,
                                 cudaStream_t st)
{
    const MsQueueLaunch L = msbfs_queue_plan(reqs, sms, max_blocks);
    if (L.items == 0) return L;
    const int W = L.W, per_item = 64 * W;
    std::vector<MqItem> items;
    for (const MsQueueRequest &r : reqs) {
        if (r.k == 0) continue;
        const DeviceGraph &g = *r.g;
        int degbits = 1;
        while (degbits < 31 && (1ll << degbits) <= (long long)g.max_degree) ++degbits;
        if (r.reach) GU_CUDA_CHECK(cudaMemsetAsync(r.reach, 0, sizeof(unsigned long long) * (size_t)r.k, st));
        for (int32_t off = 0; off < r.k; off += per_item) {
            MqItem it;
            it.R = g.R;
            it.C = g.C;
            it.RT = g.RT;
            it.CT = g.CT;
            it.light = g.light;
            it.mid = g.mid;
            it.wide = g.wide;
            it.heavy = g.heavy;
            it.n = g.n;
            it.nlight = g.nlight;
            it.nmid = g.nmid;
            it.nwide = g.nwide;
            it.nheavy = g.nheavy;
            it.degbits = degbits;
            it.m = g.m;
            it.sources = r.sources + off;
            it.k = std::min(per_item, r.k - off);
            it.dist = r.dist ? r.dist + (size_t)off * (size_t)r.ld : nullptr;
            it.ld = r.ld;
            it.reach = r.reach ? r.reach + off : nullptr;
            items.push_back(it);
        }
    }
    char *ws = (char *)wsp.get(L.bytes);
    GU_CUDA_CHECK(cudaMemset2DAsync(ws, L.stride, 0, CTL_REGION, (size_t)L.ngroups, st));
    GU_CUDA_CHECK(cudaMemsetAsync(ws + L.cnt_off, 0, sizeof(int), st));
    GU_CUDA_CHECK(cudaMemcpyAsync(ws + L.items_off, items.data(), sizeof(MqItem) * items.size(), cudaMemcpyHostToDevice,
                                  st));
    MqArgs q;
    q.items = reinterpret_cast<const MqItem *>(ws + L.items_off);
    q.nitems = (int)items.size();
    q.next = reinterpret_cast<int *>(ws + L.cnt_off);
    q.ws = ws;
    q.ws_stride = L.stride;
    q.group_size = L.group_size;
    q.alpha = env_float("GU_MS_ALPHA", 2.f);
    q.beta = env_float("GU_MS_BETA", 24.f);
    q.gamma = env_float("GU_MS_GAMMA", 4.f);
    q.rare_frac = env_float("GU_MS_RARE", MsOptions().rare_frac);
    q.wait_ns = wait_limit_ns();
    void *params[] = {&q};
    const void *fn = W == 1 ? (const void *)ms_queue_kernel<1> : W == 2 ? (const void *)ms_queue_kernel<2>
                                                                       : (const void *)ms_queue_kernel<4>;
    GU_CUDA_CHECK(cudaLaunchCooperativeKernel(fn, dim3(L.ngroups * L.group_size), dim3(MS_THREADS), params, 0, st));
    return L;
}

// First non-zero device error word of the groups of a work-queue launch (after
// its stream is synchronised).
int msbfs_queue_error(const Workspace &ws, const MsQueueLaunch &L)
{
    if (L.ngroups == 0) return 0;
    std::vector<int> e((size_t)L.ngroups, 0);
    GU_CUDA_CHECK(cudaMemcpy2D(e.data(), sizeof(int), static_cast<const char *>(ws.ptr) + offsetof(MsCtl, err), L.stride,
                               sizeof(int), (size_t)L.ngroups, cudaMemcpyDeviceToHost));
    for (int x : e)
        if (x) return x;
    return 0;
}

void msbfs_status_after_sync(DeviceGraph &g, int *dev_err, int *td_levels, int *bu_levels, int *max_level)
{
    if (!g.ctl_host) {
        msbfs_read_status(g, dev_err, td_levels, bu_levels, max_level);
        return;
    }
    const MsCtl &c = *static_cast<const MsCtl *>(g.ctl_host);
    if (dev_err) *dev_err = c.err;
    if (td_levels) *td_levels = c.td_levels;
    if (bu_levels) *bu_levels = c.bu_levels;
    if (max_level) *max_level = c.max_level;
}

// Device error word of a launch that used workspace `ws` (after its stream is synchronised).
int msbfs_ws_error(const Workspace &ws)
{
    MsCtl c;
    GU_CUDA_CHECK(cudaMemcpy(&c, ws.ptr, sizeof(MsCtl), cudaMemcpyDeviceToHost));
    return c.err;
}

// Reads the control block of the last launch (after the stream is synchronised).
void msbfs_read_status(DeviceGraph &g, int *dev_err, int *td_levels, int *bu_levels, int *max_level)
{
    MsCtl c;
    GU_CUDA_CHECK(cudaMemcpy(&c, g.ws.ptr, sizeof(MsCtl), cudaMemcpyDeviceToHost));
    if (dev_err) *dev_err = c.err;
    if (td_levels) *td_levels = c.td_levels;
    if (bu_levels) *bu_levels = c.bu_levels;
    if (max_level) *max_level = c.max_level;
}

// Copies the per-phase timeline of the last batched launch (after a stream sync).
int msbfs_read_timeline(DeviceGraph &g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                        int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms)
{
    std::vector<char> buf(CTL_REGION);
    GU_CUDA_CHECK(cudaMemcpy(buf.data(), g.ws.ptr, CTL_REGION, cudaMemcpyDeviceToHost));
    const MsEvent *ev = reinterpret_cast<const MsEvent *>(buf.data() + 256);
    const int cnt = *reinterpret_cast<const int *>(ev + TIMELINE_MAX);
    const int nout = cnt < max_entries ? cnt : max_entries;
    for (int i = 0; i < nout; ++i) {
        if (batch) batch[i] = ev[i].batch;
        if (level) level[i] = ev[i].level;
        if (kind) kind[i] = ev[i].bottom_up;
        if (frontier_vertices) frontier_vertices[i] = ev[i].qlen;
        if (frontier_edges) frontier_edges[i] = ev[i].qedges;
        if (t_ms) t_ms[i] = (double)(ev[i].t_last_ns - ev[0].t_last_ns) * 1e-6;
    }
    return nout;
}

// Idle CTA time per phase of the last batched launch (after a stream sync): for
// each timeline entry, the sum over CTAs of their waits at the grid barriers of
// that phase, in ms; *nblocks = the launch's CTAs.
int msbfs_read_idle(DeviceGraph &g, int max_entries, double *idle_ms, int *nblocks)
{
    std::vector<char> buf(CTL_REGION);
    GU_CUDA_CHECK(cudaMemcpy(buf.data(), g.ws.ptr, CTL_REGION, cudaMemcpyDeviceToHost));
    const MsCtl *c = reinterpret_cast<const MsCtl *>(buf.data());
    const MsEvent *ev = reinterpret_cast<const MsEvent *>(buf.data() + 256);
    const int cnt = *reinterpret_cast<const int *>(ev + TIMELINE_MAX);
    const int nout = cnt < max_entries ? cnt : max_entries;
    for (int i = 0; i < nout; ++i)
        if (idle_ms) idle_ms[i] = (double)ev[i].idle_ns * 1e-6;
    if (nblocks) *nblocks = c->nblocks;
    return nout;
}

// ---- allocation-free multi-source BFS (gu_bfs_noalloc) -------------------------------
// Some callers may not allocate device memory at the time they search: code that
// runs inside a host process whose allocator owns and accounts for every byte of
// the GPU (a database, an inference server, a framework's caching pool), services
// that fix their memory budget at start-up, and paths that must not pay for the
// implicit device synchronisation of cudaMalloc/cudaFree.  For them the batched
// engine can run with its scratch in the fixed-size array below instead of a
// graph handle's workspace: top-down levels only (so neither an in-edge CSR nor the
// degree-class lists are needed), one 64-bit word per vertex, the caller's own
// device CSR, sources and distance rows.

constexpr int32_t NOALLOC_MAX_VERTICES = 32768;
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)6 << 20;  // 6 MiB per device
constexpr size_t NOALLOC_FLAG_OFFSET = WS_CONTROL_BYTES - 64;

// Reserved on every device when the library's device code is loaded there and
// held until the process exits; all gu_bfs_noalloc calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

static size_t noalloc_layout_bytes(int32_t n, int *nplanes_out)
{
    auto up = [](size_t b) { return ((b + 255) / 256) * 256; };
    int nplanes = 1;
    while (nplanes < MAX_PLANES && ((int64_t)(n > 0 ? n - 1 : 0) >> nplanes) != 0) ++nplanes;
    if (nplanes_out) *nplanes_out = nplanes;
    return WS_CONTROL_BYTES + (4 + (size_t)nplanes) * up((size_t)n * sizeof(u64)) + 7 * up((size_t)n * sizeof(int32_t));
}

// Flags malformed inputs instead of letting the search index out of bounds:
// 1 = R not a valid offset array, 2 = column index out of range, 4 = source out of range.
__global__ void noalloc_validate_kernel(const int32_t *R, const int32_t *C, int32_t n, int64_t m,
                                        const int32_t *sources, int32_t k, int *flag)
{
    const long long rank = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long size = (long long)gridDim.x * blockDim.x;
    if (rank == 0 && (R[0] != 0 || (int64_t)R[n] != m)) atomicOr(flag, 1);
    for (long long v = rank; v < n; v += size)
        if (R[v + 1] < R[v]) atomicOr(flag, 1);
    for (long long e = rank; e < m; e += size) {
        const int32_t c = C[e];
        if (c < 0 || c >= n) atomicOr(flag, 2);
    }
    for (long long i = rank; i < k; i += size) {
        const int32_t s = sources[i];
        if (s < 0 || s >= n) atomicOr(flag, 4);
    }
}

// Device address of the scratch array on the current device.  The host-side name
// g_noalloc_scratch is only a stand-in, so the address is looked up with the
// device current, on every call: a cached address would outlive a
// cudaDeviceReset (which reloads the module and may place the array elsewhere).
// The first call on a device loads the library's module there; make it before
// any stream capture.  Later lookups are a host-side table search.
static char *noalloc_scratch_for_current_device()
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        throw gu_error(GU_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    return static_cast<char *>(p);
}

static void bfs_noalloc(const int32_t *R, const int32_t *C, int32_t n, int64_t m, const int32_t *sources, int32_t k,
                        int32_t *dist, int64_t ld, cudaStream_t st)
{
    if (n < 0 || m < 0 || m > INT32_MAX || k < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "negative size or m > INT32_MAX");
    if (n > NOALLOC_MAX_VERTICES)
        throw gu_error(GU_ERR_CAPACITY, "gu_bfs_noalloc handles at most " + std::to_string(NOALLOC_MAX_VERTICES) +
                                            " vertices (its static scratch is 6 MiB per device); got n = " +
                                            std::to_string(n));
    if (ld < n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
    if (k == 0) return;
    if (n == 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range (graph has no vertices)");
    if (!R || (m > 0 && !C) || !sources || !dist) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null device buffer");
    int nplanes = 1;
    if (noalloc_layout_bytes(n, &nplanes) > NOALLOC_SCRATCH_BYTES)
        throw gu_error(GU_ERR_INTERNAL, "static scratch smaller than its layout");
    char *scratch = noalloc_scratch_for_current_device();
    int dev = 0;
    GU_CUDA_CHECK(cudaGetDevice(&dev));
    const int sms = device_sm_count(dev);

    int *flag = reinterpret_cast<int *>(scratch + NOALLOC_FLAG_OFFSET);
    GU_CUDA_CHECK(cudaMemsetAsync(flag, 0, sizeof(int), st));
    noalloc_validate_kernel<<<sms * 4, 256, 0, st>>>(R, C, n, m, sources, k, flag);
    GU_CUDA_CHECK(cudaGetLastError());
    int hflag = 0;
    GU_CUDA_CHECK(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    if (hflag & 1) throw gu_error(GU_ERR_INVALID_ARGUMENT, "R must start at 0, be non-decreasing and end at m");
    if (hflag & 2) throw gu_error(GU_ERR_INVALID_ARGUMENT, "column index out of range");
    if (hflag & 4) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range");

    auto up = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t words_bytes = up((size_t)n * sizeof(u64));
    const size_t i32_bytes = up((size_t)n * sizeof(int32_t));
    MsArgs a;
    a.R = R;
    a.C = C;
    a.RT = R;  // never read: top-down levels only
    a.CT = C;
    a.F = nullptr;
    a.light = a.mid = a.wide = a.heavy = nullptr;  // top-down levels only
    a.n = n;
    a.nlight = a.nmid = a.nwide = a.nheavy = 0;
    a.m = m;
    a.sources = sources;
    a.k = k;
    a.dist = dist;
    a.reach = nullptr;
    a.ld = ld;
    char *p = scratch;
    a.ctl = reinterpret_cast<MsCtl *>(p);
    a.cover = reinterpret_cast<int *>(p + COVER_OFF);
    p += WS_CONTROL_BYTES;
    a.seen = reinterpret_cast<u64 *>(p);
    p += words_bytes;
    for (int i = 0; i < 3; ++i) {
        a.fr[i] = reinterpret_cast<u64 *>(p);
        p += words_bytes;
    }
    a.plane = reinterpret_cast<u64 *>(p);
    a.nplanes = nplanes;
    p += (size_t)nplanes * words_bytes;
    a.stamp = reinterpret_cast<int32_t *>(p);
    p += i32_bytes;
    for (int i = 0; i < 3; ++i) {
        a.q[i] = reinterpret_cast<int32_t *>(p);
        p += i32_bytes;
        a.qoff[i] = reinterpret_cast<int32_t *>(p);
        p += i32_bytes;
    }
    a.alpha = 0.f;  // never switch to bottom-up
    a.beta = 24.f;
    a.gamma = 4.f;
    a.rare_frac = 0.f;
    int degbits = 1;
    while (degbits < 31 && (1ll << degbits) <= (long long)m) ++degbits;
    a.degbits = degbits;
    a.wait_ns = wait_limit_ns();
    // the previous call's contents stay in the array: clear the control block
    GU_CUDA_CHECK(cudaMemsetAsync(a.ctl, 0, CTL_REGION, st));
    launch_one<GU_BFS_AUTO, 1>(a, sms, st);
    int err = 0;
    GU_CUDA_CHECK(cudaMemcpyAsync(&err, &a.ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    if (err == DEV_ERR_BARRIER_TIMEOUT) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit");
    if (err != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(err));
}

}  // namespace gu

extern "C" gu_status gu_bfs_noalloc(const int32_t *R_dev, const int32_t *C_dev, int32_t n, int64_t m,
                                    const int32_t *sources_dev, int32_t k, int32_t *dist_dev, int64_t ld,
                                    void *stream)
{
    try {
        gu::bfs_noalloc(R_dev, C_dev, n, m, sources_dev, k, dist_dev, ld, (cudaStream_t)stream);
        return GU_OK;
    } catch (const gu::gu_error &e) {
        gu::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        gu::set_last_error(e.what());
        return GU_ERR_INTERNAL;
    }
}
