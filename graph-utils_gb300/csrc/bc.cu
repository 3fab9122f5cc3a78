// bc.cu -- batched shortest-path counting (sigma) and Brandes betweenness
// centrality on sm_103a.
//
// Restates, for a batch of B = 64*W sources per pass, the reference's designed
// (commented-out) GPU kernels: the forward sweep counting shortest paths
// (multi_search/shuffle_based.cu:113-151, 164-214) and the backward dependency
// accumulation delta_s(w) = sum over successors v of sigma_s(w)/sigma_s(v) *
// (1 + delta_s(v)) (shuffle_based.cu:217-354), then bc[v] += delta_s(v)
// (shuffle_based.cu:350-353).  By design: sigma is uint64 and bit-exact (integer
// sums do not depend on order), delta and bc are FP64, and every floating-point
// sum runs in a fixed order -- CSR neighbour order inside a work item, work
// items of a vertex in order, a fixed-shape warp tree over the batch's sources,
// batches in order -- so results do not depend on scheduling.  No float atomics.
//
// Layout (workspace, per graph handle):
//   seen[n][W]          sources known at a vertex (lags one level, see below)
//   lvl[L+1][n][W]      lvl[j] = bitmap of the sources whose BFS level of v is j
//   sigma[n][B] uint64  shortest-path counts, sources of the batch contiguous
//   delta[n][B] double  dependencies
//   beta[n][B] double   (1 + delta) / sigma, the backward terms
//   part[slots][W][64]  backward partial sums of vertices split into several items
//   bc[n] double        accumulated over batches (output)
// Work items (graph-static, ChunkMap): one per <= 256 edges of a vertex's in-
// (forward) or out-adjacency (backward), times the word groups of the batch (up
// to four source words, 256 sources, per group), so an adjacency range is read
// once for 256 sources.  Items are grouped into work units (heaviest first, <= 32
// items and about 512 edges; smaller on small graphs) that warps take from a
// per-level counter; a warp triages a unit's items a lane each and then runs the
// items with work.  Forward, lane l owns sources 64q+l and 64q+32+l of each word
// q of the group; backward, the FP64 terms are compacted to dense source lists
// (see bc_backward_item).  One grid barrier per level (two for backward levels
// with split vertices), plus the level bitmap's clear.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <memory>
#include <vector>

namespace gu {

constexpr int BC_THREADS = 512;
constexpr int BC_UNIT_COST = 512;     // edges per work unit (about)
constexpr int BC_ITEM_OVERHEAD = 16;  // an item's fixed cost, in edges

struct __align__(128) BcCtl {
    unsigned bar;
    int err;
    int max_level;  // deepest forward level over all batches
    unsigned fwork;   // forward: next work unit of the level
    int found[2];     // forward: any new bit at level j (by parity)
    unsigned work[2]; // backward: next work unit of level l (by parity)
    u64 active[2][16];  // sources with a non-empty level, by parity
};
static_assert(sizeof(BcCtl) <= 512, "control block");

// Per-phase timeline (profiling hook, same record as the batched BFS engine's):
// every CTA's thread 0 stamps its arrival at the grid barrier that ends phase
// i (atomicMax of the global timer: the slowest CTA), and CTA 0 records what
// the phase was.  Kinds, as gu_graph_level_profile reports them:
enum : int {
    BC_PHASE_INIT = 4,       // batch set-up and seeds
    BC_PHASE_FORWARD = 8,    // forward level j: new bits and sigma
    BC_PHASE_BACKWARD = 9,   // backward level l: successor sums, delta, beta
    BC_PHASE_COMBINE = 10,   // backward level l: split vertices' partial sums
    BC_PHASE_FINISH = 11,    // bc accumulation and per-source rows of the batch
    BC_PHASE_CLEAR = 12,     // forward level j: clear its level bitmap
};
constexpr size_t BC_TIMELINE_OFF = 512;
constexpr int BC_TIMELINE_MAX = 1024;
struct BcEvent {
    u64 t_last_ns;
    int32_t batch, level;
    int32_t kind, pad;
    long long pad2;
};
constexpr size_t BC_TIMELINE_BYTES = sizeof(BcEvent) * BC_TIMELINE_MAX + 16;
static_assert(BC_TIMELINE_OFF + BC_TIMELINE_BYTES <= WS_CONTROL_BYTES, "timeline must fit the control region");

__device__ __forceinline__ void record_bc_event(BcCtl *ctl, int i, bool describe, int batch, int level, int kind)
{
    BcEvent *ev = reinterpret_cast<BcEvent *>(reinterpret_cast<char *>(ctl) + BC_TIMELINE_OFF);
    if (i >= BC_TIMELINE_MAX) return;
    atomicMax(&ev[i].t_last_ns, global_timer_ns());
    if (describe) {
        ev[i].batch = batch;
        ev[i].level = level;
        ev[i].kind = kind;
        *reinterpret_cast<int *>(ev + BC_TIMELINE_MAX) = i + 1;
    }
}

enum : int { DEV_ERR_LEVELS = 3 };

struct DevChunks {
    const int32_t *v, *e0, *e1, *slot;
    int32_t nchunks;
    const int32_t *order, *ustart;
    int32_t nunits;
    const int32_t *mv, *mfirst, *mcount;
    int32_t nmulti;
};

struct BcArgs {
    const int32_t *__restrict__ R;
    const int32_t *__restrict__ C;
    const int32_t *__restrict__ RT;
    const int32_t *__restrict__ CT;
    DevChunks cin, cout;
    int32_t n;
    int32_t W;        // words per batch (1..16)
    int32_t max_lvl;  // capacity of lvl[] minus one
    const int32_t *sources;
    int32_t k;
    u64 *seen;
    u64 *lvl;
    u64 *sigma;
    double *delta;
    double *beta;  // (1 + delta) / sigma
    double *part;
    double *bc;           // nreq x n, accumulated
    const int32_t *req_start;  // nreq+1 source offsets of the requests (null: one request)
    int32_t nreq;
    int32_t *dist_rows;   // optional k x ld
    u64 *sigma_rows;      // optional k x ld
    double *delta_rows;   // optional k x ld
    int64_t ld;
    BcCtl *ctl;
    unsigned long long wait_ns;  // bound of every grid-barrier wait (gu_set_wait_limit)
};

// Takes the next (up to) K set lanes of a ballot in ascending lane order; a
// missing one is reported as -1.
template <int K>
__device__ __forceinline__ void next_lanes(unsigned &bal, int (&src)[K])
{
#pragma unroll
    for (int t = 0; t < K; ++t) {
        src[t] = bal ? __ffs(bal) - 1 : -1;
        if (bal) bal &= bal - 1;
    }
}

__device__ __forceinline__ long long gwarp() { return ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ long long nwarps() { return ((long long)gridDim.x * blockDim.x) >> 5; }

// A word group is NQ consecutive source words (NQ = min(W, 4)) handled by one
// warp item: lane l owns sources 64q+l and 64q+32+l of each word q of the group.
// The group's words of a vertex are contiguous and 8*NQ-byte aligned, so they
// move as one vector access.
template <int NQ>
__device__ __forceinline__ void ldq(const u64 *p, u64 (&x)[NQ])
{
    if constexpr (NQ == 1) {
        x[0] = __ldcg(p);
    } else if constexpr (NQ == 2) {
        const ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(p));
        x[0] = v.x;
        x[1] = v.y;
    } else {
        static_assert(NQ == 4, "word group of 1, 2 or 4 words");
        asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];"
                     : "=l"(x[0]), "=l"(x[1]), "=l"(x[2]), "=l"(x[3]) : "l"(p) : "memory");
    }
}

template <int NQ>
__device__ __forceinline__ void stq(u64 *p, const u64 (&x)[NQ])
{
    if constexpr (NQ == 1) {
        p[0] = x[0];
    } else if constexpr (NQ == 2) {
        *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(x[0], x[1]);
    } else {
        asm volatile("st.global.v4.u64 [%0], {%1, %2, %3, %4};" ::"l"(p), "l"(x[0]), "l"(x[1]), "l"(x[2]), "l"(x[3])
                     : "memory");
    }
}

template <int NQ>
__device__ __forceinline__ bool any_bits(const u64 (&x)[NQ])
{
    u64 o = 0;
#pragma unroll
    for (int t = 0; t < NQ; ++t) o |= x[t];
    return o != 0;
}

// Per-warp staging of one 32-edge slice of an adjacency range: each lane
// stores its edge's neighbour and mask, and the warp then walks the edges that
// have work with broadcast reads (no shuffles, and the masks stay out of
// registers while the loads are in flight).
template <int NQ>
struct EdgeStage {
    u64 m[NQ][32];
    int32_t v[32];
    u64 k[NQ];        // forward: ~known at w; backward: the sources at w's level
    u64 tk[NQ][32];   // triage of a work unit: lane t's item's k words
    int32_t tc[32];   // ... and the item
};

// Writes lane t's copy of x[t] (t < NQ) to dst[t] without dynamic register indexing.
template <int NQ>
__device__ __forceinline__ void lanes_store(u64 *dst, const u64 (&x)[NQ], bool invert)
{
    const int lane = lane_id();
    u64 y = 0;
#pragma unroll
    for (int t = 0; t < NQ; ++t)
        if (t == lane) y = x[t];
    if (lane < NQ) dst[lane] = invert ? ~y : y;
}

// Forward level j, word group q0..q0+NQ-1, one work item (a range of w's
// in-edges): new bits = sources of an in-neighbour's level j-1 not known at w
// (levels <= j-1); sigma(w) += sum of the in-neighbours' sigma, each lane for
// its sources, in CSR order.  seen lags one level: known = seen | lvl[j-1] is
// invariant while the first item of w folds lvl[j-1] into seen.
// act: the sources with a non-empty level j-1; new bits are ORed into found
// (both in shared memory: they stay out of registers across items).
template <int NQ>
__device__ void bc_forward_item(const BcArgs &a, EdgeStage<NQ> &st, int j, int q0, int c, u64 *found)
{
    constexpr int EPT = 4 / NQ;  // in-neighbours per trip: 8 sigma loads in flight per lane
    const int lane = lane_id();
    const int W = a.W, B = 64 * W;
    const size_t nW = (size_t)a.n * W;
    const int32_t w = __ldg(a.cin.v + c);
    const size_t wo = (size_t)w * W + q0;
    const int32_t e0 = __ldg(a.cin.e0 + c), e1 = __ldg(a.cin.e1 + c);
    const u64 *prev = a.lvl + (size_t)(j - 1) * nW + q0;
    const u64 *sig = a.sigma + 64 * q0 + lane;
    u64 acc0[NQ], acc1[NQ];
#pragma unroll
    for (int t = 0; t < NQ; ++t) acc0[t] = acc1[t] = 0;
    unsigned hit = 0;  // bit 2t+h: the lane's source 64(q0+t)+32h+lane has a predecessor
    for (int32_t eb = e0; eb < e1; eb += 32) {
        const int32_t e = eb + lane;
        bool any = false;
        if (e < e1) {
            const int32_t v = __ldg(a.CT + e);
            u64 m[NQ];
            ldq<NQ>(prev + (size_t)v * W, m);
#pragma unroll
            for (int t = 0; t < NQ; ++t) {
                m[t] &= st.k[t];
                st.m[t][lane] = m[t];
            }
            st.v[lane] = v;
            any = any_bits(m);
        }
        unsigned bal = __ballot_sync(FULL_MASK, any);
        __syncwarp();
        while (bal) {
            int src[EPT];
            next_lanes<EPT>(bal, src);
            u64 x0[EPT][NQ], x1[EPT][NQ];
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const bool ok = src[u] >= 0;
                const int sl = ok ? src[u] : 0;
                const u64 *sv = sig + (size_t)st.v[sl] * B;
#pragma unroll
                for (int t = 0; t < NQ; ++t) {
                    const u64 mm = ok ? st.m[t][sl] : 0ull;
                    const unsigned h0 = (unsigned)(mm >> lane) & 1u, h1 = (unsigned)(mm >> (lane + 32)) & 1u;
                    hit |= (h0 | (h1 << 1)) << (2 * t);
                    x0[u][t] = h0 ? __ldcg(sv + 64 * t) : 0ull;
                    x1[u][t] = h1 ? __ldcg(sv + 64 * t + 32) : 0ull;
                }
            }
#pragma unroll
            for (int u = 0; u < EPT; ++u)
#pragma unroll
                for (int t = 0; t < NQ; ++t) {
                    acc0[t] += x0[u][t];
                    acc1[t] += x1[u][t];
                }
        }
        __syncwarp();
    }
    u64 nb[NQ];
#pragma unroll
    for (int t = 0; t < NQ; ++t)
        nb[t] = (u64)__ballot_sync(FULL_MASK, (hit >> (2 * t)) & 1u) |
                ((u64)__ballot_sync(FULL_MASK, (hit >> (2 * t + 1)) & 1u) << 32);
    if (!any_bits(nb)) return;
    const bool split = __ldg(a.cin.slot + c) >= 0;
    u64 *sw = a.sigma + (size_t)w * B + 64 * q0 + lane;
    u64 *lw = a.lvl + (size_t)j * nW + wo;
#pragma unroll
    for (int t = 0; t < NQ; ++t) {
        const bool h0 = (hit >> (2 * t)) & 1u, h1 = (hit >> (2 * t + 1)) & 1u;
        if (split) {  // sigma rows of split vertices were zeroed for the batch
            if (h0) atomicAdd(sw + 64 * t, acc0[t]);
            if (h1) atomicAdd(sw + 64 * t + 32, acc1[t]);
            if (lane == 0 && nb[t]) atomicOr(lw + t, nb[t]);
        } else {
            if (h0) sw[64 * t] = acc0[t];
            if (h1) sw[64 * t + 32] = acc1[t];
        }
        if (lane == 0 && nb[t] & ~found[t]) atomicOr(found + t, nb[t]);
    }
    if (!split && lane == 0) stq<NQ>(lw, nb);
}

// Forward, one work unit of word group q0: its (up to 32) items are triaged a
// lane each -- fold lvl[j-1] into seen at a vertex's first item, and keep the
// items with an active source not yet known -- and the warp then runs those
// items one at a time.  act: the sources with a non-empty level j-1 (shared).
template <int NQ>
__device__ void bc_forward_unit(const BcArgs &a, EdgeStage<NQ> &st, int j, int q0, int u, const u64 *act, u64 *found)
{
    const int lane = lane_id();
    const int W = a.W;
    const size_t nW = (size_t)a.n * W;
    const int32_t i0 = __ldg(a.cin.ustart + u), i1 = __ldg(a.cin.ustart + u + 1);
    bool need = false;
    if (lane < i1 - i0) {
        const int32_t c = __ldg(a.cin.order + i0 + lane);
        const int32_t w = __ldg(a.cin.v + c);
        const size_t wo = (size_t)w * W + q0;
        u64 known[NQ], prevw[NQ];
        ldq<NQ>(a.lvl + (size_t)(j - 1) * nW + wo, prevw);
        ldq<NQ>(a.seen + wo, known);
        u64 nd = 0;
#pragma unroll
        for (int t = 0; t < NQ; ++t) {
            known[t] |= prevw[t];
            nd |= act[t] & ~known[t];
            st.tk[t][lane] = ~known[t];
        }
        st.tc[lane] = c;
        if (any_bits(prevw) && __ldg(a.cin.e0 + c) == __ldg(a.RT + w)) stq<NQ>(a.seen + wo, known);
        need = nd != 0;
    }
    unsigned bal = __ballot_sync(FULL_MASK, need);
    __syncwarp();
    while (bal) {
        const int t = __ffs(bal) - 1;
        bal &= bal - 1;
        if (lane < NQ) st.k[lane] = st.tk[lane][t];
        __syncwarp();
        bc_forward_item<NQ>(a, st, j, q0, st.tc[t], found);
        __syncwarp();
    }
}

// Backward dependencies are carried as beta_s(v) = (1 + delta_s(v)) / sigma_s(v):
// delta_s(w) = sigma_s(w) * sum over successors v of beta_s(v), so a successor
// costs one FP64 add and each (vertex, source) pair one division (FP64 is the
// scarce unit on this part).  finish_delta turns the successor sum S of the
// sources owned by a lane into delta and beta.
__device__ __forceinline__ void finish_delta(const BcArgs &a, size_t o, double S)
{
    const double sg = (double)__ldcg(a.sigma + o);
    const double d = sg * S;
    a.delta[o] = d;
    a.beta[o] = (1.0 + d) / sg;
}

// Backward level l, word group q0.., one work item (a range of w's out-edges):
// for the sources whose level of w is l, sum beta over successors v (level
// l+1) in CSR order.  Unsplit vertices finish delta/beta directly; split ones
// store per-item partial sums, added in item order by bc_combine_item after a
// barrier.
//
// FP64 instructions are the scarce resource here (a warp instruction costs the
// same however few of its lanes have work), so the sums live in shared memory,
// one per source of the group, and the adds are compacted: for each successor
// the set bits of its mask become a dense list of sources, and a warp
// instruction adds 32 of them.  Each source still receives its successors'
// terms one at a time in CSR order (a successor's list holds a source at most
// once, and successive lists are separated by __syncwarp), so the sums are the
// sequential CSR-order sums.
template <int NQ>
struct SumStage {
    double acc[64 * NQ];
    unsigned char pos[4][64 * NQ];  // dense source lists of up to four successors
};

// Writes the positions (0 .. 64*NQ-1) of the set bits of m into list in
// ascending order; returns how many there are.
template <int NQ>
__device__ __forceinline__ int compact_bits(const u64 (&m)[NQ], unsigned char *list)
{
    const int lane = lane_id();
    const unsigned below = (1u << lane) - 1u;
    int base = 0;
#pragma unroll
    for (int t = 0; t < NQ; ++t) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const unsigned x = (unsigned)(m[t] >> (32 * h));
            if ((x >> lane) & 1u) list[base + __popc(x & below)] = (unsigned char)(64 * t + 32 * h + lane);
            base += __popc(x);
        }
    }
    return base;
}

template <int NQ>
__device__ void bc_backward_item(const BcArgs &a, EdgeStage<NQ> &st, SumStage<NQ> &ss, int l, int L, int q0, int c)
{
    const int lane = lane_id();
    const int W = a.W, B = 64 * W;
    const size_t nW = (size_t)a.n * W;
    const int32_t w = __ldg(a.cout.v + c);
#pragma unroll
    for (int t = 0; t < 2 * NQ; ++t) ss.acc[32 * t + lane] = 0.0;
    __syncwarp();
    if (l < L) {
        const u64 *next = a.lvl + (size_t)(l + 1) * nW + q0;
        const double *bet = a.beta + 64 * q0;
        const int32_t e0 = __ldg(a.cout.e0 + c), e1 = __ldg(a.cout.e1 + c);
        for (int32_t eb = e0; eb < e1; eb += 32) {
            const int32_t e = eb + lane;
            bool any = false;
            if (e < e1) {
                const int32_t v = __ldg(a.C + e);
                u64 m[NQ];
                ldq<NQ>(next + (size_t)v * W, m);
#pragma unroll
                for (int t = 0; t < NQ; ++t) {
                    m[t] &= st.k[t];
                    st.m[t][lane] = m[t];
                }
                st.v[lane] = v;
                any = any_bits(m);
            }
            unsigned bal = __ballot_sync(FULL_MASK, any);
            __syncwarp();
            while (bal) {  // up to four successors at a time, in CSR order
                int src[4];
                next_lanes<4>(bal, src);
                int cnt[4], cum[4], rounds = 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    cnt[u] = 0;
                    if (src[u] >= 0) {
                        u64 mm[NQ];
#pragma unroll
                        for (int t = 0; t < NQ; ++t) mm[t] = st.m[t][src[u]];
                        cnt[u] = compact_bits<NQ>(mm, ss.pos[u]);
                    }
                    rounds += (cnt[u] + 31) >> 5;
                    cum[u] = rounds;
                }
                __syncwarp();
                for (int r0 = 0; r0 < rounds; r0 += 4) {
                    double b[4];
                    int s[4];
#pragma unroll
                    for (int z = 0; z < 4; ++z) {  // four loads in flight per lane
                        const int rr = r0 + z;
                        const int u = (rr >= cum[0]) + (rr >= cum[1]) + (rr >= cum[2]);
                        const int first = u == 0 ? 0 : u == 1 ? cum[0] : u == 2 ? cum[1] : cum[2];
                        const int n_u = u == 0 ? cnt[0] : u == 1 ? cnt[1] : u == 2 ? cnt[2] : cnt[3];
                        const int s_u = u == 0 ? src[0] : u == 1 ? src[1] : u == 2 ? src[2] : src[3];
                        const int i = 32 * (rr - first) + lane;
                        s[z] = -1;
                        b[z] = 0.0;
                        if (rr < rounds && i < n_u) {
                            s[z] = ss.pos[u][i];
                            b[z] = __ldcg(bet + (size_t)st.v[s_u] * B + s[z]);
                        }
                    }
#pragma unroll
                    for (int z = 0; z < 4; ++z) {
                        if (s[z] >= 0) ss.acc[s[z]] += b[z];
                        __syncwarp();
                    }
                }
            }
            __syncwarp();
        }
    }
    // the sources of w at level l, densely: one division per source
    u64 lm[NQ];
#pragma unroll
    for (int t = 0; t < NQ; ++t) lm[t] = st.k[t];
    const int cnt = compact_bits<NQ>(lm, ss.pos[0]);
    __syncwarp();
    const int32_t slot = __ldg(a.cout.slot + c);
    for (int i = lane; i < cnt; i += 32) {
        const int s = ss.pos[0][i];
        const double S = ss.acc[s];
        if (slot >= 0) a.part[((size_t)slot * W + q0) * 64 + s] = S;
        else finish_delta(a, (size_t)w * B + 64 * q0 + s, S);
    }
    __syncwarp();
}

// Backward, one work unit of word group q0: lanes triage its items (keep those
// whose vertex has a source at level l), then the warp runs them in turn.
template <int NQ>
__device__ void bc_backward_unit(const BcArgs &a, EdgeStage<NQ> &st, SumStage<NQ> &ss, int l, int L, int q0, int u)
{
    const int lane = lane_id();
    const int W = a.W;
    const size_t nW = (size_t)a.n * W;
    const int32_t i0 = __ldg(a.cout.ustart + u), i1 = __ldg(a.cout.ustart + u + 1);
    bool need = false;
    if (lane < i1 - i0) {
        const int32_t c = __ldg(a.cout.order + i0 + lane);
        u64 lm[NQ];
        ldq<NQ>(a.lvl + (size_t)l * nW + (size_t)__ldg(a.cout.v + c) * W + q0, lm);
#pragma unroll
        for (int t = 0; t < NQ; ++t) st.tk[t][lane] = lm[t];
        st.tc[lane] = c;
        need = any_bits(lm);
    }
    unsigned bal = __ballot_sync(FULL_MASK, need);
    __syncwarp();
    while (bal) {
        const int t = __ffs(bal) - 1;
        bal &= bal - 1;
        if (lane < NQ) st.k[lane] = st.tk[lane][t];
        __syncwarp();
        bc_backward_item<NQ>(a, st, ss, l, L, q0, st.tc[t]);
        __syncwarp();
    }
}

// delta of a split vertex = its items' partials added in item order, for the
// vertex's sources at level l taken densely.
template <int NQ>
__device__ void bc_combine_item(const BcArgs &a, EdgeStage<NQ> &st, SumStage<NQ> &ss, int l, int q0, int i)
{
    const int lane = lane_id();
    const int W = a.W, B = 64 * W;
    const size_t nW = (size_t)a.n * W;
    const int32_t w = __ldg(a.cout.mv + i);
    u64 lm[NQ];
    ldq<NQ>(a.lvl + (size_t)l * nW + (size_t)w * W + q0, lm);
    if (!any_bits(lm)) return;
    const int cnt = compact_bits<NQ>(lm, ss.pos[0]);
    __syncwarp();
    const int32_t c0 = __ldg(a.cout.mfirst + i), nc = __ldg(a.cout.mcount + i);
    for (int k = lane; k < cnt; k += 32) {
        const int s = ss.pos[0][k];
        double S = 0.0;
        for (int32_t c = c0; c < c0 + nc; ++c)
            S += __ldcg(a.part + ((size_t)__ldg(a.cout.slot + c) * W + q0) * 64 + s);
        finish_delta(a, (size_t)w * B + 64 * q0 + s, S);
    }
    __syncwarp();
    (void)st;
}

// bc_r[w] += sum of delta over the batch's sources of request r whose level of
// w is >= 1, as a fixed-shape tree: each lane sums its own sources word by
// word, then a butterfly over the 32 lanes.  Requests own contiguous source
// ranges (one request when req_start is null).
__device__ __forceinline__ u64 range_bits(int q, int lo, int hi)
{
    // bits p of word q with lo <= 64q + p < hi
    const int a = max(lo - 64 * q, 0), b = min(hi - 64 * q, 64);
    if (b <= a) return 0ull;
    const u64 upto = b >= 64 ? ~0ull : ((1ull << b) - 1ull);
    return upto & ~((1ull << a) - 1ull);
}

__device__ void bc_accumulate_item(const BcArgs &a, int32_t w, int row0, int nb)
{
    const int lane = lane_id();
    const int B = 64 * a.W;
    int r = 0;
    if (a.req_start) {  // first request ending after row0
        int lo = 0, hi = a.nreq - 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(a.req_start + mid + 1) > row0) hi = mid;
            else lo = mid + 1;
        }
        r = lo;
    }
    for (; r < a.nreq; ++r) {
        const int rs = a.req_start ? __ldg(a.req_start + r) : 0;
        const int re = a.req_start ? __ldg(a.req_start + r + 1) : a.k;
        if (rs >= row0 + nb) break;
        const int lo = max(rs, row0) - row0, hi = min(re, row0 + nb) - row0;
        if (hi <= lo) continue;
        double s = 0.0;
        for (int q = 0; q < a.W && 64 * q < nb; ++q) {
            const u64 counted = __ldcg(a.seen + (size_t)w * a.W + q) & ~__ldcg(a.lvl + (size_t)w * a.W + q) &
                                range_bits(q, lo, hi);
            const double *dw = a.delta + (size_t)w * B + 64 * q;
            if ((counted >> lane) & 1ull) s += __ldcg(dw + lane);
            if ((counted >> (lane + 32)) & 1ull) s += __ldcg(dw + lane + 32);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
        if (lane == 0) a.bc[(size_t)r * a.n + w] += s;
    }
}

// Optional per-source rows (dist, sigma, delta) of this batch: lane l writes
// vertex w for sources 64q+l and 64q+l+32; levels from the level bitmaps.
__device__ void bc_rows_item(const BcArgs &a, int32_t w, int q, int row0, int nb, int maxl)
{
    const int lane = lane_id();
    const int B = 64 * a.W;
    const size_t nW = (size_t)a.n * a.W;
    const u64 seen = __ldcg(a.seen + (size_t)w * a.W + q);
    const u64 lvl0 = __ldcg(a.lvl + (size_t)w * a.W + q);
    for (int h = 0; h < 2; ++h) {
        const int bit = lane + 32 * h;
        if (64 * q + bit >= nb) continue;
        const int row = row0 + 64 * q + bit;
        const bool reached = (seen >> bit) & 1ull;
        int32_t level = INT_MAX;
        if (reached && a.dist_rows) {
            for (int l = 0; l <= maxl; ++l)
                if ((__ldcg(a.lvl + (size_t)l * nW + (size_t)w * a.W + q) >> bit) & 1ull) {
                    level = l;
                    break;
                }
        }
        const size_t o = (size_t)w * B + 64 * q + bit;
        if (a.dist_rows) a.dist_rows[(int64_t)row * a.ld + w] = level;
        if (a.sigma_rows) a.sigma_rows[(int64_t)row * a.ld + w] = reached ? __ldcg(a.sigma + o) : 0ull;
        if (a.delta_rows) {
            const bool is_src = (lvl0 >> bit) & 1ull;
            a.delta_rows[(int64_t)row * a.ld + w] = (reached && !is_src) ? __ldcg(a.delta + o) : 0.0;
        }
    }
}

// NQ = words per work item: min(W, 4).
template <int NQ>
__global__ void __launch_bounds__(BC_THREADS, 2) bc_grid_kernel(BcArgs a, int do_backward)
{
    __shared__ u64 s_act[16];
    __shared__ EdgeStage<NQ> s_stage[BC_THREADS / 32];
    extern __shared__ __align__(16) unsigned char s_dyn[];  // SumStage<NQ> per warp (backward only)
    SumStage<NQ> *s_sum = reinterpret_cast<SumStage<NQ> *>(s_dyn);
    __shared__ BcCtl s_ctl;  // control block as read by thread 0 after each barrier
    unsigned epoch = 0;
    BcCtl *ctl = a.ctl;
    int phase = 0;  // timeline entry of the current phase
    int batch = 0;
    auto barrier = [&](int kind, int level) {
        if (threadIdx.x == 0) record_bc_event(ctl, phase, blockIdx.x == 0, batch, level, kind);
        ++phase;
        return grid_barrier(&ctl->bar, &ctl->err, epoch, a.wait_ns, reinterpret_cast<const u64 *>(ctl),
                            reinterpret_cast<u64 *>(&s_ctl),
                            (int)(sizeof(BcCtl) / sizeof(u64)));
    };
    const long long rank = (long long)blockIdx.x * blockDim.x + threadIdx.x, size = (long long)gridDim.x * blockDim.x;
    const int W = a.W, B = 64 * W;
    const size_t nW = (size_t)a.n * W;
    const int nbatch = (a.k + B - 1) / B;
    for (long long i = rank; i < (long long)a.nreq * a.n; i += size) a.bc[i] = 0.0;
    if (threadIdx.x < 16) s_act[threadIdx.x] = 0;
    for (int b = 0; b < nbatch; ++b) {
        batch = b;
        const int row0 = b * B;
        const int nb = min(B, a.k - row0);
        for (size_t i = (size_t)rank; i < nW; i += (size_t)size) {
            a.seen[i] = 0;
            a.lvl[i] = 0;
        }
        // sigma rows of split vertices are accumulated with atomics: clear them
        for (long long i = rank; i < (long long)a.cin.nmulti * B; i += size)
            a.sigma[(size_t)__ldg(a.cin.mv + i / B) * B + (i % B)] = 0ull;
        if (rank == 0) {
            ctl->work[0] = ctl->work[1] = 0;
            ctl->found[0] = ctl->found[1] = 0;
            for (int q = 0; q < 16; ++q) ctl->active[0][q] = ctl->active[1][q] = 0;
        }
        if (!barrier(BC_PHASE_INIT, 0)) return;
        if (rank < nb) {
            const int32_t s = __ldg(a.sources + row0 + rank);
            const int q = (int)rank >> 6;
            const u64 bit = 1ull << (rank & 63);
            atomicOr(a.lvl + (size_t)s * W + q, bit);
            a.sigma[(size_t)s * B + rank] = 1ull;
            atomicOr(&ctl->active[0][q], bit);
        }
        if (!barrier(BC_PHASE_INIT, 0)) return;
        // forward levels
        int L = 0;
        for (int j = 1;; ++j) {
            if (j > a.max_lvl) {
                if (rank == 0) atomicCAS(&ctl->err, 0, (int)DEV_ERR_LEVELS);
                barrier(BC_PHASE_INIT, j);
                return;
            }
            for (size_t i = (size_t)rank; i < nW; i += (size_t)size) a.lvl[(size_t)j * nW + i] = 0;
            if (rank == 0) {
                ctl->fwork = 0;
                ctl->found[j & 1] = 0;
                for (int q = 0; q < 16; ++q) ctl->active[j & 1][q] = 0;
            }
            if (!barrier(BC_PHASE_CLEAR, j)) return;
            // work units of all word groups, taken dynamically (unit x = group x / nunits)
            const long long nfw = (long long)(W / NQ) * a.cin.nunits;
            // warps beyond the unit count have nothing to take (on a small graph most
            // of the grid): they skip the shared counter instead of queueing on it
            for (; gwarp() < nfw;) {
                long long x = 0;
                if (lane_id() == 0) x = atomicAdd(&ctl->fwork, 1u);
                x = __shfl_sync(FULL_MASK, x, 0);
                if (x >= nfw) break;
                const int q0 = (int)(x / a.cin.nunits) * NQ;
                bc_forward_unit<NQ>(a, s_stage[warp_in_block()], j, q0, (int)(x % a.cin.nunits),
                                    &s_ctl.active[(j - 1) & 1][q0], &s_act[q0]);
            }
            __syncthreads();
            if (threadIdx.x < W && s_act[threadIdx.x]) {
                atomicOr(&ctl->active[j & 1][threadIdx.x], s_act[threadIdx.x]);
                atomicOr(&ctl->found[j & 1], 1);
                s_act[threadIdx.x] = 0;
            }
            if (!barrier(BC_PHASE_FORWARD, j)) return;
            if (s_ctl.found[j & 1] == 0) {
                L = j - 1;  // this pass also folded lvl[L] into seen
                break;
            }
        }
        if (rank == 0 && L > ctl->max_level) ctl->max_level = L;
        if (do_backward) {
            for (int l = L; l >= 1; --l) {
                if (rank == 0) ctl->work[(l - 1) & 1] = 0;  // level l-1's counter (last used by level l+1)
                const long long nbw = (long long)(W / NQ) * a.cout.nunits;
                for (; gwarp() < nbw;) {
                    long long x = 0;
                    if (lane_id() == 0) x = atomicAdd(&ctl->work[l & 1], 1u);
                    x = __shfl_sync(FULL_MASK, x, 0);
                    if (x >= nbw) break;
                    bc_backward_unit<NQ>(a, s_stage[warp_in_block()], s_sum[warp_in_block()], l, L,
                                         (int)(x / a.cout.nunits) * NQ, (int)(x % a.cout.nunits));
                }
                if (!barrier(BC_PHASE_BACKWARD, l)) return;
                if (a.cout.nmulti) {
                    for (int q0 = 0; q0 < W; q0 += NQ)
                        for (long long i = gwarp(); i < a.cout.nmulti; i += nwarps())
                            bc_combine_item<NQ>(a, s_stage[warp_in_block()], s_sum[warp_in_block()], l, q0, (int)i);
                    if (!barrier(BC_PHASE_COMBINE, l)) return;
                }
            }
            for (long long w = gwarp(); w < a.n; w += nwarps()) bc_accumulate_item(a, (int32_t)w, row0, nb);
        }
        if (a.dist_rows || a.sigma_rows || a.delta_rows) {
            for (int q = 0; q < W; ++q)
                for (long long w = gwarp(); w < a.n; w += nwarps()) bc_rows_item(a, (int32_t)w, q, row0, nb, L);
        }
        if (!barrier(BC_PHASE_FINISH, 0)) return;
    }
}

// ---- host ----------------------------------------------------------------------------
static void build_chunks(DeviceGraph &g, const std::vector<int32_t> &R, ChunkMap &cm)
{
    const int32_t n = g.n;
    std::vector<int32_t> v, e0, e1, slot, mv, mfirst, mcount;
    int32_t nslots = 0;
    for (int32_t w = 0; w < n; ++w) {
        const int32_t a = R[w], b = R[w + 1];
        const int32_t nc = b > a ? (b - a + BC_CHUNK_EDGES - 1) / BC_CHUNK_EDGES : 1;
        if (nc > 1) {
            mv.push_back(w);
            mfirst.push_back((int32_t)v.size());
            mcount.push_back(nc);
        }
        for (int32_t c = 0; c < nc; ++c) {
            v.push_back(w);
            e0.push_back(a + c * BC_CHUNK_EDGES);
            e1.push_back(std::min(b, a + (c + 1) * BC_CHUNK_EDGES));
            slot.push_back(nc > 1 ? nslots++ : -1);
        }
    }
    auto up = [&](const std::vector<int32_t> &src, int32_t *&dst) {
        if (src.empty()) return;
        GU_CUDA_CHECK(dev_malloc((void **)&dst, sizeof(int32_t) * src.size()));
        g.extra_allocs.push_back(dst);
        GU_CUDA_CHECK(cudaMemcpy(dst, src.data(), sizeof(int32_t) * src.size(), cudaMemcpyHostToDevice));
        g.bytes += sizeof(int32_t) * src.size();
    };
    // work units: items by descending edge count (heavy items are taken first,
    // light ones fill the gaps), cut into runs of at most 32 items and about
    // BC_UNIT_COST edges (an item counts its edges plus a fixed overhead) -- or
    // less on a small graph, so that there are at least four units per warp of
    // the grid (down to one item per unit) and no level runs on a few warps
    std::vector<int32_t> order(v.size()), ustart;
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int32_t)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return e1[x] - e0[x] > e1[y] - e0[y]; });
    long long total_cost = 0;
    for (size_t i = 0; i < v.size(); ++i) total_cost += e1[i] - e0[i] + BC_ITEM_OVERHEAD;
    const long long warps = (long long)std::max(g.sm_count, 1) * 2 * (BC_THREADS / 32);
    const long long unit_cost = std::max<long long>(1, std::min<long long>(BC_UNIT_COST, total_cost / (4 * warps)));
    long long cost = 0;
    int cnt = 0;
    for (size_t i = 0; i < order.size(); ++i) {
        if (cnt == 0) ustart.push_back((int32_t)i);
        cost += e1[order[i]] - e0[order[i]] + BC_ITEM_OVERHEAD;
        if (++cnt == 32 || cost >= unit_cost) cost = cnt = 0;
    }
    ustart.push_back((int32_t)order.size());
    up(order, cm.order);
    up(ustart, cm.ustart);
    cm.nunits = (int32_t)ustart.size() - 1;
    up(v, cm.v);
    up(e0, cm.e0);
    up(e1, cm.e1);
    up(slot, cm.slot);
    up(mv, cm.mv);
    up(mfirst, cm.mfirst);
    up(mcount, cm.mcount);
    cm.nchunks = (int32_t)v.size();
    cm.nmulti = (int32_t)mv.size();
    cm.nslots = nslots;
    cm.built = true;
}

static void ensure_chunks(DeviceGraph &g)
{
    if (!g.bc_out.built) build_chunks(g, g.host_R, g.bc_out);
    if (!g.bc_in.built) {
        if (g.directed) build_chunks(g, g.host_RT, g.bc_in);
        else g.bc_in = g.bc_out;
    }
}

static int bc_words_for(int32_t k, int requested)
{
    int W = requested;
    if (W <= 0) {
        const char *s = std::getenv("GU_BC_WORDS");
        W = (s && *s) ? std::atoi(s) : 4;
    }
    if (W != 1 && W != 2 && W != 4 && W != 8 && W != 16)
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "BC batch must be 64, 128, 256, 512 or 1024 sources");
    while (W > 1 && 64 * (W / 2) >= k) W /= 2;  // no wider than the request needs
    return W;
}

static DevChunks dev_chunks(const ChunkMap &c)
{
    DevChunks d;
    d.v = c.v;
    d.e0 = c.e0;
    d.e1 = c.e1;
    d.slot = c.slot;
    d.nchunks = c.nchunks;
    d.order = c.order;
    d.ustart = c.ustart;
    d.nunits = c.nunits;
    d.mv = c.mv;
    d.mfirst = c.mfirst;
    d.mcount = c.mcount;
    d.nmulti = c.nmulti;
    return d;
}

struct BcLayout {
    int W;
    size_t words, sig, del, prt, bcb, maxl, total;
};

// Level store: levels 0..maxl-1 (a BFS level is at most n - 1); 512 MiB of
// level bitmaps by default, at least 64 levels (GU_BC_LEVEL_BUDGET_MB overrides).
static BcLayout bc_layout(const DeviceGraph &g, int32_t k, int batch, bool backward, int nslots)
{
    if (batch > 0 && batch % 64) throw gu_error(GU_ERR_INVALID_ARGUMENT, "batch must be a multiple of 64");
    BcLayout L;
    L.W = bc_words_for(k, batch > 0 ? batch / 64 : 0);
    const size_t n = (size_t)g.n, B = 64 * (size_t)L.W;
    auto up = [](size_t x) { return ((x + 255) / 256) * 256; };
    L.words = up(n * L.W * sizeof(u64));
    L.sig = up(n * B * sizeof(u64));
    L.del = backward ? 2 * up(n * B * sizeof(double)) : 0;  // delta and beta
    L.prt = backward ? up((size_t)nslots * L.W * 64 * sizeof(double)) : 0;
    L.bcb = up(n * sizeof(double));
    size_t budget = (size_t)512 << 20;
    if (const char *s = std::getenv("GU_BC_LEVEL_BUDGET_MB")) budget = (size_t)std::atoll(s) << 20;
    L.maxl = budget / (L.words ? L.words : 1);
    if (L.maxl < 64) L.maxl = 64;
    if (L.maxl > n + 1) L.maxl = n + 1;
    if (L.maxl < 2) L.maxl = 2;
    L.total = WS_CONTROL_BYTES + L.words + L.maxl * L.words + L.sig + L.del + L.prt + L.bcb;
    return L;
}

size_t bc_workspace_bytes(const DeviceGraph &g, int32_t k, int batch, bool backward)
{
    // the split-vertex slot count is known once the work items exist; bound it by m / 256 + n
    const int nslots = g.bc_out.built ? g.bc_out.nslots : (int)(g.m / BC_CHUNK_EDGES + g.n);
    return bc_layout(g, k, batch, backward, nslots).total;
}

void launch_bc(DeviceGraph &g, const int32_t *sources, int32_t k, const BcOptions &opt, double *bc, int32_t *dist_rows,
               uint64_t *sigma_rows, double *delta_rows, int64_t ld, bool backward, cudaStream_t stream)
{
    ensure_chunks(g);
    const BcLayout Lay = bc_layout(g, k, opt.batch, backward, g.bc_out.nslots);
    const int W = Lay.W;
    const size_t words = Lay.words, sig = Lay.sig, del = Lay.del, prt = Lay.prt, maxl = Lay.maxl;
    Workspace &wsp = opt.ws ? *opt.ws : g.ws;
    char *ws = (char *)wsp.get(Lay.total);
    BcArgs a;
    a.R = g.R;
    a.C = g.C;
    a.RT = g.RT;
    a.CT = g.CT;
    a.cin = dev_chunks(g.bc_in);
    a.cout = dev_chunks(g.bc_out);
    a.n = g.n;
    a.W = W;
    a.max_lvl = (int32_t)(maxl - 1);
    a.sources = sources;
    a.k = k;
    char *p = ws;
    a.ctl = reinterpret_cast<BcCtl *>(p);
    a.wait_ns = wait_limit_ns();
    p += WS_CONTROL_BYTES;
    a.seen = reinterpret_cast<u64 *>(p);
    p += words;
    a.lvl = reinterpret_cast<u64 *>(p);
    p += maxl * words;
    a.sigma = reinterpret_cast<u64 *>(p);
    p += sig;
    a.delta = backward ? reinterpret_cast<double *>(p) : nullptr;
    a.beta = backward ? reinterpret_cast<double *>(p + del / 2) : nullptr;
    p += del;
    a.part = backward ? reinterpret_cast<double *>(p) : nullptr;
    p += prt;
    a.bc = bc ? bc : reinterpret_cast<double *>(p);
    a.req_start = opt.req_start;
    a.nreq = opt.req_start ? opt.nreq : 1;
    if (!bc && a.nreq != 1) throw gu_error(GU_ERR_INTERNAL, "per-request bc needs an output");
    a.dist_rows = dist_rows;
    a.sigma_rows = reinterpret_cast<u64 *>(sigma_rows);
    a.delta_rows = delta_rows;
    a.ld = ld;
    GU_CUDA_CHECK(cudaMemsetAsync(a.ctl, 0, BC_TIMELINE_OFF + BC_TIMELINE_BYTES, stream));
    const void *kern = W == 1 ? (const void *)bc_grid_kernel<1>
                       : W == 2 ? (const void *)bc_grid_kernel<2> : (const void *)bc_grid_kernel<4>;
    const int ki = W == 1 ? 0 : W == 2 ? 1 : 2;
    const size_t dyn = (size_t)(BC_THREADS / 32) * (W == 1   ? sizeof(SumStage<1>)
                                                    : W == 2 ? sizeof(SumStage<2>)
                                                             : sizeof(SumStage<4>));
    static int occupancy[3] = {-1, -1, -1};
    int &blocks_per_sm = occupancy[ki];
    if (blocks_per_sm < 0) {
        GU_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, BC_THREADS, dyn));
        if (blocks_per_sm < 1) throw gu_error(GU_ERR_INTERNAL, "bc kernel cannot be resident");
    }
    int nblocks = g.sm_count * blocks_per_sm;
    if (opt.max_blocks > 0 && nblocks > opt.max_blocks) nblocks = opt.max_blocks;
    dim3 grid(nblocks), block(BC_THREADS);
    int do_backward = backward ? 1 : 0;
    void *params[] = {&a, &do_backward};
    if (&wsp == &g.ws) g.timeline = 1;
    if (opt.timed) g.mark_start(stream);
    GU_CUDA_CHECK(cudaLaunchCooperativeKernel(kern, grid, block, params, dyn, stream));
    if (opt.timed) g.mark_stop(stream);
}

int bc_ws_error(const Workspace &ws)
{
    BcCtl c;
    GU_CUDA_CHECK(cudaMemcpy(&c, ws.ptr, sizeof(BcCtl), cudaMemcpyDeviceToHost));
    return c.err;
}

// Copies the per-phase timeline of the last BC launch on the graph's workspace
// (after a stream sync); frontier sizes are not recorded (reported as 0).
int bc_read_timeline(DeviceGraph &g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                     int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms)
{
    std::vector<char> buf(BC_TIMELINE_BYTES);
    GU_CUDA_CHECK(cudaMemcpy(buf.data(), (char *)g.ws.ptr + BC_TIMELINE_OFF, BC_TIMELINE_BYTES, cudaMemcpyDeviceToHost));
    const BcEvent *ev = reinterpret_cast<const BcEvent *>(buf.data());
    const int cnt = *reinterpret_cast<const int *>(ev + BC_TIMELINE_MAX);
    const int nout = cnt < max_entries ? cnt : max_entries;
    for (int i = 0; i < nout; ++i) {
        if (batch) batch[i] = ev[i].batch;
        if (level) level[i] = ev[i].level;
        if (kind) kind[i] = ev[i].kind;
        if (frontier_vertices) frontier_vertices[i] = 0;
        if (frontier_edges) frontier_edges[i] = 0;
        if (t_ms) t_ms[i] = (double)(ev[i].t_last_ns - ev[0].t_last_ns) * 1e-6;
    }
    return nout;
}

void bc_read_status(DeviceGraph &g, int *dev_err, int *max_level)
{
    BcCtl c;
    GU_CUDA_CHECK(cudaMemcpy(&c, g.ws.ptr, sizeof(BcCtl), cudaMemcpyDeviceToHost));
    if (dev_err) *dev_err = c.err;
    if (max_level) *max_level = c.max_level;
}

}  // namespace gu
