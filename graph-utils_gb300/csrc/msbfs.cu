// msbfs.cu -- batched multi-source BFS on sm_103a.
//
// One persistent, cooperatively launched kernel runs every batch of 64 sources
// and every level of each batch; levels are separated by a bounded grid barrier
// (device_utils.cuh), so a whole multi-source search is a single launch.
//
// Per vertex the engine keeps one 32-byte record (one DRAM sector / L2 sector):
//   seen  : sources that have reached the vertex in an earlier level
//   f[3]  : frontier bitmaps F_j, rotating over three levels
// Bit i of every word stands for source row0+i of the current batch.  For a
// batch of 64 sources and n = 2^20 the records take 32 MiB and stay in the
// 126 MiB L2, so the random per-edge accesses are L2 hits; DRAM traffic is the
// streamed CSR plus the distance rows.
//
// Phase j of a batch (one barrier per level):
//   * finalise F_{j-1}: seen |= F_{j-1} and write distance j-1 for its bits
//     (lazily, so that readers use seen|F_{j-1}, which is invariant in the phase)
//   * clear F_{j-2}
//   * discover F_j either top-down (gather the adjacency of the F_{j-1} queue
//     with the variant's strategy; claim bits with 64-bit atomicOr on the
//     L2-resident record, append a vertex to the F_j queue when its word goes
//     from zero to non-zero) or bottom-up (every not-fully-seen vertex ORs its
//     in-neighbours' F_{j-1} words, stopping when all batch bits are covered).
// Direction choice follows Beamer et al. (SC'12): top-down -> bottom-up when the
// frontier's edges exceed the unexplored edges / alpha, back when the frontier
// holds fewer than n / beta vertices.
//
// Gather strategies restate the reference's kernels' neighbour-gathering ideas
// for warp-synchronous sm_103a code (file:line in include/gu.h).
#include "device_utils.cuh"
#include "gu_internal.h"

#include <climits>

namespace gu {

struct __align__(32) VState {
    u64 seen;
    u64 f[3];
};

// Control block of one launch; slots rotate over four levels (see ms_kernel).
struct __align__(128) MsCtl {
    unsigned bar;
    int err;
    int td_levels;
    int bu_levels;
    int qlen[4];
    int work[4];
    u64 qedges[4];
    u64 fulledges[4];
    int max_level;
    int pad[3];
};

struct MsArgs {
    const int32_t *__restrict__ R;
    const int32_t *__restrict__ C;
    const int32_t *__restrict__ RT;
    const int32_t *__restrict__ CT;
    const int32_t *__restrict__ F;
    int32_t n;
    int64_t m;
    const int32_t *sources;
    int32_t k;
    int32_t *dist;
    int64_t ld;
    VState *vs;
    int32_t *q[3];
    MsCtl *ctl;
    float alpha, beta;
};

struct Lvl {
    int cur, nxt, prv, slot;
    int qlen, qlen_prev;
    const int32_t *qcur;
    int32_t *qnxt;
    const int32_t *qprev;
    int32_t lev;  // distance value of F_{j-1}
    int row0;
    u64 full;
};

constexpr int MS_THREADS = 512;
constexpr int CTA_DEGREE_THRESHOLD = 2048;  // CTA_warp.cu:44
constexpr unsigned DEG_CAP = 1u << 26;      // keeps warp sums of degrees in 32 bits

struct GridG {
    __device__ static long long rank() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ static long long size() { return (long long)gridDim.x * blockDim.x; }
    __device__ static int blk() { return blockIdx.x; }
    __device__ static int nblk() { return gridDim.x; }
};

__device__ __forceinline__ unsigned capped_degree(const int32_t *R, int32_t v)
{
    unsigned d = (unsigned)(__ldg(R + v + 1) - __ldg(R + v));
    return d < DEG_CAP ? d : DEG_CAP;
}

__device__ __forceinline__ void warp_add_u64(u64 *p, unsigned x)
{
    const unsigned mask = __activemask();
    const unsigned tot = __reduce_add_sync(mask, x);
    if (lane_id() == __ffs(mask) - 1) atomicAdd(p, (u64)tot);
}

// ---- distance writes -------------------------------------------------------
__device__ __forceinline__ void write_bits_serial(int32_t *dist, int64_t ld, int row0, int32_t v, u64 bits,
                                                  int32_t val)
{
    while (bits) {
        const int i = __ffsll((long long)bits) - 1;
        bits &= bits - 1;
        dist[(int64_t)(row0 + i) * ld + v] = val;
    }
}

// Lanes hold consecutive vertices: for each source bit the stores of the warp
// fall into one contiguous row segment.
__device__ __forceinline__ void write_bits_sweep(int32_t *dist, int64_t ld, int row0, int32_t v, u64 bits,
                                                 int32_t val)
{
    u64 u = warp_or_u64(FULL_MASK, bits);
    while (u) {
        const int i = __ffsll((long long)u) - 1;
        u &= u - 1;
        if ((bits >> i) & 1ull) dist[(int64_t)(row0 + i) * ld + v] = val;
    }
}

template <class G>
__device__ void init_dist_rows(int32_t *dist, int64_t ld, int row0, int nb, int32_t n)
{
    const long long rank = G::rank(), size = G::size();
    if ((ld & 3) == 0 && (((uintptr_t)dist) & 15) == 0) {
        const long long n4 = n >> 2;
        const long long tot = (long long)nb * n4;
        const int4 inf4 = make_int4(INT_MAX, INT_MAX, INT_MAX, INT_MAX);
        for (long long idx = rank; idx < tot; idx += size) {
            const long long r = idx / n4, c = idx - r * n4;
            reinterpret_cast<int4 *>(dist + (int64_t)(row0 + r) * ld)[c] = inf4;
        }
        const int tail = n & 3;
        for (long long idx = rank; idx < (long long)nb * tail; idx += size) {
            const long long r = idx / tail, c = idx - r * tail;
            dist[(int64_t)(row0 + r) * ld + (n4 << 2) + c] = INT_MAX;
        }
    } else {
        const long long tot = (long long)nb * n;
        for (long long idx = rank; idx < tot; idx += size) {
            const long long r = idx / n, c = idx - r * n;
            dist[(int64_t)(row0 + r) * ld + c] = INT_MAX;
        }
    }
}

// ---- top-down visit: frontier bits f arrive at vertex w over one edge ------
__device__ __forceinline__ void td_visit(const MsArgs &a, const Lvl &L, u64 f, int32_t w)
{
    VState *s = a.vs + w;
    const u64 known = __ldcg(&s->seen) | __ldcg(&s->f[L.cur]) | __ldcg(&s->f[L.nxt]);
    const u64 nb = f & ~known;
    if (nb) {
        const u64 old = atomicOr(&s->f[L.nxt], nb);
        if (old == 0) warp_append(w, L.qnxt, &a.ctl->qlen[L.slot], &a.ctl->qedges[L.slot], capped_degree(a.R, w));
    }
}

// Finalise F_{j-1} (queue order) and clear F_{j-2}.
template <class G>
__device__ void td_update(const MsArgs &a, const Lvl &L)
{
    const long long rank = G::rank(), size = G::size();
    for (long long i = rank; i < L.qlen; i += size) {
        const int32_t v = __ldcg(L.qcur + i);
        VState *s = a.vs + v;
        const u64 f = __ldcg(&s->f[L.cur]);
        const u64 sn = __ldcg(&s->seen) | f;
        s->seen = sn;
        if (sn == L.full) warp_add_u64(&a.ctl->fulledges[L.slot], capped_degree(a.R, v));
        write_bits_serial(a.dist, a.ld, L.row0, v, f, L.lev);
    }
    for (long long i = rank; i < L.qlen_prev; i += size) {
        const int32_t v = __ldcg(L.qprev + i);
        a.vs[v].f[L.prv] = 0;
    }
}

// LINEAR: thread per frontier vertex, serial adjacency (linear_with_atomics.cu:122-135).
template <class G>
__device__ void gather_linear(const MsArgs &a, const Lvl &L)
{
    for (long long i = G::rank(); i < L.qlen; i += G::size()) {
        const int32_t v = __ldcg(L.qcur + i);
        const u64 f = __ldcg(&a.vs[v].f[L.cur]);
        const int32_t e1 = __ldg(a.R + v + 1);
        for (int32_t e = __ldg(a.R + v); e < e1; ++e) td_visit(a, L, f, __ldg(a.C + e));
    }
}

// EDGE: every CSR entry every level, source vertex from the COO array
// (edge_parallel.cu:77-88); one sweep serves all 64 sources of the batch.
template <class G>
__device__ void gather_edge(const MsArgs &a, const Lvl &L)
{
    for (long long e = G::rank(); e < a.m; e += G::size()) {
        const int32_t u = __ldg(a.F + e);
        const u64 f = __ldcg(&a.vs[u].f[L.cur]);
        if (f) td_visit(a, L, f, __ldg(a.C + e));
    }
}

// SHUFFLE: warp per frontier vertex; warps take the next vertex from a shared
// counter when done (shuffle_based.cuh:192-223).
template <class G>
__device__ void gather_shuffle(const MsArgs &a, const Lvl &L)
{
    const int lane = lane_id();
    const long long nw = G::size() >> 5;
    long long kq = G::rank() >> 5;
    while (kq < L.qlen) {
        const int32_t v = __ldcg(L.qcur + kq);
        const u64 f = __ldcg(&a.vs[v].f[L.cur]);
        const int32_t e1 = __ldg(a.R + v + 1);
        for (int32_t e = __ldg(a.R + v) + lane; e < e1; e += 32) td_visit(a, L, f, __ldg(a.C + e));
        int nk = 0;
        if (lane == 0) nk = atomicAdd(&a.ctl->work[L.slot], 1);
        kq = nw + __shfl_sync(FULL_MASK, nk, 0);
    }
}

// Warp strip-mining: each lane holds one frontier vertex; the warp elects the
// highest lane with adjacency left (race_and_resolve) and gathers its list
// together (warp_based.cu:109-145).
__device__ __forceinline__ void warp_stripmine(const MsArgs &a, const Lvl &L, int32_t r, int32_t r_end, u64 f)
{
    const int lane = lane_id();
    while (__any_sync(FULL_MASK, r < r_end)) {
        const int winner = race_and_resolve_warp(r < r_end);
        const int32_t rw = __shfl_sync(FULL_MASK, r, winner);
        const int32_t re = __shfl_sync(FULL_MASK, r_end, winner);
        const u64 fw = __shfl_sync(FULL_MASK, f, winner);
        if (lane == winner) r = r_end;  // a lane cannot win twice
        for (int32_t e = rw + lane; e < re; e += 32) td_visit(a, L, fw, __ldg(a.C + e));
    }
}

template <class G>
__device__ void gather_warp(const MsArgs &a, const Lvl &L)
{
    const int lane = lane_id();
    const long long nw = G::size() >> 5;
    for (long long base = (G::rank() >> 5) * 32; base < L.qlen; base += nw * 32) {
        const long long i = base + lane;
        int32_t r = 0, r_end = 0;
        u64 f = 0;
        if (i < L.qlen) {
            const int32_t v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            r_end = __ldg(a.R + v + 1);
            f = __ldcg(&a.vs[v].f[L.cur]);
        }
        warp_stripmine(a, L, r, r_end, f);
    }
}

// CTA_WARP: lists longer than 2048 are gathered by the whole CTA, one at a
// time (highest thread first), the rest by warp strip-mining (CTA_warp.cu:62-265).
template <class G>
__device__ void gather_cta_warp(const MsArgs &a, const Lvl &L)
{
    __shared__ int s_winner;
    __shared__ int32_t s_r, s_re;
    __shared__ u64 s_f;
    const int BD = blockDim.x;
    for (long long base = (long long)G::blk() * BD; base < L.qlen; base += (long long)G::nblk() * BD) {
        const long long i = base + threadIdx.x;
        int32_t r = 0, r_end = 0;
        u64 f = 0;
        if (i < L.qlen) {
            const int32_t v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            r_end = __ldg(a.R + v + 1);
            f = __ldcg(&a.vs[v].f[L.cur]);
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
                s_f = f;
                r = r_end;
            }
            __syncthreads();
            const int32_t re = s_re;
            const u64 fw = s_f;
            for (int32_t e = s_r + threadIdx.x; e < re; e += BD) td_visit(a, L, fw, __ldg(a.C + e));
            __syncthreads();
        }
        warp_stripmine(a, L, r, r_end, f);
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
        int t = lane < nw ? s_warp[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, ti, o);
            if (lane >= o) ti += y;
        }
        if (lane < nw) s_warp[lane] = ti - t;  // exclusive warp offsets
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
// vertex by binary search over the scanned offsets (scan_based.cu:107-149; the
// owner lookup is the load-balanced search of load_balanced_search.cu:176-191).
template <class G>
__device__ void gather_scan(const MsArgs &a, const Lvl &L)
{
    __shared__ int s_off[MS_THREADS];
    __shared__ int32_t s_r[MS_THREADS];
    __shared__ u64 s_f[MS_THREADS];
    __shared__ int s_warp[33];
    const int BD = blockDim.x;
    for (long long base = (long long)G::blk() * BD; base < L.qlen; base += (long long)G::nblk() * BD) {
        const long long i = base + threadIdx.x;
        int32_t r = 0;
        int deg = 0;
        u64 f = 0;
        if (i < L.qlen) {
            const int32_t v = __ldcg(L.qcur + i);
            r = __ldg(a.R + v);
            deg = __ldg(a.R + v + 1) - r;
            f = __ldcg(&a.vs[v].f[L.cur]);
        }
        int total;
        const int off = block_exclusive_scan(deg, &total, s_warp);
        s_off[threadIdx.x] = off;
        s_r[threadIdx.x] = r;
        s_f[threadIdx.x] = f;
        __syncthreads();
        for (int e = threadIdx.x; e < total; e += BD) {
            int lo = 0, hi = BD - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_off[mid] <= e) lo = mid;
                else hi = mid - 1;
            }
            td_visit(a, L, s_f[lo], __ldg(a.C + s_r[lo] + (e - s_off[lo])));
        }
        __syncthreads();
    }
}

// Bottom-up level: every vertex (coalesced sweep) finalises its own F_{j-1}
// bits, clears F_{j-2}, and, if some batch source has not reached it, ORs the
// F_{j-1} words of its in-neighbours until all missing bits are found.
template <class G>
__device__ void bu_sweep(const MsArgs &a, const Lvl &L)
{
    const int lane = lane_id();
    const long long size = G::size();
    for (long long base = G::rank() - lane; base < a.n; base += size) {
        const int32_t w = (int32_t)(base + lane);
        const bool valid = w < a.n;
        u64 seen = 0, f = 0;
        if (valid) {
            VState *s = a.vs + w;
            const ulonglong2 x = __ldcg(reinterpret_cast<const ulonglong2 *>(s));
            const ulonglong2 y = __ldcg(reinterpret_cast<const ulonglong2 *>(s) + 1);
            seen = x.x;
            f = L.cur == 0 ? x.y : (L.cur == 1 ? y.x : y.y);
            const u64 fp = L.prv == 0 ? x.y : (L.prv == 1 ? y.x : y.y);
            if (f) {
                seen |= f;
                s->seen = seen;
                if (seen == L.full) warp_add_u64(&a.ctl->fulledges[L.slot], capped_degree(a.R, w));
            }
            if (fp) s->f[L.prv] = 0;
        }
        write_bits_sweep(a.dist, a.ld, L.row0, w, f, L.lev);
        if (valid && seen != L.full) {
            u64 acc = 0;
            const int32_t e1 = __ldg(a.RT + w + 1);
            for (int32_t e = __ldg(a.RT + w); e < e1; ++e) {
                acc |= __ldcg(&a.vs[__ldg(a.CT + e)].f[L.cur]);
                if ((acc | seen) == L.full) break;
            }
            const u64 nb = acc & ~seen;
            if (nb) {
                a.vs[w].f[L.nxt] = nb;
                warp_append(w, L.qnxt, &a.ctl->qlen[L.slot], &a.ctl->qedges[L.slot], capped_degree(a.R, w));
            }
        }
    }
}

template <int VARIANT>
__global__ void __launch_bounds__(MS_THREADS) ms_grid_kernel(MsArgs a)
{
    unsigned epoch = 0;
    MsCtl *ctl = a.ctl;
    const long long rank = GridG::rank(), size = GridG::size();
    const int nbatch = (a.k + 63) >> 6;
    for (int b = 0; b < nbatch; ++b) {
        const int row0 = b << 6;
        const int nb = min(64, a.k - row0);
        const u64 full = nb == 64 ? ~0ull : ((1ull << nb) - 1ull);
        for (long long w = rank; w < a.n; w += size) {
            ulonglong2 *p = reinterpret_cast<ulonglong2 *>(a.vs + w);
            p[0] = make_ulonglong2(0ull, 0ull);
            p[1] = make_ulonglong2(0ull, 0ull);
        }
        init_dist_rows<GridG>(a.dist, a.ld, row0, nb, a.n);
        if (rank == 0) {
            for (int s = 0; s < 4; ++s) {
                ctl->qlen[s] = 0;
                ctl->work[s] = 0;
                ctl->qedges[s] = 0;
                ctl->fulledges[s] = 0;
            }
        }
        if (!grid_barrier(&ctl->bar, &ctl->err, epoch)) return;
        if (rank < nb) {
            const int32_t s = __ldg(a.sources + row0 + rank);
            const u64 old = atomicOr(&a.vs[s].f[0], 1ull << rank);
            if (old == 0) warp_append(s, a.q[0], &ctl->qlen[0], &ctl->qedges[0], capped_degree(a.R, s));
        }
        if (!grid_barrier(&ctl->bar, &ctl->err, epoch)) return;

        u64 fulltotal = 0;
        bool prev_bu = false;
        for (int j = 1;; ++j) {
            Lvl L;
            const int sc = (j - 1) & 3, sp = (j - 2) & 3;
            L.qlen = ld_volatile_i32(&ctl->qlen[sc]);
            if (L.qlen == 0) break;
            L.qlen_prev = j >= 2 ? ld_volatile_i32(&ctl->qlen[sp]) : 0;
            const u64 qedges = ld_volatile_u64(&ctl->qedges[sc]);
            fulltotal += ld_volatile_u64(&ctl->fulledges[sc]);
            L.slot = j & 3;
            L.cur = (j - 1) % 3;
            L.nxt = j % 3;
            L.prv = (j + 1) % 3;
            L.qcur = a.q[L.cur];
            L.qnxt = a.q[L.nxt];
            L.qprev = a.q[L.prv];
            L.lev = j - 1;
            L.row0 = row0;
            L.full = full;
            if (rank == 0) {
                const int z = (j + 1) & 3;
                ctl->qlen[z] = 0;
                ctl->work[z] = 0;
                ctl->qedges[z] = 0;
                ctl->fulledges[z] = 0;
            }
            bool bu = false;
            int policy = VARIANT;
            if (VARIANT == GU_BFS_BOTTOM_UP) {
                bu = j > 1;
            } else if (VARIANT == GU_BFS_AUTO) {
                const double unexplored = (double)a.m - (double)fulltotal;
                if (!prev_bu) bu = j > 1 && (double)qedges > unexplored / (double)a.alpha;
                else bu = (double)L.qlen >= (double)a.n / (double)a.beta;
                const double avg = (double)qedges / (double)L.qlen;
                policy = avg <= 8.0 ? GU_BFS_LINEAR : GU_BFS_SHUFFLE;
            }
            if (bu) {
                bu_sweep<GridG>(a, L);
            } else {
                td_update<GridG>(a, L);
                if (VARIANT == GU_BFS_EDGE) gather_edge<GridG>(a, L);
                else if (VARIANT == GU_BFS_WARP) gather_warp<GridG>(a, L);
                else if (VARIANT == GU_BFS_CTA_WARP) gather_cta_warp<GridG>(a, L);
                else if (VARIANT == GU_BFS_SCAN) gather_scan<GridG>(a, L);
                else if (VARIANT == GU_BFS_SHUFFLE || VARIANT == GU_BFS_BOTTOM_UP) gather_shuffle<GridG>(a, L);
                else if (VARIANT == GU_BFS_AUTO && policy == GU_BFS_SHUFFLE) gather_shuffle<GridG>(a, L);
                else gather_linear<GridG>(a, L);
            }
            if (rank == 0) {
                if (bu) ctl->bu_levels++;
                else ctl->td_levels++;
                if (j - 1 > ctl->max_level) ctl->max_level = j - 1;
            }
            prev_bu = bu;
            if (!grid_barrier(&ctl->bar, &ctl->err, epoch)) return;
        }
    }
}

// ---- host side ---------------------------------------------------------------
template <int V>
static void launch_variant(const MsArgs &a, int sms, cudaStream_t stream)
{
    static int blocks_per_sm = -1;
    if (blocks_per_sm < 0) {
        GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, ms_grid_kernel<V>, MS_THREADS, 0));
        if (blocks_per_sm < 1) throw gu_error(GU_ERR_INTERNAL, "msbfs kernel cannot be resident");
    }
    dim3 grid(sms * blocks_per_sm), block(MS_THREADS);
    MsArgs args = a;
    void *params[] = {&args};
    GU_CUDA_CHECK(cudaLaunchCooperativeKernel((const void *)ms_grid_kernel<V>, grid, block, params, 0, stream));
}

void launch_msbfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                  const MsOptions &opt, cudaStream_t stream, int *dev_err_out)
{
    (void)dev_err_out;
    if (opt.variant == GU_BFS_EDGE) ensure_coo(g, stream);
    const size_t n = (size_t)g.n;
    const size_t vs_bytes = ((n * sizeof(VState) + 255) / 256) * 256;
    const size_t q_bytes = ((n * sizeof(int32_t) + 255) / 256) * 256;
    const size_t ctl_bytes = 256;
    char *ws = (char *)g.ws.get(ctl_bytes + vs_bytes + 3 * q_bytes);
    MsArgs a;
    a.R = g.R;
    a.C = g.C;
    a.RT = g.RT;
    a.CT = g.CT;
    a.F = g.F;
    a.n = g.n;
    a.m = g.m;
    a.sources = sources;
    a.k = k;
    a.dist = dist;
    a.ld = ld;
    a.ctl = reinterpret_cast<MsCtl *>(ws);
    a.vs = reinterpret_cast<VState *>(ws + ctl_bytes);
    a.q[0] = reinterpret_cast<int32_t *>(ws + ctl_bytes + vs_bytes);
    a.q[1] = reinterpret_cast<int32_t *>(ws + ctl_bytes + vs_bytes + q_bytes);
    a.q[2] = reinterpret_cast<int32_t *>(ws + ctl_bytes + vs_bytes + 2 * q_bytes);
    a.alpha = opt.alpha;
    a.beta = opt.beta;
    GU_CUDA_CHECK(cudaMemsetAsync(a.ctl, 0, sizeof(MsCtl), stream));
    const int sms = g.sm_count;
    g.mark_start(stream);
    switch (opt.variant) {
    case GU_BFS_AUTO: launch_variant<GU_BFS_AUTO>(a, sms, stream); break;
    case GU_BFS_LINEAR: launch_variant<GU_BFS_LINEAR>(a, sms, stream); break;
    case GU_BFS_EDGE: launch_variant<GU_BFS_EDGE>(a, sms, stream); break;
    case GU_BFS_WARP: launch_variant<GU_BFS_WARP>(a, sms, stream); break;
    case GU_BFS_CTA_WARP: launch_variant<GU_BFS_CTA_WARP>(a, sms, stream); break;
    case GU_BFS_SCAN: launch_variant<GU_BFS_SCAN>(a, sms, stream); break;
    case GU_BFS_SHUFFLE: launch_variant<GU_BFS_SHUFFLE>(a, sms, stream); break;
    case GU_BFS_BOTTOM_UP: launch_variant<GU_BFS_BOTTOM_UP>(a, sms, stream); break;
    default: throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown BFS variant");
    }
    g.mark_stop(stream);
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

}  // namespace gu
