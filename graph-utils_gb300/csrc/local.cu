// local.cu -- per-source BFS for low-degree (mesh-like, high-diameter) graphs,
// and AUTO's choice between the search engines.
//
// The batched bit-matrix engine shares a level among 64 W sources, which pays off
// when the sources' frontiers overlap (small-world graphs reach most vertices in a
// handful of levels).  On meshes (a 2048 x 2048 grid has a diameter near 4000)
// every source reaches a vertex at a different level, the union frontier holds
// each vertex once per distinct level, and every visit moves whole source words.
// There the reference's own decomposition -- one CTA per source, level-
// synchronous (multi_search/shuffle_based.cuh:81-286, the atomicCAS visit of
// multi_search/linear_with_atomics.cu:130) -- is the right one, provided a level
// costs little: here the two level queues live in shared memory (up to
// LOCAL_QCAP vertices, or n when that is smaller), a thread expands the whole
// adjacency list of a low-degree vertex with four claims in flight, and appends
// are warp-aggregated shared atomics.  A frontier larger than the shared queue
// ends the launch with a flag and the caller reruns the search on the batched
// engine.  Rows mode claims vertices in the distance row itself; the counting
// modes (diameter, reachability) claim them in a per-CTA visited bitmap and
// write no rows.
//
// The adjacency is read from a padded copy (ELL: the neighbours of v in CSR
// order at v * width, width 4, 8 or 16, padded with -1), built on the graph's
// first per-source search: one 16-byte load brings a grid vertex's whole list,
// where the CSR form needs the offsets first and then a second, dependent load.
// With a few hundred sources' frontiers spread over the graph the adjacency does
// not stay in L2, so the halved sector count matters as much as the shorter
// chain.
#include "device_utils.cuh"
#include "gu_internal.h"

#include <algorithm>
#include <climits>
#include <cstdlib>

namespace gu {

// One 1024-thread CTA per source, two per SM: 256 sources fill the GPU, and a
// level's frontier (a few thousand vertices on a 2048 x 2048 mesh) takes one or
// two dependent load chains per thread.  The queues are kept small because the
// shared memory they do not use is L1: on the 2048 x 2048 grid with 256 sources,
// rows took 62.6 ms with 512 threads and two 12288-vertex queues, 40.5 ms with
// 1024 threads and two 6144-vertex queues, and no less with smaller queues.
constexpr int LOCAL_THREADS = 1024;
constexpr int LOCAL_QCAP = 6144;      // vertices per shared-memory level queue (two queues: 48 KiB)
constexpr int LOCAL_MAX_DEGREE = 16;     // AUTO takes this engine up to this out-degree
constexpr int PLAIN_MAX_VERTICES = 4096;  // ... and the one-CTA-per-source form up to this many vertices
constexpr size_t LOCAL_SMEM = 2 * LOCAL_QCAP * sizeof(int32_t);

struct LocalArgs {
    const int4 *__restrict__ ell;  // [n][width / 4]
    int32_t n;
    const int32_t *sources;
    int32_t k;
    int32_t *dist;  // rows mode: k x ld
    int64_t ld;
    uint32_t *vis;  // counting modes: [gridDim.x][vis_words]
    int64_t vis_words;
    unsigned long long *reach;  // counting: per-source reachable count (null: none)
    int *max_level;             // atomicMax of the deepest level reached (null: none)
    int *overflow;              // set when a frontier exceeds qcap
    int qcap;                   // vertices per shared level queue: min(n, LOCAL_QCAP)
};

__global__ void build_ell_kernel(const int32_t *__restrict__ R, const int32_t *__restrict__ C, int32_t n, int width,
                                 int32_t *__restrict__ ell)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n * width;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = (int32_t)(i / width), t = (int32_t)(i % width);
        const int32_t e = __ldg(R + v) + t;
        ell[i] = e < __ldg(R + v + 1) ? __ldg(C + e) : -1;
    }
}

template <bool ROWS, int WIDTH>
__global__ void __launch_bounds__(LOCAL_THREADS, 2) local_bfs_kernel(LocalArgs a)
{
    extern __shared__ int32_t sq[];  // [2][qcap]
    __shared__ int s_len[2];
    __shared__ int s_stop;
    uint32_t *vis = ROWS ? nullptr : a.vis + (size_t)blockIdx.x * a.vis_words;
    const int lane = lane_id();
    for (int si = blockIdx.x; si < a.k; si += gridDim.x) {
        if (threadIdx.x == 0) s_stop = ld_volatile_i32(a.overflow);  // another CTA overflowed: the caller reruns
        __syncthreads();
        if (s_stop) return;
        const int32_t src = __ldg(a.sources + si);
        int32_t *d = ROWS ? a.dist + (int64_t)si * a.ld : nullptr;
        if (ROWS) {
            for (int32_t v = threadIdx.x; v < a.n; v += blockDim.x) d[v] = (v == src) ? 0 : INT_MAX;
        } else {
            for (int64_t w = threadIdx.x; w < a.vis_words; w += blockDim.x)
                vis[w] = (w == (src >> 5)) ? (1u << (src & 31)) : 0u;
        }
        if (threadIdx.x == 0) {
            sq[0] = src;
            s_len[0] = 1;
            s_len[1] = 0;
        }
        __syncthreads();
        int cur = 0, level = 0, maxl = 0;
        long long reached = 1;
        while (true) {
            const int qlen = s_len[cur];
            if (qlen == 0) break;
            maxl = level;
            const int32_t *Q = sq + cur * a.qcap;
            int32_t *Q2 = sq + (cur ^ 1) * a.qcap;
            int *nlen = &s_len[cur ^ 1];
            for (int i = threadIdx.x; i < qlen; i += blockDim.x) {
                const int4 *row = a.ell + (size_t)Q[i] * (WIDTH / 4);
#pragma unroll
                for (int c = 0; c < WIDTH / 4; ++c) {
                    const int4 q4 = __ldg(row + c);
                    const int32_t w[4] = {q4.x, q4.y, q4.z, q4.w};
                    if (w[0] < 0) break;  // padding: the list ended
                    bool ok[4], seen[4];
#pragma unroll
                    for (int t = 0; t < 4; ++t)  // rows: plain reads first (the row lives in DRAM;
                        // a claimed entry never reverts, so a stale read only costs the CAS)
                        seen[t] = w[t] < 0 || (ROWS && d[w[t]] != INT_MAX);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {  // four claims in flight
                        if (seen[t]) {
                            ok[t] = false;
                        } else if (ROWS) {
                            ok[t] = atomicCAS(d + w[t], INT_MAX, level + 1) == INT_MAX;
                        } else {
                            const uint32_t bit = 1u << (w[t] & 31);
                            ok[t] = !(atomicOr(vis + (w[t] >> 5), bit) & bit);
                        }
                    }
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        if (ok[t]) {
                            const unsigned mask = __activemask();
                            const int leader = __ffs(mask) - 1;
                            int base = 0;
                            if (lane == leader) base = atomicAdd(nlen, __popc(mask));
                            base = __shfl_sync(mask, base, leader);
                            const int pos = base + __popc(mask & ((1u << lane) - 1u));
                            if (pos < a.qcap) Q2[pos] = w[t];
                        }
                    }
                }
            }
            __syncthreads();
            const int nl = *nlen;
            if (nl > a.qcap) {  // frontier too large for the shared queues: hand back to the caller
                if (threadIdx.x == 0) atomicExch(a.overflow, 1);
                return;
            }
            reached += nl;
            if (threadIdx.x == 0) s_len[cur] = 0;  // the queue just read is the next level's target
            cur ^= 1;
            ++level;
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (a.reach) a.reach[si] = (unsigned long long)reached;
            if (a.max_level) atomicMax(a.max_level, maxl);
        }
        __syncthreads();  // shared queues reused by the next source
    }
}

// AUTO's engine choice: the per-source engine for low-degree graphs (its
// thread-per-vertex expansion wants short adjacency lists), the one-CTA-per-
// source warp-per-vertex form for tiny graphs with longer lists (distance rows
// only: it has no counting mode), the batched bit-matrix engine otherwise.
// GU_AUTO_LOCAL=0 in the environment keeps AUTO on the batched engine (tests use
// it to cover every engine on the same graphs).
AutoEngine auto_engine(const DeviceGraph &g, bool rows)
{
    const char *e = std::getenv("GU_AUTO_LOCAL");
    if (e && e[0] == '0') return AutoEngine::BATCHED;
    if (g.max_degree <= LOCAL_MAX_DEGREE) return AutoEngine::LOCAL;
    if (rows && g.n <= PLAIN_MAX_VERTICES) return AutoEngine::PLAIN;
    return AutoEngine::BATCHED;
}

// Returns false if a frontier overflowed the shared queues (the caller reruns the
// search on the batched engine).  Synchronises `stream`.
bool launch_local_bfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                      unsigned long long *reach, int *max_level_host, cudaStream_t stream)
{
    if (!g.ell) {  // the padded adjacency, once per graph
        const int width = g.max_degree <= 4 ? 4 : g.max_degree <= 8 ? 8 : 16;
        if (g.max_degree > 16) throw gu_error(GU_ERR_INTERNAL, "per-source engine on a graph of out-degree > 16");
        const size_t bytes = (size_t)(g.n > 0 ? g.n : 1) * width * sizeof(int32_t);
        GU_CUDA_CHECK(dev_malloc((void **)&g.ell, bytes));
        g.extra_allocs.push_back(g.ell);
        g.bytes += bytes;
        g.ell_width = width;
        const int64_t total = (int64_t)g.n * width;
        const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)g.sm_count * 8);
        if (total > 0) build_ell_kernel<<<blocks > 0 ? blocks : 1, 256, 0, stream>>>(g.R, g.C, g.n, width, g.ell);
        GU_CUDA_CHECK(cudaGetLastError());
    }
    static bool attr_set[2][3] = {{false, false, false}, {false, false, false}};
    const bool rows = dist != nullptr;
    const int wi = g.ell_width == 4 ? 0 : g.ell_width == 8 ? 1 : 2;
    void (*const kerns[2][3])(LocalArgs) = {
        {local_bfs_kernel<false, 4>, local_bfs_kernel<false, 8>, local_bfs_kernel<false, 16>},
        {local_bfs_kernel<true, 4>, local_bfs_kernel<true, 8>, local_bfs_kernel<true, 16>}};
    auto kern = kerns[rows][wi];
    if (!attr_set[rows][wi]) {
        GU_CUDA_CHECK(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)LOCAL_SMEM));
        attr_set[rows][wi] = true;
    }
    const int qcap = g.n < LOCAL_QCAP ? (g.n > 0 ? g.n : 1) : LOCAL_QCAP;
    const size_t smem = 2 * (size_t)qcap * sizeof(int32_t);
    int per_sm = 0;
    GU_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)kern, LOCAL_THREADS, smem));
    if (per_sm < 1) throw gu_error(GU_ERR_INTERNAL, "per-source BFS kernel cannot be resident");
    int grid = g.sm_count * per_sm;
    if (grid > k) grid = k;
    const int64_t vis_words = rows ? 0 : ((int64_t)g.n + 31) / 32;
    const size_t need = WS_CONTROL_BYTES + (size_t)grid * (size_t)vis_words * sizeof(uint32_t);
    char *ws = (char *)g.ws.get(need);
    GU_CUDA_CHECK(cudaMemsetAsync(ws, 0, 64, stream));
    LocalArgs a;
    a.ell = reinterpret_cast<const int4 *>(g.ell);
    a.n = g.n;
    a.sources = sources;
    a.k = k;
    a.dist = dist;
    a.ld = ld;
    a.vis = reinterpret_cast<uint32_t *>(ws + WS_CONTROL_BYTES);
    a.vis_words = vis_words;
    a.reach = reach;
    a.max_level = reinterpret_cast<int *>(ws);
    a.overflow = reinterpret_cast<int *>(ws) + 1;
    a.qcap = qcap;
    g.mark_start(stream);
    kern<<<grid, LOCAL_THREADS, smem, stream>>>(a);
    GU_CUDA_CHECK(cudaGetLastError());
    g.mark_stop(stream);
    int flags[2] = {0, 0};
    GU_CUDA_CHECK(cudaMemcpyAsync(flags, ws, sizeof(flags), cudaMemcpyDeviceToHost, stream));
    GU_CUDA_CHECK(cudaStreamSynchronize(stream));
    if (max_level_host) *max_level_host = flags[0];
    return flags[1] == 0;
}

}  // namespace gu
