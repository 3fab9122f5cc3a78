// gu_internal.h -- internal host-side declarations shared by the library's
// translation units (never installed; the public boundary is include/gu.h).
#pragma once

#include <cstdint>
#include <cstddef>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gu.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <cuda_runtime_api.h>
#endif

namespace gu {

// Bottom-up degree classes (by in-degree, vertices with in-degree 0 in none):
// <= BU_LIGHT_DEGREE one thread per vertex, <= BU_MID_DEGREE eight lanes per
// vertex, <= BU_HEAVY_DEGREE a warp per vertex with every in-edge loaded at
// once, above that a warp stepping through the in-edges.
constexpr int BU_LIGHT_DEGREE = 8;
constexpr int BU_MID_DEGREE = 32;
constexpr int BU_HEAVY_DEGREE = 128;
// Every workspace starts with this many bytes of launch control block and
// profiling timeline; kernel scratch follows.
constexpr size_t WS_CONTROL_BYTES = 65536;

// Device-side error codes written to a launch's control block.
enum DevErr : int {
    DEV_OK = 0,
    DEV_ERR_BARRIER_TIMEOUT = 1,
    DEV_ERR_QUEUE_OVERFLOW = 2,
    DEV_ERR_BAD_SOURCE = 4,  // batched search: a source id outside [0, n) (skipped, not searched)
};

struct gu_error : std::runtime_error {
    gu_status code;
    gu_error(gu_status c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

void set_last_error(const std::string &msg);

#define GU_CUDA_CHECK(expr)                                                                          \
    do {                                                                                             \
        cudaError_t e__ = (expr);                                                                    \
        if (e__ != cudaSuccess) {                                                                    \
            throw ::gu::gu_error(e__ == cudaErrorMemoryAllocation ? GU_ERR_OUT_OF_MEMORY : GU_ERR_CUDA, \
                                 std::string(#expr) + ": " + cudaGetErrorString(e__));               \
        }                                                                                            \
    } while (0)

// Every device and pinned host allocation of the library goes through these two
// (graph.cu).  They return cudaErrorMemoryAllocation on their own when a failure
// has been injected with gu_debug_fail_allocations, so that tests can drive each
// caller's out-of-memory path (GU_ERR_OUT_OF_MEMORY, the handle left usable)
// without exhausting the GPU.
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t pinned_alloc(void **p, size_t bytes);
void set_alloc_failures(long long after, long long count);

// Bound of every device-side wait (grid barriers) in nanoseconds, passed to each
// persistent launch; gu_set_wait_limit sets it for the process (4 s by default).
unsigned long long wait_limit_ns();
void set_wait_limit_ns(unsigned long long ns);
// gu_check_grid_barrier: returns the number of CTAs launched; throws GU_ERR_TIMEOUT
// when the absent CTA's missing arrival made the others' wait run out.
int check_grid_barrier(int absent, unsigned long long limit_ns, cudaStream_t st, double *seconds);

// Host CSR graph (the reference's host_graph, parse.h:15-35, without F; F is
// derived on the device when a variant needs it).
struct HostGraph {
    int32_t n = 0;
    bool directed = false;
    std::vector<int32_t> R, C;
    int64_t m() const { return (int64_t)C.size(); }
};

HostGraph gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, bool permute);
HostGraph gen_er(int32_t n, int64_t m, uint64_t seed);
HostGraph gen_grid(int32_t rows, int32_t cols, double p_delete, uint64_t seed);
HostGraph gen_dag(int32_t n, int64_t m, uint64_t seed);
std::vector<int32_t> gen_sources(int32_t n, int32_t k, uint64_t seed);
HostGraph transpose(const HostGraph &g);
// Graph files (io.cpp): "dimacs"/"metis", "edgelist", "edgelist_h", "market", "csrbin".
HostGraph parse_graph_file(const char *path, const char *format);
void write_csr_cache(const HostGraph &g, const char *path);
void write_edgelist(const HostGraph &g, const char *path, bool header);
uint64_t count_degree_zero(const HostGraph &g);
void sort_adjacency_by_key(const int32_t *R, int32_t *C, int32_t n, const int32_t *key);
void build_csr(int32_t n, const std::vector<int32_t> &eu, const std::vector<int32_t> &ev, bool symmetric,
               std::vector<int32_t> &R, std::vector<int32_t> &C);

// Device workspace: one allocation grown on demand, owned by a graph handle.
struct Workspace {
    void *ptr = nullptr;
    size_t bytes = 0;
    int device = -1;
    void *get(size_t need);  // grows (synchronously) when needed
    void release();
};

// Adjacency cut into work items of at most BC_CHUNK_EDGES edges (every vertex
// has at least one, possibly empty, item).  Device arrays; built on first use.
constexpr int BC_CHUNK_EDGES = 256;
struct ChunkMap {
    int32_t *v = nullptr;      // [nchunks] vertex of the item
    int32_t *e0 = nullptr;     // [nchunks] first edge
    int32_t *e1 = nullptr;     // [nchunks] end edge
    int32_t *slot = nullptr;   // [nchunks] partial slot of a split vertex's item, -1 if not split
    int32_t nchunks = 0;
    int32_t *mv = nullptr;     // [nmulti] vertices split into several items
    int32_t *mfirst = nullptr; // [nmulti] their first item
    int32_t *mcount = nullptr; // [nmulti] their number of items
    int32_t nmulti = 0;
    int32_t nslots = 0;        // items of split vertices
    int32_t *order = nullptr;  // [nchunks] items by descending edge count
    int32_t *ustart = nullptr; // [nunits+1] work units: runs of order[] of <= 32 items and about 512 edges
    int32_t nunits = 0;
    bool built = false;
};

// Device-resident graph (the reference's device_graph, device_graph.h:7-22):
// 256-byte-aligned int32 arrays in HBM.  RT/CT is the transposed (in-edge)
// CSR, identical to R/C for undirected graphs.  F (COO source of every CSR
// entry) is built on first use by the edge-parallel variant.
// The batched engine's default rare-source fraction (MsOptions::rare_frac).  On
// R-MAT graphs against 1/3: scale 20 x 512 sources 1.637 -> 1.610 ms, scale 18 x
// 1024 sources 1.465 -> 1.311 ms (0.06: 1.227), scale 22 x 256 sources 2.82 ->
// 2.84 ms; gu_graph_autotune also tries 0.06 and 1/3.
constexpr float MS_RARE_FRAC = 0.15f;

struct DeviceGraph {
    int device = 0;
    int32_t n = 0;
    int64_t m = 0;
    bool directed = false;
    int32_t *R = nullptr, *C = nullptr;
    int32_t *RT = nullptr, *CT = nullptr;
    int32_t *F = nullptr;
    int32_t max_degree = 0;
    // AUTO's measured choice (gu_graph_autotune / gu_graph_set_tuning); unset: by shape
    struct Tuning {
        bool set = false;
        int engine = 0;  // gu_engine
        float alpha = 2.f, beta = 24.f;
        int words = 0;
        int ctas_per_sm = 0;  // batched engine's grid: CTAs per SM (0: as many as fit)
        float rare_frac = MS_RARE_FRAC;
    } tune;
    void *ctl_host = nullptr;  // pinned copy of the batched engine's control block, written after each launch
    int32_t *ell = nullptr;  // low-degree graphs: neighbours padded to ell_width per vertex (-1), built on first use
    int ell_width = 0;
    // bottom-up degree classes by in-degree, each ascending: light (1 ..
    // BU_LIGHT_DEGREE), mid (.. BU_MID_DEGREE), wide (.. BU_HEAVY_DEGREE),
    // heavy (above)
    int32_t *light = nullptr, *mid = nullptr, *wide = nullptr, *heavy = nullptr;
    int32_t nlight = 0, nmid = 0, nwide = 0, nheavy = 0;
    size_t bytes = 0;
    std::mutex mu;  // serialises calls on one handle (workspace reuse)
    Workspace ws;  // kernel scratch
    Workspace io;  // device staging for calls that take host buffers
    int sm_count = 0;
    // BC work items over in-edges (forward) and out-edges (backward); for
    // undirected graphs bc_out aliases bc_in
    ChunkMap bc_in, bc_out;
    std::vector<int32_t> host_R, host_RT;  // offsets kept on the host for building work items
    std::vector<void *> extra_allocs;  // freed with the graph
    // events bracketing the last main kernel launch (kernel-only timing): the
    // current slot of a ring that keeps the last LAUNCH_RING launches' events
    static constexpr int LAUNCH_RING = 64;
    cudaEvent_t ring_start[LAUNCH_RING] = {}, ring_stop[LAUNCH_RING] = {};
    int ring_next = 0, ring_count = 0;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaStream_t copy_st = nullptr;  // host-form calls copy rows out on it while later sources run
    bool timed = false;
    int timeline = 0;  // engine whose phase timeline the workspace holds: 0 batched BFS, 1 BC
    void mark_start(cudaStream_t s);
    void mark_stop(cudaStream_t s);
    ~DeviceGraph();
};

// Per-call options of the batched multi-source engine.
struct MsOptions {
    int variant = GU_BFS_AUTO;
    int batch_words = 0;  // 64-source words per batch (0: by the number of sources)
    float alpha = 2.f;    // top-down -> bottom-up when frontier out-edges > m / alpha
    float beta = 24.f;    // bottom-up -> top-down when frontier vertices < n / beta
    float gamma = 4.f;    // ... or when frontier out-edges < n / gamma
    // bottom-up levels expand top-down the sources that fewer than this fraction
    // of the CTAs discovered in the previous level (0: none)
    float rare_frac = MS_RARE_FRAC;
    bool tuned = false;  // alpha, beta, rare_frac, words come from the graph's tuning: the GU_MS_* variables do not apply
    Workspace *ws = nullptr;  // scratch to use (default: the graph's)
    int max_blocks = 0;       // cap on the persistent grid (0: the whole GPU)
    bool timed = true;        // record the graph's launch events
    unsigned long long *reach = nullptr;  // device, k per-source reachable counts (zeroed by the caller)
};

// Per-call options of the batched sigma / Brandes engine.
struct BcOptions {
    int batch = 0;                      // sources per pass (0: default)
    Workspace *ws = nullptr;            // scratch to use (default: the graph's)
    int max_blocks = 0;                 // cap on the persistent grid
    bool timed = true;
    const int32_t *req_start = nullptr; // device, nreq+1 source offsets of the requests (null: one request)
    int32_t nreq = 1;                   // bc receives nreq x n values
};

// Kernel launchers (device pointers, stream ordered; return after enqueue).
void launch_msbfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                  const MsOptions &opt, cudaStream_t stream, int *dev_err_out);
void launch_plain_bfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                      cudaStream_t stream);
// Per-source engine for low-degree graphs (AUTO's choice there): rows
// (dist non-null) or counts (reach, deepest level).  Synchronises; returns false
// if a frontier overflowed its shared queues (rerun on the batched engine).
// Reachable-set sizes of every vertex of a DAG (self excluded) and their sum.
void dag_reach(DeviceGraph &g, int64_t *counts, int64_t *total_host, cudaStream_t st);
int msbfs_words_for(int32_t k);  // 64-source words per batch for k sources
enum class AutoEngine { LOCAL, PLAIN, BATCHED };
AutoEngine auto_engine(const DeviceGraph &g, bool rows);
bool launch_local_bfs(DeviceGraph &g, const int32_t *sources, int32_t k, int32_t *dist, int64_t ld,
                      unsigned long long *reach, int *max_level_host, cudaStream_t stream);
// Batched sigma / Brandes: bc (n doubles, may be null), optional rows (k x ld).
void launch_bc(DeviceGraph &g, const int32_t *sources, int32_t k, const BcOptions &opt, double *bc, int32_t *dist_rows,
               uint64_t *sigma_rows, double *delta_rows, int64_t ld, bool backward, cudaStream_t stream);
size_t bc_workspace_bytes(const DeviceGraph &g, int32_t k, int batch, bool backward);
// One request of a work-queue launch: BFS rows (dist, k x ld) and/or reachable
// counts (reach, k) of k sources on graph g (any graph on the current device).
struct MsQueueRequest {
    DeviceGraph *g = nullptr;
    const int32_t *sources = nullptr;
    int32_t k = 0;
    int32_t *dist = nullptr;
    int64_t ld = 0;
    unsigned long long *reach = nullptr;
};
struct MsQueueLaunch {
    int W = 0, ngroups = 0, group_size = 0, items = 0;
    size_t stride = 0;                             // bytes of workspace per group
    size_t items_off = 0, cnt_off = 0, bytes = 0;  // item array, counter, total workspace
};
MsQueueLaunch msbfs_queue_plan(const std::vector<MsQueueRequest> &reqs, int sms, int max_blocks);
// Runs every request in one persistent launch whose CTA groups drain a device
// queue of (graph, source block) items (asynchronous on st; the graphs' lazily
// built structures are not touched).  msbfs_queue_error reads the groups' device
// error words once st is synchronised (0: none).
MsQueueLaunch launch_msbfs_queue(const std::vector<MsQueueRequest> &reqs, Workspace &ws, int sms, int max_blocks,
                                 cudaStream_t st);
int msbfs_queue_error(const Workspace &ws, const MsQueueLaunch &L);
size_t msbfs_workspace_bytes(const DeviceGraph &g, int32_t k);
void bc_read_status(DeviceGraph &g, int *dev_err, int *max_level);
int bc_read_timeline(DeviceGraph &g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                     int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms);
size_t lbs_scratch_bytes(int32_t N, int64_t result_capacity);
void launch_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result, int64_t result_capacity,
                int32_t *total_dev, int64_t *total_host, void *scratch_ptr, size_t scratch_bytes, cudaStream_t st);
double lbs_last_ms(int device);
void launch_race_and_resolve(const int32_t *pred, int32_t nwarps, int32_t *winner, cudaStream_t st);

// Board power sampling through NVML loaded at run time (power.cpp).
struct PowerSampler;
PowerSampler *power_start(int device, int period_ms);
void power_stop(PowerSampler *s, double *avg_w, long long *samples);  // joins and frees

class Server;
Server *server_create(size_t budget, int nslots, int max_batch);
void server_destroy(Server *s);
int64_t server_submit(Server *s, int kind, DeviceGraph *g, const int32_t *src, int32_t k, void *out);
gu_status server_wait(Server *s, int64_t id, double timeout, double *latency, std::string &err);
void server_stats(Server *s, int64_t *completed, int64_t *batches, double *p50, double *p99, double *mean_batch);
void msbfs_read_status(DeviceGraph &g, int *dev_err, int *td_levels, int *bu_levels, int *max_level);
// The same, from the pinned copy launch_msbfs queued after its kernel (valid once
// the launch's stream is synchronised; the launch used the graph's workspace).
void msbfs_status_after_sync(DeviceGraph &g, int *dev_err, int *td_levels, int *bu_levels, int *max_level);
void ensure_coo(DeviceGraph &g, cudaStream_t stream);
int device_sm_count(int device);

}  // namespace gu
