// capi.cpp -- the extern "C" boundary declared in include/gu.h.
//
// Every entry point converts exceptions into a gu_status and a thread-local
// message (the reference exits the process instead, util_device.cuh:10-22).
#include "gu_internal.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <functional>
#include <memory>

namespace gu {
DeviceGraph *create_device_graph(const int32_t *R, const int32_t *C, int32_t n, int64_t m, bool directed,
                                 cudaStream_t stream);
void msbfs_read_status(DeviceGraph &g, int *dev_err, int *td_levels, int *bu_levels, int *max_level);
int msbfs_read_idle(DeviceGraph &g, int max_entries, double *idle_ms, int *nblocks);
int msbfs_read_timeline(DeviceGraph &g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                        int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms);

static thread_local std::string t_last_error;
void set_last_error(const std::string &msg) { t_last_error = msg; }

template <class F>
static gu_status guarded(F &&fn)
{
    try {
        fn();
        return GU_OK;
    } catch (const gu_error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return GU_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return GU_ERR_INTERNAL;
    }
}

// Makes the graph's device current for the scope of a call.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev)
    {
        GU_CUDA_CHECK(cudaGetDevice(&prev));
        if (prev != dev) GU_CUDA_CHECK(cudaSetDevice(dev));
    }
    ~DeviceScope()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// After launch_msbfs on the graph's workspace: waits for the launch and reads its
// control block from the pinned copy the launch queued behind its kernel.
static void check_dev_status(DeviceGraph &g, cudaStream_t stream)
{
    GU_CUDA_CHECK(cudaStreamSynchronize(stream));
    GU_CUDA_CHECK(cudaGetLastError());
    int err = 0;
    msbfs_status_after_sync(g, &err, nullptr, nullptr, nullptr);
    if (err == DEV_ERR_BARRIER_TIMEOUT) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit");
    if (err == DEV_ERR_BAD_SOURCE) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range");
    if (err != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(err));
}

}  // namespace gu

using namespace gu;

struct gu_graph_s {
    std::unique_ptr<DeviceGraph> g;
};
struct gu_hgraph_s {
    HostGraph h;
};
struct gu_power_s {
    PowerSampler *s = nullptr;
};
struct gu_timer_s {
    cudaEvent_t a = nullptr, b = nullptr;
};

extern "C" {

int gu_version(void) { return 10000; }

const char *gu_last_error(void) { return t_last_error.c_str(); }

const char *gu_status_string(gu_status s)
{
    switch (s) {
    case GU_OK: return "ok";
    case GU_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GU_ERR_CUDA: return "CUDA error";
    case GU_ERR_OUT_OF_MEMORY: return "out of memory";
    case GU_ERR_CAPACITY: return "capacity exceeded";
    case GU_ERR_OVERFLOW: return "overflow";
    case GU_ERR_TIMEOUT: return "device wait timed out";
    case GU_ERR_UNSUPPORTED: return "unsupported";
    case GU_ERR_INTERNAL: return "internal error";
    case GU_ERR_PENDING: return "request pending";
    }
    return "unknown status";
}

gu_status gu_choose_device(int requested, int *chosen)
{
    return guarded([&] {
        int count = 0;
        GU_CUDA_CHECK(cudaGetDeviceCount(&count));
        if (count < 1) throw gu_error(GU_ERR_CUDA, "no CUDA device");
        int best = requested;
        if (requested == -1) {
            double best_bw = -1;
            for (int d = 0; d < count; ++d) {
                int clk = 0, bus = 0;
                GU_CUDA_CHECK(cudaDeviceGetAttribute(&clk, cudaDevAttrMemoryClockRate, d));
                GU_CUDA_CHECK(cudaDeviceGetAttribute(&bus, cudaDevAttrGlobalMemoryBusWidth, d));
                const double bw = (double)clk * 1000.0 * (bus / 8) * 2 / 1e9;
                if (bw > best_bw) {
                    best_bw = bw;
                    best = d;
                }
            }
        } else if (requested < -1 || requested >= count) {
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "device index out of range 0.." + std::to_string(count - 1));
        }
        GU_CUDA_CHECK(cudaSetDevice(best));
        if (chosen) *chosen = best;
    });
}

gu_status gu_set_wait_limit(double seconds)
{
    return guarded([&] {
        if (!(seconds >= 1e-4 && seconds <= 3600.0))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "wait limit must be in [1e-4, 3600] seconds");
        set_wait_limit_ns((unsigned long long)(seconds * 1e9));
    });
}

gu_status gu_get_wait_limit(double *seconds)
{
    return guarded([&] {
        if (!seconds) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output");
        *seconds = (double)wait_limit_ns() * 1e-9;
    });
}

gu_status gu_check_grid_barrier(int absent_block, double limit_seconds, void *stream, double *elapsed_seconds)
{
    return guarded([&] {
        if (!(limit_seconds >= 1e-4 && limit_seconds <= 60.0))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "limit must be in [1e-4, 60] seconds");
        check_grid_barrier(absent_block, (unsigned long long)(limit_seconds * 1e9), (cudaStream_t)stream,
                           elapsed_seconds);
    });
}

gu_status gu_debug_fail_allocations(int64_t after, int64_t count)
{
    return guarded([&] {
        if (after < 0 || count < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "after and count must be >= 0");
        set_alloc_failures(after, count);
    });
}

gu_status gu_timer_start(void *stream, gu_timer *out)
{
    return guarded([&] {
        if (!out) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null timer");
        std::unique_ptr<gu_timer_s> t(new gu_timer_s());
        GU_CUDA_CHECK(cudaEventCreate(&t->a));
        GU_CUDA_CHECK(cudaEventCreate(&t->b));
        GU_CUDA_CHECK(cudaEventRecord(t->a, (cudaStream_t)stream));
        *out = t.release();
    });
}

gu_status gu_timer_stop(gu_timer t, void *stream, double *seconds)
{
    return guarded([&] {
        if (!t) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null timer");
        std::unique_ptr<gu_timer_s> own(t);
        GU_CUDA_CHECK(cudaEventRecord(t->b, (cudaStream_t)stream));
        GU_CUDA_CHECK(cudaEventSynchronize(t->b));
        float ms = 0;
        GU_CUDA_CHECK(cudaEventElapsedTime(&ms, t->a, t->b));
        cudaEventDestroy(t->a);
        cudaEventDestroy(t->b);
        if (seconds) *seconds = ms / 1000.0;
    });
}

// ---- host graphs -----------------------------------------------------------------
static gu_status make_hgraph(gu_hgraph *out, const std::function<HostGraph()> &fn)
{
    return guarded([&] {
        if (!out) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output handle");
        std::unique_ptr<gu_hgraph_s> h(new gu_hgraph_s());
        h->h = fn();
        *out = h.release();
    });
}

gu_status gu_hgraph_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute,
                         gu_hgraph *out)
{
    return make_hgraph(out, [&] { return gen_rmat(scale, edge_factor, a, b, c, seed, permute != 0); });
}

gu_status gu_hgraph_er(int32_t n, int64_t m, uint64_t seed, gu_hgraph *out)
{
    return make_hgraph(out, [&] { return gen_er(n, m, seed); });
}

gu_status gu_hgraph_grid(int32_t rows, int32_t cols, double p_delete, uint64_t seed, gu_hgraph *out)
{
    return make_hgraph(out, [&] { return gen_grid(rows, cols, p_delete, seed); });
}

gu_status gu_hgraph_dag(int32_t n, int64_t m, uint64_t seed, gu_hgraph *out)
{
    return make_hgraph(out, [&] { return gen_dag(n, m, seed); });
}

gu_status gu_hgraph_from_edges(int32_t n, const int32_t *u, const int32_t *v, int64_t count, int symmetric,
                               gu_hgraph *out)
{
    return make_hgraph(out, [&] {
        if (n < 0 || count < 0 || (count > 0 && (!u || !v))) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad edge list");
        std::vector<int32_t> eu(u, u + count), ev(v, v + count);
        for (int64_t i = 0; i < count; ++i)
            if (eu[i] < 0 || eu[i] >= n || ev[i] < 0 || ev[i] >= n)
                throw gu_error(GU_ERR_INVALID_ARGUMENT, "edge endpoint out of range");
        HostGraph g;
        g.n = n;
        g.directed = symmetric == 0;
        build_csr(n, eu, ev, symmetric != 0, g.R, g.C);
        return g;
    });
}

gu_status gu_hgraph_arrays(gu_hgraph h, const int32_t **R, const int32_t **C, int32_t *n, int64_t *m, int *directed)
{
    return guarded([&] {
        if (!h) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        if (R) *R = h->h.R.data();
        if (C) *C = h->h.C.data();
        if (n) *n = h->h.n;
        if (m) *m = h->h.m();
        if (directed) *directed = h->h.directed ? 1 : 0;
    });
}

gu_status gu_hgraph_from_csr(const int32_t *R, const int32_t *C, int32_t n, int64_t m, int directed, gu_hgraph *out)
{
    return make_hgraph(out, [&] {
        if (n < 0 || m < 0 || !R || (m > 0 && !C)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad CSR arrays");
        if (R[0] != 0 || R[n] != m) throw gu_error(GU_ERR_INVALID_ARGUMENT, "R must start at 0 and end at m");
        for (int32_t v = 0; v < n; ++v)
            if (R[v + 1] < R[v]) throw gu_error(GU_ERR_INVALID_ARGUMENT, "R must be non-decreasing");
        for (int64_t e = 0; e < m; ++e)
            if (C[e] < 0 || C[e] >= n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "column index out of range");
        HostGraph g;
        g.n = n;
        g.directed = directed != 0;
        g.R.assign(R, R + n + 1);
        g.C.assign(C, C + m);
        return g;
    });
}

gu_status gu_hgraph_parse(const char *path, const char *format, gu_hgraph *out)
{
    return make_hgraph(out, [&] { return parse_graph_file(path, format); });
}

gu_status gu_hgraph_write_csr(gu_hgraph h, const char *path)
{
    return guarded([&] {
        if (!h) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        write_csr_cache(h->h, path);
    });
}

gu_status gu_hgraph_write_edgelist(gu_hgraph h, const char *path, int header)
{
    return guarded([&] {
        if (!h) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        write_edgelist(h->h, path, header != 0);
    });
}

gu_status gu_hgraph_count_degree_zero(gu_hgraph h, uint64_t *count)
{
    return guarded([&] {
        if (!h || !count) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null argument");
        *count = count_degree_zero(h->h);
    });
}

gu_status gu_hgraph_destroy(gu_hgraph h)
{
    delete h;
    return GU_OK;
}

gu_status gu_sources(int32_t n, int32_t k, uint64_t seed, int32_t *out_host)
{
    return guarded([&] {
        if (!out_host && k > 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output");
        std::vector<int32_t> s = gen_sources(n, k, seed);
        std::memcpy(out_host, s.data(), sizeof(int32_t) * (size_t)k);
    });
}

// ---- device graphs -------------------------------------------------------------
gu_status gu_graph_create(const int32_t *R_host, const int32_t *C_host, int32_t n, int64_t m, int directed,
                          void *stream, gu_graph *out)
{
    return guarded([&] {
        if (!out) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output handle");
        std::unique_ptr<gu_graph_s> h(new gu_graph_s());
        h->g.reset(create_device_graph(R_host, C_host, n, m, directed != 0, (cudaStream_t)stream));
        *out = h.release();
    });
}

gu_status gu_graph_destroy(gu_graph g)
{
    return guarded([&] {
        if (!g) return;
        {
            std::lock_guard<std::mutex> lk(g->g->mu);
        }
        delete g;
    });
}

gu_status gu_graph_info(gu_graph g, int32_t *n, int64_t *m, int *directed, size_t *device_bytes)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        if (n) *n = g->g->n;
        if (m) *m = g->g->m;
        if (directed) *directed = g->g->directed ? 1 : 0;
        if (device_bytes) *device_bytes = g->g->bytes + g->g->ws.bytes;
    });
}

gu_status gu_graph_last_launch(gu_graph g, double *kernel_seconds, int *td_levels, int *bu_levels, int *max_level)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        if (!dg.timed) throw gu_error(GU_ERR_INVALID_ARGUMENT, "no launch recorded on this graph yet");
        GU_CUDA_CHECK(cudaEventSynchronize(dg.ev_stop));
        float ms = 0;
        GU_CUDA_CHECK(cudaEventElapsedTime(&ms, dg.ev_start, dg.ev_stop));
        if (kernel_seconds) *kernel_seconds = ms / 1000.0;
        int err = 0, td = 0, bu = 0, ml = 0;
        if (dg.ws.ptr) msbfs_read_status(dg, &err, &td, &bu, &ml);
        if (td_levels) *td_levels = td;
        if (bu_levels) *bu_levels = bu;
        if (max_level) *max_level = ml;
    });
}

gu_status gu_graph_launch_times(gu_graph g, int max_entries, double *kernel_seconds, int *count)
{
    return guarded([&] {
        if (!g || max_entries < 0 || (max_entries > 0 && !kernel_seconds))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad arguments");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        const int n = std::min(dg.ring_count, max_entries);
        for (int i = 0; i < n; ++i) {  // oldest first
            const int slot = (dg.ring_next - n + i + 2 * DeviceGraph::LAUNCH_RING) % DeviceGraph::LAUNCH_RING;
            GU_CUDA_CHECK(cudaEventSynchronize(dg.ring_stop[slot]));
            float ms = 0;
            GU_CUDA_CHECK(cudaEventElapsedTime(&ms, dg.ring_start[slot], dg.ring_stop[slot]));
            kernel_seconds[i] = ms / 1000.0;
        }
        if (count) *count = n;
    });
}

gu_status gu_graph_level_profile(gu_graph g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                                 int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms, int *count)
{
    return guarded([&] {
        if (!g || max_entries < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad arguments");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        if (!dg.timed || !dg.ws.ptr) throw gu_error(GU_ERR_INVALID_ARGUMENT, "no launch recorded on this graph yet");
        GU_CUDA_CHECK(cudaEventSynchronize(dg.ev_stop));
        const int c = dg.timeline == 1
                          ? bc_read_timeline(dg, max_entries, batch, level, kind, frontier_vertices, frontier_edges, t_ms)
                          : msbfs_read_timeline(dg, max_entries, batch, level, kind, frontier_vertices, frontier_edges, t_ms);
        if (count) *count = c;
    });
}

gu_status gu_graph_level_idle(gu_graph g, int max_entries, double *idle_cta_ms, int *nblocks, int *count)
{
    return guarded([&] {
        if (!g || max_entries < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad arguments");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        if (!dg.timed || !dg.ws.ptr || dg.timeline == 1)
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "no batched search recorded on this graph yet");
        GU_CUDA_CHECK(cudaEventSynchronize(dg.ev_stop));
        const int c = msbfs_read_idle(dg, max_entries, idle_cta_ms, nblocks);
        if (count) *count = c;
    });
}

gu_status gu_graph_arrays(gu_graph g, const int32_t **R_dev, const int32_t **C_dev, const int32_t **RT_dev,
                          const int32_t **CT_dev)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        if (R_dev) *R_dev = g->g->R;
        if (C_dev) *C_dev = g->g->C;
        if (RT_dev) *RT_dev = g->g->RT;
        if (CT_dev) *CT_dev = g->g->CT;
    });
}

// ---- BFS ---------------------------------------------------------------------------
static void validate_sources_host(const int32_t *s, int32_t k, int32_t n)
{
    for (int32_t i = 0; i < k; ++i)
        if (s[i] < 0 || s[i] >= n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range");
}

static void bfs_device(DeviceGraph &g, int variant, const int32_t *sources_dev, int32_t k, int32_t *dist_dev,
                       int64_t ld, cudaStream_t stream)
{
    if (k == 0) return;
    if (variant == GU_BFS_PLAIN) {
        launch_plain_bfs(g, sources_dev, k, dist_dev, ld, stream);
        GU_CUDA_CHECK(cudaStreamSynchronize(stream));
        GU_CUDA_CHECK(cudaGetLastError());
        return;
    }
    MsOptions opt;
    opt.variant = variant;
    if (variant == GU_BFS_AUTO && g.tune.set) {  // the measured choice (gu_graph_autotune)
        if (g.tune.engine == GU_ENGINE_PER_SOURCE &&
            launch_local_bfs(g, sources_dev, k, dist_dev, ld, nullptr, nullptr, stream))
            return;
        if (g.tune.engine == GU_ENGINE_ONE_CTA) {
            launch_plain_bfs(g, sources_dev, k, dist_dev, ld, stream);
            GU_CUDA_CHECK(cudaStreamSynchronize(stream));
            GU_CUDA_CHECK(cudaGetLastError());
            return;
        }
        if (g.tune.engine == GU_ENGINE_BATCHED) {
            opt.alpha = g.tune.alpha;
            opt.beta = g.tune.beta;
            opt.batch_words = g.tune.words;
            opt.max_blocks = g.tune.ctas_per_sm > 0 ? g.sm_count * g.tune.ctas_per_sm : 0;
            opt.rare_frac = g.tune.rare_frac;
            opt.tuned = true;
        }
    } else if (variant == GU_BFS_AUTO) {
        const AutoEngine eng = auto_engine(g, true);
        if (eng == AutoEngine::LOCAL && launch_local_bfs(g, sources_dev, k, dist_dev, ld, nullptr, nullptr, stream))
            return;
        if (eng == AutoEngine::PLAIN) {
            launch_plain_bfs(g, sources_dev, k, dist_dev, ld, stream);
            GU_CUDA_CHECK(cudaStreamSynchronize(stream));
            GU_CUDA_CHECK(cudaGetLastError());
            return;
        }
    }
    launch_msbfs(g, sources_dev, k, dist_dev, ld, opt, stream, nullptr);
    check_dev_status(g, stream);
}

// ---- autotuning AUTO ------------------------------------------------------------------
static double last_kernel_seconds(DeviceGraph &g)
{
    GU_CUDA_CHECK(cudaEventSynchronize(g.ev_stop));
    float ms = 0;
    GU_CUDA_CHECK(cudaEventElapsedTime(&ms, g.ev_start, g.ev_stop));
    return ms / 1000.0;
}

gu_status gu_graph_autotune(gu_graph g, const int32_t *sources_dev, int32_t k, gu_tuning *best, gu_tuning *trials,
                            int max_trials, int *ntrials)
{
    return guarded([&] {
        if (!g || !sources_dev || k <= 0 || max_trials < 0 || (max_trials > 0 && !trials))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad arguments");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        std::vector<int32_t> hs((size_t)k);
        GU_CUDA_CHECK(cudaMemcpy(hs.data(), sources_dev, sizeof(int32_t) * k, cudaMemcpyDeviceToHost));
        validate_sources_host(hs.data(), k, dg.n);
        const size_t row_bytes = (size_t)k * (size_t)dg.n * sizeof(int32_t);
        if (row_bytes > ((size_t)4 << 30)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "sample too large: k x n x 4 > 4 GiB");
        struct Scratch {  // released on every exit, errors included
            int32_t *rows = nullptr;
            cudaStream_t st = nullptr;
            ~Scratch()
            {
                if (st) cudaStreamDestroy(st);
                if (rows) cudaFree(rows);
            }
        } scratch;
        GU_CUDA_CHECK(dev_malloc(reinterpret_cast<void **>(&scratch.rows), row_bytes ? row_bytes : 4));
        GU_CUDA_CHECK(cudaStreamCreateWithFlags(&scratch.st, cudaStreamNonBlocking));
        int32_t *const rows = scratch.rows;
        const cudaStream_t st = scratch.st;
        std::vector<gu_tuning> cand;
        auto add = [&](int engine, float alpha, float beta, int words, int ctas = 0, float rare = MS_RARE_FRAC) {
            gu_tuning t;
            t.engine = engine;
            t.alpha = alpha;
            t.beta = beta;
            t.words = words;
            t.ctas_per_sm = ctas;
            t.rare_frac = rare;
            t.seconds = 0;
            cand.push_back(t);
        };
        if (dg.max_degree <= 16) add(GU_ENGINE_PER_SOURCE, 0, 0, 0);
        if (dg.n <= 65536) add(GU_ENGINE_ONE_CTA, 0, 0, 0);
        const int wd = msbfs_words_for(k);
        const float grid[][2] = {{2.f, 24.f}, {1.f, 24.f}, {4.f, 24.f}, {8.f, 24.f}, {2.f, 12.f}, {2.f, 48.f}};
        for (int w = wd; w >= 1 && w >= wd / 2; w /= 2) {
            for (const auto &ab : grid) add(GU_ENGINE_BATCHED, ab[0], ab[1], w);
            add(GU_ENGINE_BATCHED, 2.f, 24.f, w, 1);  // half the grid: one CTA per SM
            add(GU_ENGINE_BATCHED, 2.f, 24.f, w, 0, 0.06f);  // more sources left to the bottom-up parts
            add(GU_ENGINE_BATCHED, 2.f, 24.f, w, 0, 1.f / 3.f);
        }
        const DeviceGraph::Tuning saved = dg.tune;
        gu_tuning pick{};
        pick.seconds = -1;
        int nt = 0;
        try {
            for (gu_tuning &t : cand) {
                dg.tune.set = true;
                dg.tune.engine = t.engine;
                dg.tune.alpha = t.alpha;
                dg.tune.beta = t.beta;
                dg.tune.words = t.words;
                dg.tune.ctas_per_sm = t.ctas_per_sm;
                dg.tune.rare_frac = t.rare_frac;
                bool fell_back = false;
                double best_t = 1e30;
                for (int rep = 0; rep < 3; ++rep) {
                    if (t.engine == GU_ENGINE_PER_SOURCE &&
                        !launch_local_bfs(dg, sources_dev, k, rows, dg.n, nullptr, nullptr, st)) {
                        fell_back = true;  // a frontier overflowed the shared queues: not a candidate here
                        break;
                    }
                    if (t.engine != GU_ENGINE_PER_SOURCE) bfs_device(dg, GU_BFS_AUTO, sources_dev, k, rows, dg.n, st);
                    const double sec = last_kernel_seconds(dg);
                    if (rep > 0 || sec > 0.02) best_t = std::min(best_t, sec);  // first run warms up, unless slow
                    if (pick.seconds >= 0 && sec > 3 * pick.seconds) {            // far behind: one run is enough
                        best_t = std::min(best_t, sec);
                        break;
                    }
                }
                if (fell_back) continue;
                t.seconds = best_t;
                if (nt < max_trials) trials[nt] = t;
                ++nt;
                if (pick.seconds < 0 || t.seconds < pick.seconds) pick = t;
            }
        } catch (...) {
            dg.tune = saved;
            throw;
        }
        GU_CUDA_CHECK(cudaStreamSynchronize(st));
        if (pick.seconds < 0) {
            dg.tune = saved;
            throw gu_error(GU_ERR_INTERNAL, "no candidate completed");
        }
        dg.tune.set = true;
        dg.tune.engine = pick.engine;
        dg.tune.alpha = pick.alpha;
        dg.tune.beta = pick.beta;
        dg.tune.words = pick.words;
        dg.tune.ctas_per_sm = pick.ctas_per_sm;
        dg.tune.rare_frac = pick.rare_frac;
        if (best) *best = pick;
        if (ntrials) *ntrials = std::min(nt, max_trials);
    });
}

gu_status gu_graph_set_tuning(gu_graph g, const gu_tuning *t)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        if (!t) {
            dg.tune = DeviceGraph::Tuning();
            return;
        }
        if (t->engine < GU_ENGINE_BATCHED || t->engine > GU_ENGINE_ONE_CTA)
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown engine");
        if (t->engine == GU_ENGINE_PER_SOURCE && dg.max_degree > 16)
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "the per-source engine needs out-degree <= 16");
        if (t->engine == GU_ENGINE_BATCHED &&
            (!(t->alpha > 0) || !(t->beta > 0) || (t->words != 0 && t->words != 1 && t->words != 2 && t->words != 4)))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "batched engine needs alpha, beta > 0 and words 0, 1, 2 or 4");
        if (t->ctas_per_sm < 0 || t->ctas_per_sm > 2)
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "ctas_per_sm must be 0, 1 or 2");
        if (!(t->rare_frac >= 0.f && t->rare_frac <= 1.f))
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "rare_frac must be in [0, 1]");
        dg.tune.set = true;
        dg.tune.engine = t->engine;
        dg.tune.alpha = t->alpha;
        dg.tune.beta = t->beta;
        dg.tune.words = t->words;
        dg.tune.ctas_per_sm = t->ctas_per_sm;
        dg.tune.rare_frac = t->rare_frac;
    });
}

static void check_bfs_args(gu_graph g, int variant, int32_t k, int64_t ld)
{
    if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
    if (variant < GU_BFS_AUTO || variant > GU_BFS_PLAIN) throw gu_error(GU_ERR_INVALID_ARGUMENT, "unknown BFS variant");
    if (k < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "k must be >= 0");
    if (ld < g->g->n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
}

gu_status gu_bfs(gu_graph g, int variant, const int32_t *sources_dev, int32_t k, int32_t *dist_dev, int64_t ld,
                 void *stream)
{
    return guarded([&] {
        check_bfs_args(g, variant, k, ld);
        if (k > 0 && (!sources_dev || !dist_dev)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null device buffer");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        // Source ids are checked before they index anything: by the batched kernel
        // itself where it is the engine that runs (it skips a bad id and reports it
        // as GU_ERR_INVALID_ARGUMENT), else here on the host, which costs a copy and a
        // synchronisation per call.
        const bool batched = variant != GU_BFS_PLAIN &&
                             (variant != GU_BFS_AUTO ||
                              (dg.tune.set ? dg.tune.engine == GU_ENGINE_BATCHED
                                           : auto_engine(dg, true) == AutoEngine::BATCHED));
        if (!batched && k > 0) {
            std::vector<int32_t> hs((size_t)k);
            GU_CUDA_CHECK(cudaMemcpyAsync(hs.data(), sources_dev, sizeof(int32_t) * (size_t)k, cudaMemcpyDeviceToHost,
                                          (cudaStream_t)stream));
            GU_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
            validate_sources_host(hs.data(), k, dg.n);
        }
        bfs_device(dg, variant, sources_dev, k, dist_dev, ld, (cudaStream_t)stream);
    });
}

gu_status gu_bfs_host(gu_graph g, int variant, const int32_t *sources_host, int32_t k, int32_t *dist_host, int64_t ld,
                      void *stream)
{
    return guarded([&] {
        check_bfs_args(g, variant, k, ld);
        if (k > 0 && (!sources_host || !dist_host)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null host buffer");
        DeviceGraph &dg = *g->g;
        validate_sources_host(sources_host, k, dg.n);
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        cudaStream_t st = (cudaStream_t)stream;
        if (k == 0) return;
        const size_t src_bytes = ((sizeof(int32_t) * (size_t)k + 255) / 256) * 256;
        char *io = (char *)dg.io.get(src_bytes + sizeof(int32_t) * (size_t)k * (size_t)dg.n);
        int32_t *d_src = reinterpret_cast<int32_t *>(io);
        int32_t *d_dist = reinterpret_cast<int32_t *>(io + src_bytes);
        GU_CUDA_CHECK(cudaMemcpyAsync(d_src, sources_host, sizeof(int32_t) * (size_t)k, cudaMemcpyHostToDevice, st));
        // Rows leave the device while later sources are still being searched: the
        // sources go in chunks (a small first one, so the host link starts early,
        // then one 256-source engine batch each), each searched on `st`, and each
        // chunk's rows are copied on the graph's copy stream once its search has
        // finished.  The host link, not the search, then bounds the call.
        if (!dg.copy_st) GU_CUDA_CHECK(cudaStreamCreateWithFlags(&dg.copy_st, cudaStreamNonBlocking));
        struct CopyFence {  // no copy into the caller's rows outlives the call, errors included
            cudaStream_t s;
            ~CopyFence() { cudaStreamSynchronize(s); }
        } fence{dg.copy_st};
        const size_t row = sizeof(int32_t) * (size_t)dg.n;
        int32_t b = 0;
        while (b < k) {
            const int32_t e = b == 0 ? std::min(k, 64) : std::min(k, b + 256);
            bfs_device(dg, variant, d_src + b, e - b, d_dist + (size_t)b * dg.n, dg.n, st);  // synchronises st
            GU_CUDA_CHECK(cudaMemcpy2DAsync(dist_host + (size_t)b * (size_t)ld, sizeof(int32_t) * (size_t)ld,
                                            d_dist + (size_t)b * dg.n, row, row, (size_t)(e - b),
                                            cudaMemcpyDeviceToHost, dg.copy_st));
            b = e;
        }
        GU_CUDA_CHECK(cudaStreamSynchronize(dg.copy_st));
    });
}

// ---- shortest-path counts, betweenness, diameter, reachability -------------------------
static void check_sources_device(DeviceGraph &dg, const int32_t *sources_dev, int32_t k, cudaStream_t st)
{
    if (k < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "k must be >= 0");
    if (k > 0 && !sources_dev) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null sources");
    std::vector<int32_t> hs((size_t)k);
    if (k > 0) {
        GU_CUDA_CHECK(cudaMemcpyAsync(hs.data(), sources_dev, sizeof(int32_t) * (size_t)k, cudaMemcpyDeviceToHost, st));
        GU_CUDA_CHECK(cudaStreamSynchronize(st));
    }
    validate_sources_host(hs.data(), k, dg.n);
}

static void finish_bc(DeviceGraph &dg, cudaStream_t st)
{
    GU_CUDA_CHECK(cudaStreamSynchronize(st));
    GU_CUDA_CHECK(cudaGetLastError());
    int err = 0;
    bc_read_status(dg, &err, nullptr);
    if (err == DEV_ERR_BARRIER_TIMEOUT) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit");
    if (err == 3) throw gu_error(GU_ERR_CAPACITY, "BFS deeper than the level store (raise GU_BC_LEVEL_BUDGET_MB)");
    if (err != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(err));
}

gu_status gu_sigma(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t *dist_dev, uint64_t *sigma_dev,
                   int64_t ld, void *stream)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        DeviceGraph &dg = *g->g;
        if (ld < dg.n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
        if (k > 0 && !sigma_dev) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null sigma rows");
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        cudaStream_t st = (cudaStream_t)stream;
        check_sources_device(dg, sources_dev, k, st);
        if (k == 0) return;
        BcOptions opt;
        launch_bc(dg, sources_dev, k, opt, nullptr, dist_dev, sigma_dev, nullptr, ld, false, st);
        finish_bc(dg, st);
    });
}

gu_status gu_bc(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t batch, double *bc_dev, double *delta_dev,
                int64_t ld, void *stream)
{
    return guarded([&] {
        if (!g) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph");
        DeviceGraph &dg = *g->g;
        if (!bc_dev) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null bc output");
        if (delta_dev && ld < dg.n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        cudaStream_t st = (cudaStream_t)stream;
        check_sources_device(dg, sources_dev, k, st);
        if (k == 0) {
            GU_CUDA_CHECK(cudaMemsetAsync(bc_dev, 0, sizeof(double) * (size_t)dg.n, st));
            GU_CUDA_CHECK(cudaStreamSynchronize(st));
            return;
        }
        BcOptions opt;
        opt.batch = batch;
        launch_bc(dg, sources_dev, k, opt, bc_dev, nullptr, nullptr, delta_dev, ld, true, st);
        finish_bc(dg, st);
    });
}

// ---- load-balanced search and race-and-resolve ------------------------------------
// per-device scratch for calls without a graph handle (grown on demand)
static Workspace &device_scratch(int dev)
{
    static std::mutex mu;
    static Workspace ws[128];
    if (dev < 0 || dev >= 128) throw gu_error(GU_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    return ws[dev];
}
static std::mutex g_scratch_call_mu;

gu_status gu_lbs(const int32_t *counts_dev, int32_t N, int32_t *scanned_dev, int32_t *result_dev,
                 int64_t result_capacity, int32_t *total_dev, int64_t *total_host, void *stream)
{
    return guarded([&] {
        std::lock_guard<std::mutex> lk(g_scratch_call_mu);
        int dev = 0;
        GU_CUDA_CHECK(cudaGetDevice(&dev));
        Workspace &ws = device_scratch(dev);
        const size_t need = lbs_scratch_bytes(N, result_capacity);
        void *p = ws.get(need);
        launch_lbs(counts_dev, N, scanned_dev, result_dev, result_capacity, total_dev, total_host, p, ws.bytes,
                   (cudaStream_t)stream);
    });
}

gu_status gu_lbs_last_ms(double *ms)
{
    return guarded([&] {
        if (!ms) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output");
        int dev = 0;
        GU_CUDA_CHECK(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> lk(g_scratch_call_mu);
        *ms = lbs_last_ms(dev);
    });
}

gu_status gu_race_and_resolve(const int32_t *predicates_dev, int32_t nwarps, int32_t *winners_dev, void *stream)
{
    return guarded([&] {
        if (nwarps < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "nwarps must be >= 0");
        if (nwarps > 0 && (!predicates_dev || !winners_dev)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null buffer");
        launch_race_and_resolve(predicates_dev, nwarps, winners_dev, (cudaStream_t)stream);
    });
}

// ---- many searches in one work-queue launch -----------------------------------------
gu_status gu_bfs_many(const gu_search_item *items, int32_t count, void *stream)
{
    return guarded([&] {
        if (count < 0 || (count > 0 && !items)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad item list");
        if (count == 0) return;
        std::vector<DeviceGraph *> graphs;
        for (int32_t i = 0; i < count; ++i) {
            if (!items[i].graph) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null graph in item " + std::to_string(i));
            graphs.push_back(items[i].graph->g.get());
        }
        const int dev = graphs[0]->device;
        for (DeviceGraph *g : graphs)
            if (g->device != dev) throw gu_error(GU_ERR_INVALID_ARGUMENT, "all graphs must live on one device");
        std::sort(graphs.begin(), graphs.end());
        graphs.erase(std::unique(graphs.begin(), graphs.end()), graphs.end());
        std::vector<std::unique_lock<std::mutex>> locks;  // in address order: no lock-order cycle
        for (DeviceGraph *g : graphs) locks.emplace_back(g->mu);
        DeviceScope ds(dev);
        std::vector<MsQueueRequest> reqs((size_t)count);
        for (int32_t i = 0; i < count; ++i) {
            const gu_search_item &it = items[i];
            MsQueueRequest &r = reqs[(size_t)i];
            r.g = it.graph->g.get();
            r.sources = it.sources_dev;
            r.k = it.k;
            r.dist = it.dist_dev;
            r.ld = it.ld;
            r.reach = reinterpret_cast<unsigned long long *>(it.reach_dev);
            if (it.k < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "k must be >= 0 (item " + std::to_string(i) + ")");
            if (it.k > 0 && (!it.sources_dev || (!it.dist_dev && !it.reach_dev)))
                throw gu_error(GU_ERR_INVALID_ARGUMENT, "item " + std::to_string(i) + " needs sources and an output");
            if (it.dist_dev && it.ld < r.g->n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "ld must be >= n");
        }
        static std::mutex mu;  // the per-device queue workspace is one per process
        static Workspace wsq[128];
        if (dev < 0 || dev >= 128) throw gu_error(GU_ERR_UNSUPPORTED, "device ordinal out of range");
        std::lock_guard<std::mutex> lk(mu);
        cudaStream_t st = (cudaStream_t)stream;
        const MsQueueLaunch L = launch_msbfs_queue(reqs, wsq[dev], graphs[0]->sm_count, 0, st);
        GU_CUDA_CHECK(cudaStreamSynchronize(st));
        const int e = msbfs_queue_error(wsq[dev], L);
        if (e == DEV_ERR_BAD_SOURCE) throw gu_error(GU_ERR_INVALID_ARGUMENT, "source vertex out of range");
        if (e == DEV_ERR_BARRIER_TIMEOUT) throw gu_error(GU_ERR_TIMEOUT, "a device-side wait exceeded its limit");
        if (e != 0) throw gu_error(GU_ERR_INTERNAL, "device reported error code " + std::to_string(e));
    });
}

// ---- serving -----------------------------------------------------------------------
struct gu_server_s {
    Server *s = nullptr;
};

gu_status gu_server_create(size_t hbm_budget_bytes, int slots, int max_batch_sources, gu_server *out)
{
    return guarded([&] {
        if (!out || slots < 1 || max_batch_sources < 1 || hbm_budget_bytes == 0)
            throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad server parameters");
        std::unique_ptr<gu_server_s> h(new gu_server_s());
        h->s = server_create(hbm_budget_bytes, slots, max_batch_sources);
        *out = h.release();
    });
}

gu_status gu_server_destroy(gu_server s)
{
    return guarded([&] {
        if (!s) return;
        server_destroy(s->s);
        delete s;
    });
}

gu_status gu_server_submit(gu_server s, gu_graph g, int query, const int32_t *sources_host, int32_t k, void *out_host,
                           int64_t *request_id)
{
    return guarded([&] {
        if (!s || !g || !request_id) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null argument");
        *request_id = server_submit(s->s, query, g->g.get(), sources_host, k, out_host);
    });
}

gu_status gu_server_wait(gu_server s, int64_t request_id, double timeout_s, double *latency_s)
{
    try {
        if (!s) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null server");
        std::string err;
        const gu_status st = server_wait(s->s, request_id, timeout_s, latency_s, err);
        if (st != GU_OK) set_last_error(st == GU_ERR_PENDING ? "request still running" : err);
        return st;
    } catch (const gu_error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return GU_ERR_INTERNAL;
    }
}

gu_status gu_server_stats(gu_server s, int64_t *completed, int64_t *batches, double *p50_s, double *p99_s,
                          double *mean_requests_per_batch)
{
    return guarded([&] {
        if (!s) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null server");
        server_stats(s->s, completed, batches, p50_s, p99_s, mean_requests_per_batch);
    });
}

gu_status gu_diameter(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t *diameter, void *stream)
{
    return guarded([&] {
        if (!g || !diameter) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null argument");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        cudaStream_t st = (cudaStream_t)stream;
        check_sources_device(dg, sources_dev, k, st);
        *diameter = 0;
        if (k == 0) return;
        int ml = 0;
        if (auto_engine(dg, false) == AutoEngine::LOCAL &&
            launch_local_bfs(dg, sources_dev, k, nullptr, dg.n, nullptr, &ml, st)) {
            *diameter = ml;
            return;
        }
        MsOptions opt;
        opt.variant = GU_BFS_AUTO;
        launch_msbfs(dg, sources_dev, k, nullptr, dg.n, opt, st, nullptr);
        check_dev_status(dg, st);
        int err = 0, td = 0, bu = 0;
        msbfs_read_status(dg, &err, &td, &bu, &ml);
        *diameter = ml;
    });
}

gu_status gu_power_start(int device, int period_ms, gu_power *out)
{
    return guarded([&] {
        if (!out) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null output handle");
        std::unique_ptr<gu_power_s> p(new gu_power_s());
        p->s = power_start(device, period_ms);
        *out = p.release();
    });
}

gu_status gu_power_stop(gu_power p, double *avg_watts, int64_t *samples)
{
    return guarded([&] {
        if (!p) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null sampler");
        std::unique_ptr<gu_power_s> h(p);
        long long n = 0;
        power_stop(h->s, avg_watts, &n);
        h->s = nullptr;
        if (samples) *samples = n;
    });
}

gu_status gu_dag_reach(gu_graph g, int64_t *counts_dev, int64_t *total_pairs, void *stream)
{
    return guarded([&] {
        if (!g || !total_pairs || (g->g->n > 0 && !counts_dev)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null argument");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        dag_reach(dg, counts_dev, total_pairs, (cudaStream_t)stream);
    });
}

gu_status gu_reach(gu_graph g, const int32_t *sources_dev, int32_t k, int64_t *counts_dev, void *stream)
{
    return guarded([&] {
        if (!g || (k > 0 && !counts_dev)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null argument");
        DeviceGraph &dg = *g->g;
        std::lock_guard<std::mutex> lk(dg.mu);
        DeviceScope ds(dg.device);
        cudaStream_t st = (cudaStream_t)stream;
        check_sources_device(dg, sources_dev, k, st);
        if (k == 0) return;
        GU_CUDA_CHECK(cudaMemsetAsync(counts_dev, 0, sizeof(int64_t) * (size_t)k, st));
        auto *cnt = reinterpret_cast<unsigned long long *>(counts_dev);
        if (auto_engine(dg, false) == AutoEngine::LOCAL &&
            launch_local_bfs(dg, sources_dev, k, nullptr, dg.n, cnt, nullptr, st))
            return;
        GU_CUDA_CHECK(cudaMemsetAsync(counts_dev, 0, sizeof(int64_t) * (size_t)k, st));
        MsOptions opt;
        opt.variant = GU_BFS_AUTO;
        opt.reach = cnt;
        launch_msbfs(dg, sources_dev, k, nullptr, dg.n, opt, st, nullptr);
        check_dev_status(dg, st);
    });
}

}  // extern "C"
