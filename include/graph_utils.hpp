// graph_utils.hpp -- C++ drop-in for graph-utils' multi-source search entry points.
//
// Header-only layer over the C ABI (gu.h), so it compiles against the caller's
// own host_graph (the reference's parse.h:15-35) and adds no C++ symbols to the
// library.  Include the reference's parse.h / util.h first, or define
// GU_DEFINE_HOST_TYPES to get layout-compatible host_graph / program_options.
//
// Replaces: device_graph (device_graph.h:7-22); multi_search_*_setup
// (linear_with_atomics.cuh:14, edge_parallel.cuh:13, warp_based.cuh:15,
// CTA_warp.cuh:15, scan_based.cuh:15, shuffle_based.cuh:16);
// betweenness_centrality_setup (betweenness_centrality.cuh:14);
// count_shortest_paths_setup (count_shortest_paths.cuh:13);
// diameter_sampling_setup (diameter_sampling.cuh:13); transitive_closure_setup
// (transitive_closure.cuh:13); extract_edges_{block,warp}
// (load_balanced_search.cuh:12-13, called as host functions here, without the
// <<<1, BLOCK_SIZE>>> launch configuration); parse / parse_metis / parse_snap /
// parse_market (parse.h:37-40); get_reachability_dag (dag_reachability.h:15);
// start_clock / end_clock, choose_device and power_measurer (util_device.cuh:38-60).
//
// Semantics kept: every source in [start, end) is searched; the returned rows
// are those of the last R = min(end - start, #SMs) sources, source s in row
// (s - start) % R (the reference's one-CTA-per-source grid, common.cu:3-28, and
// its checker multi_search_test.cu:43-63).  Timing lines are printed like the
// reference's.  Errors throw std::runtime_error (the reference exits).
#pragma once

#include <algorithm>
#include <cmath>  // the reference's headers brought it in through CUDA's
#include <cstdint>
#include <cstdio>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>

#include "gu.h"

#ifdef GU_DEFINE_HOST_TYPES
class host_graph {
public:
    std::vector<int> C;  // neighbours
    std::vector<int> R;  // offsets
    std::vector<int> F;  // edge sources
    int n = 0;
    int m = 0;
    bool directed = false;
};
class program_options {
public:
    int device = -1;
    char *infile = nullptr;
    char *outfile = nullptr;
    bool verify = false;
    int approx = 0;
    char *format = nullptr;
    bool isTesla = false;
    bool nvml = false;
};
#endif

namespace gu_shim {

inline void check(gu_status s, const char *what)
{
    if (s != GU_OK) throw std::runtime_error(std::string(what) + ": " + gu_last_error());
}

inline int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// Device buffer owned by the shim for the duration of one call.
template <class T>
struct dbuf {
    T *p = nullptr;
    explicit dbuf(size_t count)
    {
        if (count && cudaMalloc((void **)&p, sizeof(T) * count) != cudaSuccess)
            throw std::runtime_error("cudaMalloc failed");
    }
    ~dbuf() { if (p) cudaFree(p); }
    dbuf(const dbuf &) = delete;
    dbuf &operator=(const dbuf &) = delete;
};

inline double seconds_since(const cudaEvent_t &a)
{
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(b);
    return ms / 1000.0;
}

struct timer {
    cudaEvent_t a;
    timer() { cudaEventCreate(&a); cudaEventRecord(a, 0); }
    ~timer() { cudaEventDestroy(a); }
    double stop() const { return seconds_since(a); }
};

// Rows of the last R sources of [start, end): returns R and the row of s.
inline int rows_for(int start, int end) { return std::min(end - start, sm_count()); }

}  // namespace gu_shim

// Timing, device choice and power sampling (util_device.cuh:38-60, util_device.cu:4-130).
inline void start_clock(cudaEvent_t &start, cudaEvent_t &end)
{
    cudaEventCreate(&start);
    cudaEventCreate(&end);
    cudaEventRecord(start, 0);
}

inline float end_clock(cudaEvent_t &start, cudaEvent_t &end)
{
    float ms = 0;
    cudaEventRecord(end, 0);
    cudaEventSynchronize(end);
    cudaEventElapsedTime(&ms, start, end);
    cudaEventDestroy(start);
    cudaEventDestroy(end);
    return ms / 1000.0f;  // seconds, as the reference returns
}

// op.device >= 0 selects it; -1 picks the device with the highest memory bandwidth.
inline void choose_device(program_options &op)
{
    int chosen = -1;
    gu_shim::check(gu_choose_device(op.device, &chosen), "choose_device");
    op.device = chosen;
    std::printf("Chosen device: %d\n", chosen);
}

// Board power over an interval, sampled every `period` ms (NVML, read-only).
class power_measurer {
public:
    power_measurer(long period, const program_options &op) : period_(period), device_(op.device < 0 ? 0 : op.device) {}
    ~power_measurer() { if (p_) gu_power_stop(p_, nullptr, nullptr); }
    void start_power_sample() { gu_shim::check(gu_power_start(device_, (int)period_, &p_), "start_power_sample"); }
    double end_power_sample()
    {
        double w = 0;
        int64_t samples = 0;
        gu_power p = p_;
        p_ = nullptr;
        gu_shim::check(gu_power_stop(p, &w, &samples), "end_power_sample");
        return w;
    }

private:
    long period_;
    int device_;
    gu_power p_ = nullptr;
};

class device_graph {
public:
    explicit device_graph(const host_graph &g) : n(g.n), m(g.m), directed(g.directed)
    {
        gu_shim::check(gu_graph_create(g.R.data(), g.m ? g.C.data() : nullptr, g.n, g.m, g.directed ? 1 : 0, nullptr,
                                       &handle),
                       "device_graph");
    }
    ~device_graph() { if (handle) gu_graph_destroy(handle); }
    device_graph(const device_graph &) = delete;
    device_graph &operator=(const device_graph &) = delete;

    int n;
    int m;
    bool directed;
    gu_graph handle = nullptr;
};

namespace gu_shim {

// Searches every source of [start, end) with `variant` in chunks and keeps the
// rows of the last R sources (row (s - start) % R).
inline std::vector<std::vector<int> > search_rows(const device_graph &g, int variant, int start, int end)
{
    std::vector<std::vector<int> > out;
    if (end <= start) return out;
    const int R = rows_for(start, end);
    out.assign((size_t)R, std::vector<int>((size_t)g.n));
    const int total = end - start;
    const int chunk = std::max(R, std::min(total, 4096));
    dbuf<int32_t> src((size_t)chunk), dist((size_t)chunk * g.n);
    std::vector<int32_t> hs((size_t)chunk);
    for (int c0 = start; c0 < end; c0 += chunk) {
        const int k = std::min(chunk, end - c0);
        for (int i = 0; i < k; ++i) hs[i] = c0 + i;
        cudaMemcpy(src.p, hs.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice);
        check(gu_bfs(g.handle, variant, src.p, k, dist.p, g.n, nullptr), "multi_search");
        for (int i = 0; i < k; ++i) {
            const int s = c0 + i;
            if (s < end - R) continue;
            cudaMemcpy(out[(size_t)((s - start) % R)].data(), dist.p + (size_t)i * g.n, sizeof(int) * g.n,
                       cudaMemcpyDeviceToHost);
        }
    }
    return out;
}

inline std::vector<int32_t> iota_sources(int start, int end)
{
    std::vector<int32_t> s((size_t)(end > start ? end - start : 0));
    for (int i = start; i < end; ++i) s[(size_t)(i - start)] = i;
    return s;
}

}  // namespace gu_shim

inline std::vector<std::vector<int> > multi_search_linear_atomics_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_LINEAR, start, end);
    std::printf("Time for baseline linear algorithm with atomics: %.9f s\n", t.stop());
    return r;
}

inline std::vector<std::vector<int> > multi_search_edge_parallel_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_EDGE, start, end);
    std::printf("Time for baseline edge-parallel algorithm: %.9f s\n", t.stop());
    return r;
}

inline std::vector<std::vector<int> > multi_search_warp_based_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_WARP, start, end);
    std::printf("Time for warp-based neighbor gathering: %.9f s\n", t.stop());
    return r;
}

inline std::vector<std::vector<int> > multi_search_CTA_warp_based_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_CTA_WARP, start, end);
    std::printf("Time for CTA+warp-based neighbor gathering: %.9f s\n", t.stop());
    return r;
}

inline std::vector<std::vector<int> > multi_search_scan_based_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_SCAN, start, end);
    std::printf("Time for scan-based neighbor gathering: %.9f s\n", t.stop());
    return r;
}

inline std::vector<std::vector<int> > multi_search_shuffle_based_setup(const device_graph &g, const program_options &,
                                                                       int start, int end)
{
    gu_shim::timer t;
    auto r = gu_shim::search_rows(g, GU_BFS_SHUFFLE, start, end);
    std::printf("Time for shuffle-based neighbor gathering: %.9f s\n", t.stop());
    return r;
}

inline void transitive_closure_setup(const device_graph &g, int start, int end, std::vector<std::vector<int> > &d)
{
    gu_shim::timer t;
    d = gu_shim::search_rows(g, GU_BFS_AUTO, start, end);
    std::printf("Time for shuffle-based transitive closure: %.9f s\n", t.stop());
}

inline int diameter_sampling_setup(const device_graph &g, int start, int end)
{
    gu_shim::timer t;
    std::vector<int32_t> hs = gu_shim::iota_sources(start, end);
    gu_shim::dbuf<int32_t> src(hs.size());
    if (!hs.empty()) cudaMemcpy(src.p, hs.data(), sizeof(int32_t) * hs.size(), cudaMemcpyHostToDevice);
    int32_t diam = 0;
    gu_shim::check(gu_diameter(g.handle, src.p, (int32_t)hs.size(), &diam, nullptr), "diameter_sampling");
    std::printf("Time for shuffle-based diameter sampling: %.9f s\n", t.stop());
    return diam;
}

// Rows of the last R sources (sigma), all sources searched.
inline void count_shortest_paths_setup(const device_graph &g, int start, int end,
                                       std::vector<std::vector<unsigned long long> > &sigma_h)
{
    gu_shim::timer t;
    sigma_h.clear();
    if (end > start) {
        const int R = gu_shim::rows_for(start, end);
        std::vector<int32_t> hs = gu_shim::iota_sources(start, end);
        gu_shim::dbuf<int32_t> src(hs.size());
        cudaMemcpy(src.p, hs.data(), sizeof(int32_t) * hs.size(), cudaMemcpyHostToDevice);
        gu_shim::dbuf<uint64_t> sig(hs.size() * (size_t)g.n);
        gu_shim::check(gu_sigma(g.handle, src.p, (int32_t)hs.size(), nullptr, sig.p, g.n, nullptr), "count_shortest_paths");
        sigma_h.assign((size_t)R, std::vector<unsigned long long>((size_t)g.n));
        for (int s = end - R; s < end; ++s)
            cudaMemcpy(sigma_h[(size_t)((s - start) % R)].data(), sig.p + (size_t)(s - start) * g.n,
                       sizeof(uint64_t) * g.n, cudaMemcpyDeviceToHost);
    }
    std::printf("Time for shuffle-based shortest-path counting: %.9f s\n", t.stop());
}

// Brandes over all sources of [start, end); the float dependency rows of the
// last R sources are returned (the reference keeps bc on the device only).
inline void betweenness_centrality_setup(const device_graph &g, int start, int end,
                                         std::vector<std::vector<float> > &delta_h)
{
    gu_shim::timer t;
    delta_h.clear();
    if (end > start) {
        const int R = gu_shim::rows_for(start, end);
        std::vector<int32_t> hs = gu_shim::iota_sources(start, end);
        gu_shim::dbuf<int32_t> src(hs.size());
        cudaMemcpy(src.p, hs.data(), sizeof(int32_t) * hs.size(), cudaMemcpyHostToDevice);
        gu_shim::dbuf<double> bc((size_t)g.n), delta(hs.size() * (size_t)g.n);
        gu_shim::check(gu_bc(g.handle, src.p, (int32_t)hs.size(), 0, bc.p, delta.p, g.n, nullptr), "betweenness_centrality");
        delta_h.assign((size_t)R, std::vector<float>((size_t)g.n));
        std::vector<double> row((size_t)g.n);
        for (int s = end - R; s < end; ++s) {
            cudaMemcpy(row.data(), delta.p + (size_t)(s - start) * g.n, sizeof(double) * g.n, cudaMemcpyDeviceToHost);
            std::vector<float> &dst = delta_h[(size_t)((s - start) % R)];
            for (int v = 0; v < g.n; ++v) dst[(size_t)v] = (float)row[(size_t)v];
        }
    }
    std::printf("Time for shuffle-based BC: %.9f s\n", t.stop());
}

// LBS over device arrays; *edges (device) receives the total.
inline void extract_edges_block(int vertex_frontier_size, int *edge_counts, int *scanned_edges, int *result, int *edges)
{
    int64_t total = 0;
    gu_shim::check(gu_lbs(edge_counts, vertex_frontier_size, scanned_edges, result, INT32_MAX, edges, &total, nullptr),
                   "extract_edges_block");
}

inline void extract_edges_warp(int vertex_frontier_size, int *edge_counts, int *scanned_edges, int *result, int *edges)
{
    extract_edges_block(vertex_frontier_size, edge_counts, scanned_edges, result, edges);
}

// ---- graph files (parse.h:37-40) ----------------------------------------------
namespace gu_shim {
// host_graph from a file through the library's readers (same CSR as the
// reference parser), with F (each entry's source) filled as the reference's is.
inline host_graph read_graph(const char *file, const char *format)
{
    gu_hgraph h = nullptr;
    check(gu_hgraph_parse(file, format, &h), "parse");
    const int32_t *R = nullptr, *C = nullptr;
    int32_t n = 0;
    int64_t m = 0;
    int directed = 0;
    gu_status st = gu_hgraph_arrays(h, &R, &C, &n, &m, &directed);
    host_graph g;
    if (st == GU_OK) {
        g.n = n;
        g.m = (int)m;
        g.directed = directed != 0;
        g.R.assign(R, R + n + 1);
        g.C.assign(C, C + m);
        g.F.resize((size_t)m);
        for (int v = 0; v < n; ++v)
            for (int e = R[v]; e < R[v + 1]; ++e) g.F[(size_t)e] = v;
    }
    gu_hgraph_destroy(h);
    check(st, "parse");
    return g;
}
}  // namespace gu_shim

inline host_graph parse_metis(char *file) { return gu_shim::read_graph(file, "dimacs"); }
inline host_graph parse_snap(char *file, bool header) { return gu_shim::read_graph(file, header ? "edgelist_h" : "edgelist"); }
inline host_graph parse_market(char *file) { return gu_shim::read_graph(file, "market"); }
inline host_graph parse(const program_options &op) { return gu_shim::read_graph(op.infile, op.format ? op.format : ""); }

// ---- DAG reachability (dag_reachability.h:15) ----------------------------------
// The reachable set of every vertex (itself excluded), from the batched search's
// distance rows.  Needs a directed graph, as the reference's does.
inline std::vector<std::set<int> > get_reachability_dag(host_graph &g)
{
    if (!g.directed) throw std::runtime_error("get_reachability_dag: the graph must be directed");
    device_graph dg(g);
    std::vector<std::set<int> > reach((size_t)g.n);
    const int chunk = 256;
    gu_shim::dbuf<int32_t> src((size_t)chunk), dist((size_t)chunk * (size_t)g.n);
    std::vector<int32_t> hs((size_t)chunk), row((size_t)chunk * (size_t)g.n);
    for (int c0 = 0; c0 < g.n; c0 += chunk) {
        const int k = std::min(chunk, g.n - c0);
        for (int i = 0; i < k; ++i) hs[(size_t)i] = c0 + i;
        cudaMemcpy(src.p, hs.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice);
        gu_shim::check(gu_bfs(dg.handle, GU_BFS_AUTO, src.p, k, dist.p, g.n, nullptr), "get_reachability_dag");
        cudaMemcpy(row.data(), dist.p, sizeof(int32_t) * (size_t)k * g.n, cudaMemcpyDeviceToHost);
        for (int i = 0; i < k; ++i)
            for (int v = 0; v < g.n; ++v)
                if (v != c0 + i && row[(size_t)i * g.n + v] != GU_DIST_UNREACHABLE) reach[(size_t)(c0 + i)].insert(v);
    }
    return reach;
}
