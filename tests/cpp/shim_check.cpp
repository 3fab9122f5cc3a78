// shim_check.cpp -- drives the C++ drop-in (include/graph_utils.hpp) the way the
// reference's example drivers drive their *_setup functions, and verifies the
// results with the oracle using the reference checkers' conventions
// (examples/multi_search/multi_search_test.cu:40-127: rows of the last #SM
// sources, source s in row (s - start) % rows).  Test infrastructure.
//
//   shim_check <scale> <edge_factor> <start> <end>
#define GU_DEFINE_HOST_TYPES
#include "graph_utils.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <unistd.h>

#include "gu_oracle.h"

static int failures = 0;
static void report(const char *what, bool ok)
{
    std::printf("%s: %s\n", what, ok ? "Test passed." : "Test FAILED.");
    if (!ok) ++failures;
}

// source held by each returned row (reference convention)
static std::vector<int> row_sources(int start, int end, int rows)
{
    std::vector<int> s((size_t)rows);
    for (int v = end - rows; v < end; ++v) s[(size_t)((v - start) % rows)] = v;
    return s;
}

int main(int argc, char **argv)
{
    if (argc != 5) {
        std::fprintf(stderr, "usage: shim_check scale edge_factor start end\n");
        return 2;
    }
    const int scale = std::atoi(argv[1]), ef = std::atoi(argv[2]);
    const int start = std::atoi(argv[3]);
    int end = std::atoi(argv[4]);

    gu_hgraph hgh;
    if (gu_hgraph_rmat(scale, ef, 0.57, 0.19, 0.19, 11, 1, &hgh) != GU_OK) return 3;
    const int32_t *R, *C;
    int32_t n;
    int64_t m;
    int directed;
    gu_hgraph_arrays(hgh, &R, &C, &n, &m, &directed);
    host_graph h;
    h.R.assign(R, R + n + 1);
    h.C.assign(C, C + m);
    h.F.resize((size_t)m);
    for (int v = 0; v < n; ++v)
        for (int e = R[v]; e < R[v + 1]; ++e) h.F[(size_t)e] = v;
    h.n = n;
    h.m = (int)m;
    h.directed = false;
    gu_hgraph_destroy(hgh);
    if (end > n) end = n;

    int dev = -1;
    if (gu_choose_device(-1, &dev) != GU_OK || dev < 0) {
        std::printf("FAIL gu_choose_device: %s\n", gu_last_error());
        return 1;
    }
    device_graph g(h);
    program_options op;

    std::vector<int> expect((size_t)n);
    auto check_rows = [&](const char *name, const std::vector<std::vector<int> > &rows) {
        const int R_ = gu_shim::rows_for(start, end);
        bool ok = (int)rows.size() == R_;
        const std::vector<int> src = row_sources(start, end, R_);
        for (int r = 0; ok && r < R_; ++r) {
            oracle_bfs(h.R.data(), h.C.data(), n, src[(size_t)r], expect.data());
            ok = rows[(size_t)r] == expect;
        }
        report(name, ok);
    };
    check_rows("Linear with atomics", multi_search_linear_atomics_setup(g, start, end));
    check_rows("Edge parallel", multi_search_edge_parallel_setup(g, start, end));
    check_rows("Warp based", multi_search_warp_based_setup(g, start, end));
    check_rows("CTA+warp", multi_search_CTA_warp_based_setup(g, start, end));
    check_rows("Scan based", multi_search_scan_based_setup(g, start, end));
    check_rows("Shuffle based", multi_search_shuffle_based_setup(g, op, start, end));
    {
        std::vector<std::vector<int> > d;
        transitive_closure_setup(g, start, end, d);
        check_rows("Transitive closure", d);
    }
    {
        std::vector<int32_t> srcs;
        for (int s = start; s < end; ++s) srcs.push_back(s);
        const int diam = diameter_sampling_setup(g, start, end);
        report("Diameter sampling", diam == oracle_diameter(h.R.data(), h.C.data(), n, srcs.data(), (int)srcs.size(), 4));
    }
    {
        std::vector<std::vector<unsigned long long> > sig;
        count_shortest_paths_setup(g, start, end, sig);
        const int R_ = gu_shim::rows_for(start, end);
        const std::vector<int> src = row_sources(start, end, R_);
        bool ok = (int)sig.size() == R_;
        std::vector<int32_t> d((size_t)n);
        std::vector<uint64_t> s((size_t)n);
        for (int r = 0; ok && r < R_; ++r) {
            oracle_sigma(h.R.data(), h.C.data(), n, src[(size_t)r], d.data(), s.data());
            for (int v = 0; ok && v < n; ++v) ok = sig[(size_t)r][(size_t)v] == s[(size_t)v];
        }
        report("Counting shortest paths", ok);
    }
    {
        std::vector<std::vector<float> > delta;
        betweenness_centrality_setup(g, start, end, delta);
        const int R_ = gu_shim::rows_for(start, end);
        const std::vector<int> src = row_sources(start, end, R_);
        bool ok = (int)delta.size() == R_;
        double max_err = 0;
        std::vector<int32_t> d((size_t)n);
        std::vector<uint64_t> s((size_t)n);
        std::vector<double> de((size_t)n);
        for (int r = 0; ok && r < R_; ++r) {
            oracle_brandes_f64(h.R.data(), h.C.data(), n, src[(size_t)r], d.data(), s.data(), de.data());
            for (int v = 0; v < n; ++v) {
                const double err = std::fabs((double)delta[(size_t)r][(size_t)v] - de[(size_t)v]);
                const double tol = 1e-6 * std::fmax(1.0, std::fabs(de[(size_t)v]));
                if (err > tol) ok = false;
                max_err = std::fmax(max_err, err);
            }
        }
        std::printf("Maximum Error: %g\n", max_err);
        report("Betweenness centrality (float delta rows)", ok);
    }
    {
        // load-balanced search over the degree array
        std::vector<int> counts((size_t)n);
        for (int v = 0; v < n; ++v) counts[(size_t)v] = h.R[(size_t)v + 1] - h.R[(size_t)v];
        gu_shim::dbuf<int> cd((size_t)n), sd((size_t)n), rd((size_t)m), td(1);
        cudaMemcpy(cd.p, counts.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        extract_edges_block(n, cd.p, sd.p, rd.p, td.p);
        int total = 0;
        cudaMemcpy(&total, td.p, sizeof(int), cudaMemcpyDeviceToHost);
        std::vector<int> scanned((size_t)n), result((size_t)m), es((size_t)n), er((size_t)m);
        cudaMemcpy(scanned.data(), sd.p, sizeof(int) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(result.data(), rd.p, sizeof(int) * m, cudaMemcpyDeviceToHost);
        int64_t et = 0;
        oracle_lbs(counts.data(), n, es.data(), er.data(), m, &et);
        report("Scan", scanned == es);
        report("Load-balanced search", total == et && result == er);
    }
    {
        // parse_snap on a graph's edge list (write_edgelist_to_file's format) gives
        // back its CSR and COO sources (a grid: every id appears, as SNAP needs)
        gu_hgraph w = nullptr;
        gu_hgraph_grid(30, 40, 0.0, 1, &w);
        const int32_t *WR, *WC;
        int32_t wn;
        int64_t wm;
        int wd;
        gu_hgraph_arrays(w, &WR, &WC, &wn, &wm, &wd);
        std::vector<int> F((size_t)wm);
        for (int v = 0; v < wn; ++v)
            for (int e = WR[v]; e < WR[v + 1]; ++e) F[(size_t)e] = v;
        char path[] = "/tmp/gu_shim_edgesXXXXXX";
        const int fd = mkstemp(path);
        if (fd >= 0) close(fd);
        gu_hgraph_write_edgelist(w, path, 0);
        host_graph p = parse_snap(path, false);
        std::remove(path);
        report("Parse (SNAP edge list)", p.n == wn && p.R == std::vector<int>(WR, WR + wn + 1) &&
                                             p.C == std::vector<int>(WC, WC + wm) && p.F == F && p.directed);
        gu_hgraph_destroy(w);
    }
    {
        // get_reachability_dag on a random DAG: set sizes against the oracle
        gu_hgraph dh = nullptr;
        gu_hgraph_dag(3000, 20000, 5, &dh);
        const int32_t *DR, *DC;
        int32_t dn;
        int64_t dm;
        int dd;
        gu_hgraph_arrays(dh, &DR, &DC, &dn, &dm, &dd);
        host_graph d;
        d.R.assign(DR, DR + dn + 1);
        d.C.assign(DC, DC + dm);
        d.n = dn;
        d.m = (int)dm;
        d.directed = true;
        std::vector<int64_t> cnt((size_t)dn);
        oracle_dag_reach_counts(DR, DC, dn, cnt.data());
        gu_hgraph_destroy(dh);
        const std::vector<std::set<int> > reach = get_reachability_dag(d);
        bool ok = (int)reach.size() == dn;
        for (int v = 0; ok && v < dn; ++v) ok = (int64_t)reach[(size_t)v].size() == cnt[(size_t)v];
        report("DAG reachability", ok);
    }
    std::printf("%s\n", failures ? "FAILED" : "ALL PASSED");
    return failures ? 1 : 0;
}
