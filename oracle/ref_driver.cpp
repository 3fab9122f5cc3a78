// ref_driver.cpp -- command-line driver around the reference graph-utils CPU
// checkers, compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/ref_oracle.  Test infrastructure only: it pins the C restatement
// in oracle/gu_oracle.c and generates the golden vectors in tests/golden/.
//
// The reference functions called here (renamed at compile time with -D so that
// the identically named checkers of different examples can be linked together):
//   ms_sequential  examples/multi_search/multi_search_test.cu:17-38
//   bc_sequential  examples/betweenness_centrality/bc.cu:11-57
//   sp_sequential  examples/counting_shortest_paths/shortest_paths.cu:11-39
//   ds_sequential  examples/diameter_sampling/diameter_sampling_test.cu:9-38
//   tc_sequential  examples/transitive_closure/reachability.cu:11-33
//   load_balance_search          examples/load_balanced_search/lbs.cu:18-31
//   get_reachability_dag         graph-utils/dag_reachability.cpp:36-65
//   parse / parse_metis / parse_snap / parse_market   parse.cpp:88-441
//
// Binary files are little-endian raw arrays; a CSR prefix P names P.R (int32
// n+1), P.C (int32 m) and P.meta (text: "n m directed").
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "parse.h"
#include "util.h"

void ms_sequential(host_graph &g, int source, std::vector<int> &expected);
void bc_sequential(host_graph &g, int source, std::vector<int> &expected, std::vector<float> &delta);
void sp_sequential(host_graph &g, int source, std::vector<int> &expected,
                   std::vector<unsigned long long> &paths);
void ds_sequential(host_graph &g, int source, std::vector<int> &expected, int &max);
void tc_sequential(host_graph &g, int source, std::vector<int> &expected);
void load_balance_search(int num_edges, const std::vector<int> &scanned_edges, std::vector<int> &result);
std::vector<std::set<int> > get_reachability_dag(host_graph &g);

template <class T>
static std::vector<T> read_vec(const std::string &path)
{
    std::vector<T> v;
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    v.resize(bytes / sizeof(T));
    if (!v.empty() && fread(v.data(), sizeof(T), v.size(), f) != v.size()) { fprintf(stderr, "short read\n"); exit(2); }
    fclose(f);
    return v;
}

template <class T>
static void write_vec(const std::string &path, const std::vector<T> &v)
{
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
    fclose(f);
}

static host_graph read_csr(const std::string &prefix)
{
    host_graph g;
    g.R = read_vec<int>(prefix + ".R");
    g.C = read_vec<int>(prefix + ".C");
    FILE *f = fopen((prefix + ".meta").c_str(), "r");
    if (!f) { fprintf(stderr, "cannot open meta\n"); exit(2); }
    int d = 0;
    if (fscanf(f, "%d %d %d", &g.n, &g.m, &d) != 3) { fprintf(stderr, "bad meta\n"); exit(2); }
    fclose(f);
    g.directed = d != 0;
    g.F.resize(g.m);
    for (int v = 0; v < g.n; ++v)
        for (int k = g.R[v]; k < g.R[v + 1]; ++k) g.F[k] = v;
    return g;
}

static void write_csr(const std::string &prefix, const host_graph &g)
{
    write_vec(prefix + ".R", g.R);
    write_vec(prefix + ".C", g.C);
    write_vec(prefix + ".F", g.F);
    FILE *f = fopen((prefix + ".meta").c_str(), "w");
    fprintf(f, "%d %d %d\n", g.n, g.m, g.directed ? 1 : 0);
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr,
                "usage: ref_oracle parse <file> <format> <out_prefix>\n"
                "       ref_oracle run <csr_prefix> <sources.i32> <out_prefix>\n"
                "       ref_oracle lbs <counts.i32> <out_prefix>\n"
                "       ref_oracle dag <csr_prefix> <out_prefix>\n"
                "       ref_oracle time_bfs <csr_prefix> <sources.i32>\n");
        return 2;
    }
    std::string mode = argv[1];
    if (mode == "parse" && argc == 5) {
        program_options op;
        op.infile = argv[2];
        op.format = argv[3];
        host_graph g = parse(op);
        write_csr(argv[4], g);
        return 0;
    }
    if (mode == "run" && argc == 5) {
        host_graph g = read_csr(argv[2]);
        std::vector<int> sources = read_vec<int>(argv[3]);
        std::string out = argv[4];
        size_t k = sources.size(), n = (size_t)g.n;
        std::vector<int> dist(k * n), dist_tc(k * n);
        std::vector<unsigned long long> sigma(k * n);
        std::vector<float> delta(k * n);
        int diam = 0;
        for (size_t i = 0; i < k; ++i) {
            std::vector<int> d, d2, d3, d4;
            std::vector<float> de;
            std::vector<unsigned long long> p;
            ms_sequential(g, sources[i], d);
            bc_sequential(g, sources[i], d2, de);
            sp_sequential(g, sources[i], d3, p);
            ds_sequential(g, sources[i], d4, diam);
            std::vector<int> d5;
            tc_sequential(g, sources[i], d5);
            for (size_t v = 0; v < n; ++v) {
                dist[i * n + v] = d[v];
                dist_tc[i * n + v] = d5[v];
                sigma[i * n + v] = p[v];
                delta[i * n + v] = de[v];
                if (d2[v] != d[v] || d3[v] != d[v]) { fprintf(stderr, "checker disagreement\n"); return 3; }
            }
        }
        write_vec(out + ".dist", dist);
        write_vec(out + ".dist_tc", dist_tc);
        write_vec(out + ".sigma", sigma);
        write_vec(out + ".delta_f32", delta);
        std::vector<int> dv(1, diam);
        write_vec(out + ".diameter", dv);
        return 0;
    }
    if (mode == "time_bfs" && argc == 4) {
        // The reference's BFS checker, one source after another on one thread;
        // prints the seconds spent inside it and the CSR entries its searches
        // scanned (the adjacency of every reached vertex).
        host_graph g = read_csr(argv[2]);
        std::vector<int> sources = read_vec<int>(argv[3]);
        double secs = 0;
        long long scanned = 0;
        for (int src : sources) {
            std::vector<int> d;
            const auto t0 = std::chrono::steady_clock::now();
            ms_sequential(g, src, d);
            secs += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            for (int v = 0; v < g.n; ++v)
                if (d[v] != INT_MAX) scanned += g.R[v + 1] - g.R[v];
        }
        printf("%.6f %lld\n", secs, scanned);
        return 0;
    }
    if (mode == "lbs" && argc == 4) {
        std::vector<int> counts = read_vec<int>(argv[2]);
        std::vector<int> scanned(counts.size());
        long long acc = 0;
        for (size_t i = 0; i < counts.size(); ++i) { scanned[i] = (int)acc; acc += counts[i]; }
        if (acc > 2147483647LL) { fprintf(stderr, "total overflows int32\n"); return 3; }
        // lbs.cu:44 computes the scan with thrust::exclusive_scan on the host;
        // the sequential sum above is the same value for int inputs in range.
        std::vector<int> result((size_t)acc);
        load_balance_search((int)acc, scanned, result);
        write_vec(std::string(argv[3]) + ".scanned", scanned);
        write_vec(std::string(argv[3]) + ".result", result);
        return 0;
    }
    if (mode == "dag" && argc == 4) {
        host_graph g = read_csr(argv[2]);
        g.directed = true;
        std::vector<std::set<int> > reach = get_reachability_dag(g);
        long long pairs = 0;
        for (auto &s : reach) pairs += (long long)s.size();
        std::vector<long long> pv(1, pairs);
        write_vec(std::string(argv[3]) + ".pairs", pv);
        return 0;
    }
    fprintf(stderr, "bad arguments\n");
    return 2;
}
