/*
 * gu_oracle.h -- CPU oracle for the multi-source search hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * graph-utils CPU checkers.  It is linked only by tests/, by the smoke() check
 * in __graft_entry__.py and by the cpu_baseline / --impl reference legs of
 * bench.py.  Nothing in the product library calls it, and the product has no
 * CPU fallback.
 *
 * Every function names the reference file:line it restates.  Parity of this
 * restatement with the reference's own compiled code is pinned by
 * tests/test_oracle_pin.py (against oracle/_ref, built from the reference
 * sources by oracle/build_ref.sh) and by the committed golden vectors in
 * tests/golden/ (generated by tests/golden/make_golden.py from the same
 * reference build).
 *
 * Graphs are CSR: R[n+1] offsets, C[m] column indices (int32).
 */
#ifndef GU_ORACLE_H
#define GU_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_INF 2147483647

/* Single-source BFS distances; restates examples/multi_search/multi_search_test.cu:17-38
 * (FIFO queue, INT_MAX for unreachable). */
void oracle_bfs(const int32_t *R, const int32_t *C, int32_t n, int32_t source, int32_t *dist);

/* BFS distances + number of shortest paths (uint64, wrapping);
 * restates examples/counting_shortest_paths/shortest_paths.cu:11-39
 * (same loop as examples/betweenness_centrality/bc.cu:28-40). */
void oracle_sigma(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                  int32_t *dist, uint64_t *sigma);

/* Brandes dependencies delta_s(v), FP32 exactly as
 * examples/betweenness_centrality/bc.cu:11-57 (push over w's adjacency while
 * popping the BFS stack; delta[source] stays 0).  Used to pin this restatement
 * bit-for-bit against the reference build. */
void oracle_brandes_f32(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                        int32_t *dist, uint64_t *sigma, float *delta);

/* Same algorithm as oracle_brandes_f32 in FP64 with (double)sigma ratios:
 * the FP64 oracle the BC kernels are held to (<= 1e-12 relative). */
void oracle_brandes_f64(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                        int32_t *dist, uint64_t *sigma, double *delta);

/* Successor-pull form of the backward sweep, as designed in the reference's GPU
 * kernel graph-utils/multi_search/shuffle_based.cu:217-354 (delta(w) = sum over
 * out-neighbours v with d(v)=d(w)+1 of sigma(w)/sigma(v)*(1+delta(v))), in FP64,
 * levels from deepest to 1.  Identical to oracle_brandes_f64 on undirected
 * graphs; on directed graphs it is the textbook Brandes value, whereas bc.cu's
 * push over out-edges of w is only meaningful for symmetric adjacency. */
void oracle_brandes_pull_f64(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                             int32_t *dist, uint64_t *sigma, double *delta);

/* BC[v] = sum over the given sources s (in array order) of delta_s(v), v != s,
 * with Neumaier-compensated summation; FP64.  pull != 0 selects the successor
 * form.  nthreads > 1 splits sources into contiguous chunks (chunk partial sums
 * are combined in chunk order, so the result is deterministic for a given
 * thread count). */
void oracle_bc(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
               int32_t k, int pull, double *bc, int nthreads);

/* Max finite distance over all given sources; restates
 * examples/diameter_sampling/diameter_sampling_test.cu:9-38 (sequential + max). */
int32_t oracle_diameter(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                        int32_t k, int nthreads);

/* Number of (source, vertex) pairs with finite distance (reachability count,
 * examples/transitive_closure/reachability.cu:11-33 restated as a count). */
int64_t oracle_reach_count(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                           int32_t k, int nthreads);

/* Multi-source BFS: row i of dist (stride ld) = distances from sources[i].
 * Sources are independent; nthreads > 1 runs them on that many host threads
 * (the per-source function is oracle_bfs, unchanged).  Returns the number of
 * CSR entries scanned (sum over sources of the out-degrees of reached vertices). */
int64_t oracle_bfs_multi(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                         int32_t k, int32_t *dist, int64_t ld, int nthreads);

/* Multi-source sigma: rows of dist / sigma as above. */
void oracle_sigma_multi(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                        int32_t k, int32_t *dist, uint64_t *sigma, int64_t ld, int nthreads);

/* Load-balanced search: scanned = exclusive prefix sum of counts
 * (thrust::exclusive_scan, examples/load_balanced_search/lbs.cu:44), total = sum,
 * result[i] for i in [0,total) = index of the item owning work slot i
 * (merge-path restatement of examples/load_balanced_search/lbs.cu:18-31).
 * Returns 0, or -1 if total exceeds result_capacity or INT32_MAX. */
int oracle_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result,
               int64_t result_capacity, int64_t *total);

/* Warp leader election: the highest lane whose predicate is true, or the
 * caller's own lane when no lane votes; restates
 * graph-utils/race_and_resolve.cuh:13-25 with graph-utils/race_and_resolve.cu:5-10. */
int32_t oracle_race_and_resolve(uint32_t vote, int32_t lane);

/* Reachable sets from all roots of a DAG as a count of (u, v) pairs with u != v
 * and v reachable from u; semantics of graph-utils/dag_reachability.cpp:36-65
 * (computed iteratively in reverse topological order, no recursion). */
int64_t oracle_dag_reach_pairs(const int32_t *R, const int32_t *C, int32_t n);
int64_t oracle_dag_reach_counts(const int32_t *R, const int32_t *C, int32_t n, int64_t *counts);

/* The benchmark's R-MAT graph (symmetrised int32 CSR, malloc'd: free with
 * oracle_free) and its k distinct sources, restated from the library's generator
 * definition so that the CPU baseline builds its input on its own. */
int oracle_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute,
                int32_t **R_out, int32_t **C_out, int64_t *m_out);
int oracle_sources(int32_t n, int32_t k, uint64_t seed, int32_t *out);
void oracle_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
