/*
 * gu.h -- C ABI of graph-utils for GB300 (sm_103a).
 *
 * Drop-in boundary for the multi-source search hot path of graph-utils.  Plain
 * pointers and sizes only.  Every call returns a gu_status (the reference calls
 * exit() on any error, util_device.cuh:10-22); gu_last_error() gives the
 * message of the last failing call on the calling thread.
 *
 * Pointer conventions: arguments named *_dev are device pointers on the graph's
 * device and the call is ordered on `stream` (a cudaStream_t, NULL = legacy
 * default stream); the call synchronises `stream` before returning so that a
 * device-side failure is reported as a status.  Arguments named *_host are host
 * pointers (pinned memory gives full copy bandwidth); the call copies them
 * through the device inside the call, as the reference's *_setup functions do.
 *
 * Graph handles are thread-safe: concurrent calls on one handle are serialised.
 */
#ifndef GU_H
#define GU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gu_status {
    GU_OK = 0,
    GU_ERR_INVALID_ARGUMENT = 1,
    GU_ERR_CUDA = 2,
    GU_ERR_OUT_OF_MEMORY = 3,
    GU_ERR_CAPACITY = 4,
    GU_ERR_OVERFLOW = 5,
    GU_ERR_TIMEOUT = 6,
    GU_ERR_UNSUPPORTED = 7,
    GU_ERR_INTERNAL = 8,
    GU_ERR_PENDING = 9 /* gu_server_wait: the request has not finished within the timeout */
} gu_status;

/* Breadth-first-search variants.  Each names the neighbour-gathering strategy
 * of one reference kernel; all variants return identical distances.
 *   LINEAR    thread per frontier vertex   (multi_search/linear_with_atomics.cu:42-159)
 *   EDGE      sweep of all CSR entries     (multi_search/edge_parallel.cu:37-92)
 *   WARP      warp strip-mining with race-and-resolve election
 *                                          (multi_search/warp_based.cu:47-190)
 *   CTA_WARP  CTA gathers degree > 2048, warps the rest (multi_search/CTA_warp.cu:42-289)
 *   SCAN      block-scan ranked gather     (multi_search/scan_based.cu:43-194)
 *   SHUFFLE   warp per vertex, dynamic queue (multi_search/shuffle_based.cuh:81-286)
 *   BOTTOM_UP frontier bitmap pull (no reference counterpart)
 *   AUTO      engine by graph shape -- per-source BFS with shared-memory queues
 *             for out-degree <= 16 (meshes; falls back on frontier overflow), the
 *             PLAIN form for n <= 4096, else the batched engine with per-level
 *             direction and gather choice
 *   PLAIN     one CTA per source, int32 distance row as the visited set -- the
 *             reference's own structure, kept as the one-launch-per-request baseline.
 * All but PLAIN run 64 sources per bitmap word in one persistent launch. */
typedef enum gu_bfs_variant {
    GU_BFS_AUTO = 0,
    GU_BFS_LINEAR = 1,
    GU_BFS_EDGE = 2,
    GU_BFS_WARP = 3,
    GU_BFS_CTA_WARP = 4,
    GU_BFS_SCAN = 5,
    GU_BFS_SHUFFLE = 6,
    GU_BFS_BOTTOM_UP = 7,
    GU_BFS_PLAIN = 8
} gu_bfs_variant;

#define GU_DIST_UNREACHABLE 2147483647 /* INT_MAX, as the reference (warp_based.cu:73) */

typedef struct gu_graph_s *gu_graph;   /* device-resident graph */
typedef struct gu_hgraph_s *gu_hgraph; /* host CSR graph (generators) */

/* ---- library ------------------------------------------------------------ */
int gu_version(void);
const char *gu_last_error(void);
const char *gu_status_string(gu_status s);

/* Select a device: `requested` >= 0 selects it; -1 picks the device with the
 * highest memory bandwidth.  Replaces choose_device (util_device.cu:23-76). */
gu_status gu_choose_device(int requested, int *chosen);

/* Stream-ordered interval timer on `stream`, in seconds; replaces
 * start_clock/end_clock (util_device.cu:4-21). */
typedef struct gu_timer_s *gu_timer;
gu_status gu_timer_start(void *stream, gu_timer *out);
gu_status gu_timer_stop(gu_timer t, void *stream, double *seconds); /* also frees t */

/* Bound of every device-side wait (the grid barriers between the levels of the
 * persistent kernels), in seconds, for launches made after the call; 4 s by
 * default, accepted range [1e-4, 3600].  A wait that runs out ends the launch:
 * the call returns GU_ERR_TIMEOUT and its handle stays usable.  The reference
 * has no bounded waits (its kernels end levels with __syncthreads and kernel
 * boundaries), so no counterpart. */
gu_status gu_set_wait_limit(double seconds);
gu_status gu_get_wait_limit(double *seconds);

/* Diagnostic of the grid barrier every persistent kernel is built on: a
 * cooperative launch of one 128-thread CTA per SM whose CTAs meet at two grid
 * barriers bounded by `limit_seconds`.  absent_block = -1: every CTA arrives and
 * the call returns GU_OK.  absent_block = b: CTA b leaves without arriving, the
 * others' wait runs out after limit_seconds and the call returns GU_ERR_TIMEOUT
 * (no fault, no trap: the device stays usable).  *elapsed_seconds = the launch's
 * CUDA-event time.  No reference counterpart. */
gu_status gu_check_grid_barrier(int absent_block, double limit_seconds, void *stream, double *elapsed_seconds);

/* Test hook: after `after` more successful device or pinned-host allocations by
 * this library, the next `count` fail as if the GPU were out of memory (count 0
 * switches it off).  Lets tests drive every call's GU_ERR_OUT_OF_MEMORY path on
 * the host side.  No reference counterpart (the reference exits on failure,
 * util_device.cuh:10-22). */
gu_status gu_debug_fail_allocations(int64_t after, int64_t count);

/* Board power during a run (power_measurer::start_power_sample /
 * end_power_sample, util_device.cu:78-130): a background thread reads the
 * device's power draw every period_ms until gu_power_stop, which returns the
 * mean in watts and the sample count and frees the sampler.  NVML is loaded at
 * run time (libnvidia-ml.so.1, or $GU_NVML_LIBRARY); without it the start
 * returns GU_ERR_UNSUPPORTED.  Reads only: no GPU setting is changed. */
typedef struct gu_power_s *gu_power;
gu_status gu_power_start(int device, int period_ms, gu_power *out);
gu_status gu_power_stop(gu_power p, double *avg_watts, int64_t *samples);

/* ---- host graphs (generators; no reference counterpart) ------------------ */
/* R-MAT: 2^scale vertices, edge_factor*2^scale edge draws, quadrant
 * probabilities a,b,c (d = 1-a-b-c); symmetrised, duplicates and self-loops
 * removed; permute != 0 relabels vertices by a seeded random permutation. */
gu_status gu_hgraph_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                         int permute, gu_hgraph *out);
/* Erdos-Renyi G(n, m): m distinct undirected edges. */
gu_status gu_hgraph_er(int32_t n, int64_t m, uint64_t seed, gu_hgraph *out);
/* rows x cols 4-neighbour grid, each edge deleted with probability p_delete. */
gu_status gu_hgraph_grid(int32_t rows, int32_t cols, double p_delete, uint64_t seed, gu_hgraph *out);
/* Random DAG: m edge draws u -> v with u before v in a random topological order. */
gu_status gu_hgraph_dag(int32_t n, int64_t m, uint64_t seed, gu_hgraph *out);
/* CSR from an edge list (u[i], v[i]); symmetric != 0 adds both directions. */
gu_status gu_hgraph_from_edges(int32_t n, const int32_t *u, const int32_t *v, int64_t count, int symmetric,
                               gu_hgraph *out);
/* A host graph holding a copy of the given CSR as it is (validated, not rebuilt). */
gu_status gu_hgraph_from_csr(const int32_t *R, const int32_t *C, int32_t n, int64_t m, int directed, gu_hgraph *out);
gu_status gu_hgraph_arrays(gu_hgraph h, const int32_t **R, const int32_t **C, int32_t *n, int64_t *m,
                           int *directed);
gu_status gu_hgraph_destroy(gu_hgraph h);
/* k distinct sources drawn uniformly without replacement from [0, n). */
gu_status gu_sources(int32_t n, int32_t k, uint64_t seed, int32_t *out_host);

/* ---- graph files ------------------------------------------------------------ */
/* Reads a graph file.  format: "dimacs" (or "metis"), "edgelist", "edgelist_h",
 * "market" -- the reference's formats, giving the same CSR as its parser
 * (parse(), parse.cpp:88-113; parse_metis 115-208, parse_market 210-346,
 * parse_snap 349-441) -- or "csrbin", the binary CSR cache written by
 * gu_hgraph_write_csr.  Malformed files give GU_ERR_INVALID_ARGUMENT (the
 * reference exits or reads out of bounds). */
gu_status gu_hgraph_parse(const char *path, const char *format, gu_hgraph *out);
/* Binary CSR cache: magic "GUCSR1", n, m, directed, R, C (little-endian). */
gu_status gu_hgraph_write_csr(gu_hgraph h, const char *path);
/* host_graph::write_edgelist_to_file (parse.cpp:443-465): optional "n m" line,
 * then "source target" per CSR entry. */
gu_status gu_hgraph_write_edgelist(gu_hgraph h, const char *path, int header);
/* host_graph::count_degree_zero_vertices (parse.cpp:467-478). */
gu_status gu_hgraph_count_degree_zero(gu_hgraph h, uint64_t *count);

/* ---- device graphs ------------------------------------------------------- */
/* Copies the CSR (R: n+1 offsets, C: m neighbours, host pointers) to the
 * current device.  Replaces device_graph::device_graph(const host_graph&)
 * (device_graph.h:11, device_graph.cpp:3-14). */
gu_status gu_graph_create(const int32_t *R_host, const int32_t *C_host, int32_t n, int64_t m, int directed,
                          void *stream, gu_graph *out);
gu_status gu_graph_destroy(gu_graph g);
gu_status gu_graph_info(gu_graph g, int32_t *n, int64_t *m, int *directed, size_t *device_bytes);
/* Device pointers of the resident CSR (R, C) and the in-edge CSR (RT, CT). */
gu_status gu_graph_arrays(gu_graph g, const int32_t **R_dev, const int32_t **C_dev, const int32_t **RT_dev,
                          const int32_t **CT_dev);

/* Duration of the last search kernel launched on g (CUDA events on the call's
 * stream, kernel only) and, for the batched engine, the number of top-down and
 * bottom-up levels it ran and the deepest level reached.  Replaces the
 * per-call timing prints of the reference's *_setup functions
 * (e.g. shuffle_based.cu:42-44). */
gu_status gu_graph_last_launch(gu_graph g, double *kernel_seconds, int *td_levels, int *bu_levels, int *max_level);

/* Kernel durations of the graph's last launches (up to 64, oldest first; CUDA
 * events on each call's stream around its main kernel): a caller timing many
 * calls reads them once afterwards instead of querying after every call. */
gu_status gu_graph_launch_times(gu_graph g, int max_entries, double *kernel_seconds, int *count);

/* Profiling hook: the per-phase timeline of the last batched search or BC /
 * sigma pass on g (up to max_entries phases).  Entry i: batch, level j of the
 * phase, kind (0 top-down, 1 bottom-up, 2 distance write-out, 4 batch
 * initialised; inside a bottom-up phase 5 marks the end of the finalise step, 6
 * the end of the light class's scan as seen by warp 0 of each CTA, 7 the end of
 * the scans before the rare sources' top-down expansion; BC and sigma passes: 8
 * forward level, 9 backward level, 10 split vertices' sums of a backward level,
 * 11 bc accumulation and per-source rows, 12 a forward level's bitmap cleared),
 * vertices and out-edges of the frontier it expanded (batched search only; 0 for
 * BC), and the time the slowest CTA finished it, in ms from the end of entry 0.
 * No reference counterpart (the reference times whole calls only). */
gu_status gu_graph_level_profile(gu_graph g, int max_entries, int32_t *batch, int32_t *level, int32_t *kind,
                                 int64_t *frontier_vertices, int64_t *frontier_edges, double *t_ms, int *count);

/* Idle time of the last batched search per timeline entry (the entries of
 * gu_graph_level_profile, same order): the sum over the launch's CTAs of the
 * time each waited at the grid barriers of that phase, in CTA-milliseconds;
 * *nblocks = the launch's CTAs.  Batched search only.  No reference counterpart. */
gu_status gu_graph_level_idle(gu_graph g, int max_entries, double *idle_cta_ms, int *nblocks, int *count);

/* ---- autotuning AUTO --------------------------------------------------------- */
/* AUTO's built-in choice goes by graph shape (out-degree, size) and fixed
 * direction thresholds.  gu_graph_autotune measures instead: it runs the
 * candidate engines and settings on a sample of sources (distance rows into a
 * scratch buffer it allocates, k x n int32: keep the sample modest), times each
 * by its kernel, and makes the fastest the graph's AUTO choice for later gu_bfs
 * / gu_bfs_host calls (the server and the counting calls keep the built-in
 * choice).  Candidates: the per-source engine (out-degree <= 16), the
 * one-CTA-per-source form (n <= 65536), and the batched engine over a grid of
 * direction thresholds (alpha: top-down -> bottom-up when the frontier's
 * out-edges exceed m / alpha; beta: back when the frontier holds fewer than
 * n / beta vertices), source words per batch and the persistent grid's CTAs
 * per SM (the CTA itself is 512 threads: its register budget fixes that); slow candidates are cut after
 * one run.  trials (optional, room for max_trials) receives every measured
 * candidate in order; best receives the choice.  Distances do not depend on the
 * choice.  No reference counterpart (its examples pick the kernel by hand). */
typedef enum gu_engine {
    GU_ENGINE_BATCHED = 0,    /* bit-matrix engine, 64 x words sources per batch */
    GU_ENGINE_PER_SOURCE = 1, /* one CTA per source, shared-memory level queues */
    GU_ENGINE_ONE_CTA = 2     /* PLAIN: one CTA per source, distance row as visited set */
} gu_engine;

typedef struct gu_tuning {
    int32_t engine;     /* gu_engine */
    float alpha, beta;  /* batched engine's direction thresholds */
    int32_t words;      /* batched engine: 64-source words per batch (1, 2 or 4) */
    int32_t ctas_per_sm; /* batched engine: CTAs per SM of its persistent grid (0: as many as fit, or 1, 2) */
    float rare_frac;    /* batched engine: bottom-up levels expand top-down the sources fewer than this
                           fraction of the CTAs found in the previous level (0 .. 1; 0: none) */
    double seconds;     /* measured kernel time on the sample (autotune output) */
} gu_tuning;

gu_status gu_graph_autotune(gu_graph g, const int32_t *sources_dev, int32_t k, gu_tuning *best, gu_tuning *trials,
                            int max_trials, int *ntrials);
/* Sets the graph's AUTO choice explicitly (t = NULL: back to the built-in choice). */
gu_status gu_graph_set_tuning(gu_graph g, const gu_tuning *t);

/* ---- multi-source BFS ------------------------------------------------------ */
/* Row i of dist (row stride ld >= n elements) receives the distances from
 * sources[i]; GU_DIST_UNREACHABLE where unreachable.  Replaces
 * multi_search_{linear_atomics,edge_parallel,warp_based,CTA_warp_based,
 * scan_based,shuffle_based}_setup (linear_with_atomics.cuh:14,
 * edge_parallel.cuh:13, warp_based.cuh:15, CTA_warp.cuh:15, scan_based.cuh:15,
 * shuffle_based.cuh:16), which return the rows of the last #SM sources only;
 * this call returns every row. */
gu_status gu_bfs(gu_graph g, int variant, const int32_t *sources_dev, int32_t k, int32_t *dist_dev, int64_t ld,
                 void *stream);
gu_status gu_bfs_host(gu_graph g, int variant, const int32_t *sources_host, int32_t k, int32_t *dist_host,
                      int64_t ld, void *stream);

/* ---- shortest-path counts and betweenness ------------------------------------ */
/* Row i of sigma_dev (uint64, stride ld) = number of shortest paths from
 * sources[i] to every vertex (wrapping uint64 arithmetic, 0 where unreachable,
 * 1 at the source); dist_dev (nullable, int32) receives the distances.  Replaces
 * count_shortest_paths_setup (count_shortest_paths/count_shortest_paths.cuh:13),
 * whose kernel the reference only designed (shuffle_based.cu:113-151). */
gu_status gu_sigma(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t *dist_dev, uint64_t *sigma_dev,
                   int64_t ld, void *stream);

/* Brandes betweenness from the given sources: bc_dev[v] = sum over sources s of
 * delta_s(v), v != s (unnormalised, ordered pairs, as the reference's bc.cu:11-57
 * and shuffle_based.cu:153-542), in FP64 with a fixed summation order
 * (deterministic).  `batch` = sources per pass (64, 128, 256, 512 or 1024; 0 =
 * default 256).  delta_dev (nullable, k x ld doubles) receives the per-source
 * dependencies, 0 at the source and where unreachable.  Replaces
 * betweenness_centrality_setup (betweenness_centrality.cuh:14), which returns
 * float delta rows. */
gu_status gu_bc(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t batch, double *bc_dev, double *delta_dev,
                int64_t ld, void *stream);

/* Largest finite BFS distance from the given sources (0 if none).  Replaces
 * diameter_sampling_setup (diameter_sampling/diameter_sampling.cuh:13). */
gu_status gu_diameter(gu_graph g, const int32_t *sources_dev, int32_t k, int32_t *diameter, void *stream);

/* counts_dev[i] (int64) = number of vertices reachable from sources_dev[i],
 * the source included (reachability.cu:11-33 counts reachable ordered pairs,
 * self pairs included), without materialising distance rows.  The counting
 * form of transitive_closure_setup (transitive_closure/transitive_closure.cuh:13),
 * whose rows gu_bfs returns. */
gu_status gu_reach(gu_graph g, const int32_t *sources_dev, int32_t k, int64_t *counts_dev, void *stream);

/* All-vertex reachability of a DAG: counts_dev[v] (int64, n) = size of the set
 * of vertices reachable from v, v itself excluded, and *total_pairs their sum --
 * the sets get_reachability_dag (graph-utils/dag_reachability.cpp:36-65)
 * returns, as sizes (gu_bfs rows give the sets).  The graph must be directed
 * (GU_ERR_INVALID_ARGUMENT otherwise, as the reference exits); like the
 * reference it assumes no cycles. */
gu_status gu_dag_reach(gu_graph g, int64_t *counts_dev, int64_t *total_pairs, void *stream);

/* Many searches in one launch: BFS rows and/or reachable counts for requests on
 * any number of graphs (all on the current device), run by one persistent grid
 * whose CTA groups drain a device work queue of (graph, block of up to 256
 * sources) items -- small graphs and large ones side by side, no launch per
 * request.  Per item: dist_dev (k x ld int32 rows, ld >= the graph's n, or NULL)
 * and/or reach_dev (k int64 counts, the source included, or NULL); at least one.
 * Results equal gu_bfs / gu_reach on each graph alone.  A source out of range
 * gives GU_ERR_INVALID_ARGUMENT (the outputs are then unspecified).  The
 * reference runs one graph per setup call with a grid stride over its sources
 * (multi_search/shuffle_based.cuh:104); this is the cross-graph form. */
typedef struct gu_search_item {
    gu_graph graph;
    const int32_t *sources_dev;
    int32_t k;
    int32_t *dist_dev;
    int64_t ld;
    int64_t *reach_dev;
} gu_search_item;
gu_status gu_bfs_many(const gu_search_item *items, int32_t count, void *stream);

/* ---- load-balanced search and race-and-resolve ------------------------------- */
/* Load-balanced search over N work counts (device pointers, counts >= 0):
 * scanned_dev[i] = exclusive prefix sum of counts (int32), total = sum, and
 * result_dev[j] for every work slot j < total = the item that owns it
 * (upper_bound(scanned, j) - 1).  The total is returned in *total_host and/or
 * *total_dev (either may be NULL).  GU_ERR_OVERFLOW if the total exceeds
 * INT32_MAX, GU_ERR_CAPACITY if it exceeds result_capacity, GU_ERR_INVALID_ARGUMENT
 * for a negative count: result_dev and *total_dev are not written then (the
 * checks run on the device, so scanned_dev may hold the prefix sums).  Replaces extract_edges_{warp,block} / load_balance_search_{warp,
 * block} (load_balanced_search.cuh:10-13, load_balanced_search.cu:63-202). */
gu_status gu_lbs(const int32_t *counts_dev, int32_t N, int32_t *scanned_dev, int32_t *result_dev,
                 int64_t result_capacity, int32_t *total_dev, int64_t *total_host, void *stream);

/* Device time of the last gu_lbs call on the current device, in ms (CUDA events
 * around its kernels on the call's stream; 0 before the first call).  A
 * profiling hook with no reference counterpart. */
gu_status gu_lbs_last_ms(double *ms);

/* Warp leader election over nwarps groups of 32 predicates: winners_dev[32w+l] =
 * the highest lane of group w whose predicate is non-zero, or l itself if none
 * is.  Exposes race_and_resolve_warp (race_and_resolve.cuh:13-25), the device
 * primitive the WARP and CTA_WARP gathers use. */
gu_status gu_race_and_resolve(const int32_t *predicates_dev, int32_t nwarps, int32_t *winners_dev, void *stream);

/* ---- serving ---------------------------------------------------------------------- */
/* A query server with continuous batching over device-resident graphs (no
 * reference counterpart: the reference runs one synchronous call at a time).
 * Requests from any host thread join a FIFO; a worker merges the oldest
 * request with later ones for the same graph and kind into a batch of at most
 * max_batch_sources sources, admits it when one of `slots` streams is free and
 * its device footprint fits hbm_budget_bytes next to the running batches, and
 * runs it on 1/slots of the GPU, so batches overlap.  Results:
 *   GU_QUERY_BFS    out_host = k x n int32 distance rows (as gu_bfs)
 *   GU_QUERY_BC     out_host = n doubles, betweenness from the k sources (as gu_bc)
 *   GU_QUERY_REACH  out_host = k int64, vertices reachable from each source
 *                   (itself included; the reference's transitive closure rows
 *                   reduced to counts, transitive_closure.cu:4-37)
 * BFS rows and reach counts equal a lone call bit for bit; BC is within 1e-12
 * relative of a lone call.  The graph must outlive its requests. */
typedef enum gu_query { GU_QUERY_BFS = 0, GU_QUERY_BC = 1, GU_QUERY_REACH = 2 } gu_query;
typedef struct gu_server_s *gu_server;
gu_status gu_server_create(size_t hbm_budget_bytes, int slots, int max_batch_sources, gu_server *out);
gu_status gu_server_destroy(gu_server s); /* finishes queued work first */
/* sources_host is copied; out_host must stay valid until the request is waited for. */
gu_status gu_server_submit(gu_server s, gu_graph g, int query, const int32_t *sources_host, int32_t k, void *out_host,
                           int64_t *request_id);
/* Blocks until the request finishes (timeout_s < 0: no limit; GU_ERR_PENDING on
 * timeout) and returns its status; the latency from submit to completion goes
 * to *latency_s.  A finished request can be waited for once. */
gu_status gu_server_wait(gu_server s, int64_t request_id, double timeout_s, double *latency_s);
/* Completed requests, batches launched, latency percentiles (s) and the mean
 * number of requests per batch since creation. */
gu_status gu_server_stats(gu_server s, int64_t *completed, int64_t *batches, double *p50_s, double *p99_s,
                          double *mean_requests_per_batch);

/* Multi-source BFS that allocates no device memory.  No counterpart in the
 * reference: it exists for callers that may not call cudaMalloc while they
 * search -- code living in a process whose allocator owns every byte of the GPU
 * (a database or inference server, a framework's caching pool), services whose
 * memory budget is fixed at start-up, and paths that cannot afford the implicit
 * device synchronisation of cudaMalloc/cudaFree.
 *
 * The caller passes its own device CSR (R_dev: n+1 offsets, C_dev: m neighbours,
 * directed or undirected), device sources and device rows, as for gu_bfs; the
 * rows are identical to gu_bfs's.  Scratch is a fixed 6 MiB array compiled into
 * the library, which every device that loads the library holds until the process
 * exits; it limits n to 32768 vertices (larger graphs: GU_ERR_CAPACITY, nothing
 * launched).  The search runs top-down levels only.  Malformed CSR arrays and
 * out-of-range sources are rejected with GU_ERR_INVALID_ARGUMENT before the
 * search.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call before
 * any stream capture.  All calls on a device share the one array and it keeps
 * the previous call's contents (each call clears what must start at zero):
 * calls whose work overlaps on the GPU -- on different streams or from several
 * host threads -- race and must be serialised by the caller.  Synchronises
 * `stream` before returning. */
gu_status gu_bfs_noalloc(const int32_t *R_dev, const int32_t *C_dev, int32_t n, int64_t m,
                         const int32_t *sources_dev, int32_t k, int32_t *dist_dev, int64_t ld, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GU_H */
