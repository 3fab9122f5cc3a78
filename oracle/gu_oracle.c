/*
 * gu_oracle.c -- CPU oracle (test infrastructure only; see gu_oracle.h).
 *
 * Plain C restatement of the reference graph-utils CPU checkers.  Build with
 * -ffp-contract=off so that the FP32 Brandes restatement rounds exactly like
 * the reference's bc.cu on every host (no fused multiply-add).
 */
#include "gu_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---- BFS: examples/multi_search/multi_search_test.cu:17-38 ---------------- */
static int64_t bfs_into(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                        int32_t *dist, int32_t *queue)
{
    int64_t scanned = 0;
    for (int32_t i = 0; i < n; ++i) dist[i] = ORACLE_INF;
    dist[source] = 0;
    int32_t head = 0, tail = 0;
    queue[tail++] = source;
    while (head < tail) {
        int32_t v = queue[head++];
        scanned += R[v + 1] - R[v];
        for (int32_t k = R[v]; k < R[v + 1]; ++k) {
            int32_t w = C[k];
            if (dist[w] == ORACLE_INF) {
                dist[w] = dist[v] + 1;
                queue[tail++] = w;
            }
        }
    }
    return scanned;
}

void oracle_bfs(const int32_t *R, const int32_t *C, int32_t n, int32_t source, int32_t *dist)
{
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    bfs_into(R, C, n, source, dist, queue);
    free(queue);
}

/* ---- sigma: examples/counting_shortest_paths/shortest_paths.cu:11-39 ------- */
/* Returns the number of vertices in BFS order (stored in order[]). */
static int32_t sigma_into(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                          int32_t *dist, uint64_t *sigma, int32_t *order)
{
    for (int32_t i = 0; i < n; ++i) { dist[i] = ORACLE_INF; sigma[i] = 0; }
    dist[source] = 0;
    sigma[source] = 1;
    int32_t head = 0, tail = 0;
    order[tail++] = source;
    while (head < tail) {
        int32_t v = order[head++];
        for (int32_t k = R[v]; k < R[v + 1]; ++k) {
            int32_t w = C[k];
            if (dist[w] == ORACLE_INF) {
                dist[w] = dist[v] + 1;
                order[tail++] = w;
            }
            if (dist[w] == dist[v] + 1) sigma[w] += sigma[v];
        }
    }
    return tail;
}

void oracle_sigma(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                  int32_t *dist, uint64_t *sigma)
{
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    sigma_into(R, C, n, source, dist, sigma, order);
    free(order);
}

/* ---- Brandes: examples/betweenness_centrality/bc.cu:11-57 ------------------ */
/* The stack S of bc.cu holds vertices in BFS pop order; popping it visits them
 * in reverse BFS order, which is order[] walked backwards. */
void oracle_brandes_f32(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                        int32_t *dist, uint64_t *sigma, float *delta)
{
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t cnt = sigma_into(R, C, n, source, dist, sigma, order);
    for (int32_t i = 0; i < n; ++i) delta[i] = 0.0f;
    for (int32_t idx = cnt - 1; idx >= 0; --idx) {
        int32_t w = order[idx];
        for (int32_t k = R[w]; k < R[w + 1]; ++k) {
            int32_t v = C[k];
            if (dist[v] == dist[w] - 1 && v != source)
                delta[v] += ((float)sigma[v] / (float)sigma[w]) * (1.0f + delta[w]);
        }
    }
    free(order);
}

static void brandes_f64_into(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                             int32_t *dist, uint64_t *sigma, double *delta, int32_t *order)
{
    int32_t cnt = sigma_into(R, C, n, source, dist, sigma, order);
    for (int32_t i = 0; i < n; ++i) delta[i] = 0.0;
    for (int32_t idx = cnt - 1; idx >= 0; --idx) {
        int32_t w = order[idx];
        for (int32_t k = R[w]; k < R[w + 1]; ++k) {
            int32_t v = C[k];
            if (dist[v] == dist[w] - 1 && v != source)
                delta[v] += ((double)sigma[v] / (double)sigma[w]) * (1.0 + delta[w]);
        }
    }
}

void oracle_brandes_f64(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                        int32_t *dist, uint64_t *sigma, double *delta)
{
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    brandes_f64_into(R, C, n, source, dist, sigma, delta, order);
    free(order);
}

/* Successor pull (graph-utils/multi_search/shuffle_based.cu:217-354 design):
 * vertices are finalised in reverse BFS order, so every successor v of w
 * (dist[v] = dist[w]+1) already holds its final delta. */
static void brandes_pull_into(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                              int32_t *dist, uint64_t *sigma, double *delta, int32_t *order)
{
    int32_t cnt = sigma_into(R, C, n, source, dist, sigma, order);
    for (int32_t i = 0; i < n; ++i) delta[i] = 0.0;
    for (int32_t idx = cnt - 1; idx >= 1; --idx) { /* idx 0 is the source: delta 0 */
        int32_t w = order[idx];
        double acc = 0.0;
        for (int32_t k = R[w]; k < R[w + 1]; ++k) {
            int32_t v = C[k];
            if (dist[v] != ORACLE_INF && dist[v] == dist[w] + 1)
                acc += ((double)sigma[w] / (double)sigma[v]) * (1.0 + delta[v]);
        }
        delta[w] = acc;
    }
}

void oracle_brandes_pull_f64(const int32_t *R, const int32_t *C, int32_t n, int32_t source,
                             int32_t *dist, uint64_t *sigma, double *delta)
{
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    brandes_pull_into(R, C, n, source, dist, sigma, delta, order);
    free(order);
}

/* ---- thread pool helper ---------------------------------------------------- */
typedef struct {
    const int32_t *R, *C;
    int32_t n;
    const int32_t *sources;
    int32_t lo, hi;
    /* outputs / mode */
    int mode; /* 0 bfs rows, 1 sigma rows, 2 bc partial, 3 diameter, 4 reach count */
    int32_t *dist;
    uint64_t *sigma;
    int64_t ld;
    int pull;
    double *bc_sum, *bc_comp; /* per-chunk Neumaier accumulators */
    int64_t scanned;
    int32_t diam;
    int64_t reach;
} chunk_t;

static void *chunk_run(void *arg)
{
    chunk_t *c = (chunk_t *)arg;
    int32_t n = c->n;
    size_t nn = (size_t)(n > 0 ? n : 1);
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * nn);
    int32_t *tmpd = NULL;
    uint64_t *tmps = NULL;
    double *delta = NULL;
    if (c->mode >= 2) {
        tmpd = (int32_t *)malloc(sizeof(int32_t) * nn);
        tmps = (uint64_t *)malloc(sizeof(uint64_t) * nn);
        delta = (double *)malloc(sizeof(double) * nn);
    }
    c->scanned = 0;
    c->diam = 0;
    c->reach = 0;
    for (int32_t i = c->lo; i < c->hi; ++i) {
        int32_t s = c->sources[i];
        if (c->mode == 0) {
            c->scanned += bfs_into(c->R, c->C, n, s, c->dist + (int64_t)i * c->ld, queue);
        } else if (c->mode == 1) {
            sigma_into(c->R, c->C, n, s, c->dist + (int64_t)i * c->ld,
                       c->sigma + (int64_t)i * c->ld, queue);
        } else if (c->mode == 2) {
            if (c->pull)
                brandes_pull_into(c->R, c->C, n, s, tmpd, tmps, delta, queue);
            else
                brandes_f64_into(c->R, c->C, n, s, tmpd, tmps, delta, queue);
            for (int32_t v = 0; v < n; ++v) {
                if (v == s) continue;
                /* Neumaier compensated add */
                double x = delta[v], sum = c->bc_sum[v];
                double t = sum + x;
                if ((sum >= 0 ? sum : -sum) >= (x >= 0 ? x : -x))
                    c->bc_comp[v] += (sum - t) + x;
                else
                    c->bc_comp[v] += (x - t) + sum;
                c->bc_sum[v] = t;
            }
        } else {
            bfs_into(c->R, c->C, n, s, tmpd, queue);
            for (int32_t v = 0; v < n; ++v) {
                if (tmpd[v] != ORACLE_INF) {
                    if (tmpd[v] > c->diam) c->diam = tmpd[v];
                    c->reach++;
                }
            }
        }
    }
    free(queue);
    free(tmpd);
    free(tmps);
    free(delta);
    return NULL;
}

static void run_chunks(chunk_t *proto, int32_t k, int nthreads, chunk_t **out_chunks, int *out_nt)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > k && k > 0) nthreads = k;
    if (k == 0) nthreads = 1;
    chunk_t *ch = (chunk_t *)calloc((size_t)nthreads, sizeof(chunk_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        ch[t] = *proto;
        ch[t].lo = (int32_t)((int64_t)k * t / nthreads);
        ch[t].hi = (int32_t)((int64_t)k * (t + 1) / nthreads);
        if (proto->mode == 2) {
            ch[t].bc_sum = (double *)calloc((size_t)(proto->n > 0 ? proto->n : 1), sizeof(double));
            ch[t].bc_comp = (double *)calloc((size_t)(proto->n > 0 ? proto->n : 1), sizeof(double));
        }
    }
    if (nthreads == 1) {
        chunk_run(&ch[0]);
    } else {
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, chunk_run, &ch[t]);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    }
    free(th);
    *out_chunks = ch;
    *out_nt = nthreads;
}

int64_t oracle_bfs_multi(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                         int32_t k, int32_t *dist, int64_t ld, int nthreads)
{
    chunk_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.R = R; proto.C = C; proto.n = n; proto.sources = sources;
    proto.mode = 0; proto.dist = dist; proto.ld = ld;
    chunk_t *ch; int nt;
    run_chunks(&proto, k, nthreads, &ch, &nt);
    int64_t scanned = 0;
    for (int t = 0; t < nt; ++t) scanned += ch[t].scanned;
    free(ch);
    return scanned;
}

void oracle_sigma_multi(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                        int32_t k, int32_t *dist, uint64_t *sigma, int64_t ld, int nthreads)
{
    chunk_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.R = R; proto.C = C; proto.n = n; proto.sources = sources;
    proto.mode = 1; proto.dist = dist; proto.sigma = sigma; proto.ld = ld;
    chunk_t *ch; int nt;
    run_chunks(&proto, k, nthreads, &ch, &nt);
    free(ch);
}

void oracle_bc(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
               int32_t k, int pull, double *bc, int nthreads)
{
    chunk_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.R = R; proto.C = C; proto.n = n; proto.sources = sources;
    proto.mode = 2; proto.pull = pull;
    chunk_t *ch; int nt;
    run_chunks(&proto, k, nthreads, &ch, &nt);
    for (int32_t v = 0; v < n; ++v) {
        double sum = 0.0, comp = 0.0;
        for (int t = 0; t < nt; ++t) {
            double x = ch[t].bc_sum[v] + ch[t].bc_comp[v];
            double s2 = sum + x;
            if ((sum >= 0 ? sum : -sum) >= (x >= 0 ? x : -x)) comp += (sum - s2) + x;
            else comp += (x - s2) + sum;
            sum = s2;
        }
        bc[v] = sum + comp;
    }
    for (int t = 0; t < nt; ++t) { free(ch[t].bc_sum); free(ch[t].bc_comp); }
    free(ch);
}

int32_t oracle_diameter(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                        int32_t k, int nthreads)
{
    chunk_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.R = R; proto.C = C; proto.n = n; proto.sources = sources;
    proto.mode = 3;
    chunk_t *ch; int nt;
    run_chunks(&proto, k, nthreads, &ch, &nt);
    int32_t d = 0;
    for (int t = 0; t < nt; ++t) if (ch[t].diam > d) d = ch[t].diam;
    free(ch);
    return d;
}

int64_t oracle_reach_count(const int32_t *R, const int32_t *C, int32_t n, const int32_t *sources,
                           int32_t k, int nthreads)
{
    chunk_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.R = R; proto.C = C; proto.n = n; proto.sources = sources;
    proto.mode = 4;
    chunk_t *ch; int nt;
    run_chunks(&proto, k, nthreads, &ch, &nt);
    int64_t r = 0;
    for (int t = 0; t < nt; ++t) r += ch[t].reach;
    free(ch);
    return r;
}

/* ---- LBS: examples/load_balanced_search/lbs.cu:18-31 and :44 ------------- */
int oracle_lbs(const int32_t *counts, int32_t N, int32_t *scanned, int32_t *result,
               int64_t result_capacity, int64_t *total)
{
    int64_t acc = 0;
    for (int32_t i = 0; i < N; ++i) {
        if (acc > 2147483647LL) return -1;
        scanned[i] = (int32_t)acc;
        acc += counts[i];
    }
    *total = acc;
    if (acc > 2147483647LL || acc > result_capacity) return -1;
    /* merge path of the work-slot keys 0..total-1 against scanned[] (upper bound) */
    int64_t ai = 0;
    int32_t bi = 0;
    while (ai < acc || bi < N) {
        int p;
        if (bi >= N) p = 1;
        else if (ai >= acc) p = 0;
        else p = ai < scanned[bi];
        if (p) result[ai++] = bi - 1;
        else ++bi;
    }
    return 0;
}

/* ---- race_and_resolve: graph-utils/race_and_resolve.cuh:13-25 ------------- */
int32_t oracle_race_and_resolve(uint32_t vote, int32_t lane)
{
    if (vote == 0) return lane;
    int32_t b = 31;
    while (!((vote >> b) & 1u)) --b; /* bfind.u32: most significant set bit */
    return b;
}

/* ---- DAG reachable pairs: graph-utils/dag_reachability.cpp:36-65 ---------- */
int64_t oracle_dag_reach_pairs(const int32_t *R, const int32_t *C, int32_t n)
{
    return oracle_dag_reach_counts(R, C, n, NULL);
}

/* Per-vertex sizes of the reachable sets (the vertex itself excluded) that
 * get_reachability_dag (graph-utils/dag_reachability.cpp:36-65) returns;
 * counts may be NULL.  Returns their sum. */
int64_t oracle_dag_reach_counts(const int32_t *R, const int32_t *C, int32_t n, int64_t *counts)
{
    /* Kahn order, then bitset union in reverse topological order. */
    int32_t *indeg = (int32_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int32_t));
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int32_t v = 0; v < n; ++v)
        for (int32_t k = R[v]; k < R[v + 1]; ++k) indeg[C[k]]++;
    int32_t head = 0, tail = 0;
    for (int32_t v = 0; v < n; ++v) if (indeg[v] == 0) order[tail++] = v;
    while (head < tail) {
        int32_t v = order[head++];
        for (int32_t k = R[v]; k < R[v + 1]; ++k)
            if (--indeg[C[k]] == 0) order[tail++] = C[k];
    }
    size_t words = ((size_t)n + 63) / 64;
    uint64_t *bits = (uint64_t *)calloc((size_t)(n > 0 ? n : 1) * (words ? words : 1), sizeof(uint64_t));
    int64_t pairs = 0;
    for (int32_t idx = tail - 1; idx >= 0; --idx) {
        int32_t v = order[idx];
        uint64_t *bv = bits + (size_t)v * words;
        for (int32_t k = R[v]; k < R[v + 1]; ++k) {
            int32_t w = C[k];
            uint64_t *bw = bits + (size_t)w * words;
            bv[w >> 6] |= 1ull << (w & 63);
            for (size_t q = 0; q < words; ++q) bv[q] |= bw[q];
        }
        int64_t cnt = 0;
        for (size_t q = 0; q < words; ++q) cnt += __builtin_popcountll(bv[q]);
        if (counts) counts[v] = cnt;
        pairs += cnt;
    }
    free(bits);
    free(indeg);
    free(order);
    return pairs;
}

/* ---- the benchmark graph generator, restated for the CPU baseline --------------
 * The reference ships no generator; the benchmark's R-MAT graph and its sources
 * are defined by the library's generator (SplitMix64 seeding xoshiro256**, the
 * published PRNGs of Steele-Lea-Flood and Blackman-Vigna; R-MAT descent of
 * Chakrabarti-Zhan-Faloutsos; chunks of 65536 edges each seeded from the graph
 * seed; Fisher-Yates relabelling; symmetrised CSR with sorted, duplicate-free
 * lists and no self-loops).  This is an independent single-threaded statement of
 * that definition, so that the reference arm builds its input without the
 * library; tests/test_oracle.py checks it equals the library's output. */
static uint64_t g_mix(uint64_t *x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s[4];
} g_rng;

static void g_seed(g_rng *r, uint64_t seed)
{
    for (int i = 0; i < 4; ++i) r->s[i] = g_mix(&seed);
}

static uint64_t g_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t g_next(g_rng *r)
{
    uint64_t *s = r->s;
    const uint64_t out = g_rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = g_rotl(s[3], 45);
    return out;
}

static uint64_t g_below(g_rng *r, uint64_t bound)
{
    if (bound <= 1) return 0;
    const uint64_t lim = ~0ull - (~0ull % bound);
    uint64_t x;
    do {
        x = g_next(r);
    } while (x >= lim);
    return x % bound;
}

static int g_cmp_i32(const void *p, const void *q)
{
    const int32_t a = *(const int32_t *)p, b = *(const int32_t *)q;
    return (a > b) - (a < b);
}

int oracle_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int permute,
                int32_t **R_out, int32_t **C_out, int64_t *m_out)
{
    if (scale < 1 || scale > 30 || edge_factor < 1) return -1;
    const int32_t n = (int32_t)(1u << scale);
    const int64_t ne = (int64_t)edge_factor << scale, chunk = 65536;
    int32_t *eu = malloc(sizeof(int32_t) * (size_t)ne), *ev = malloc(sizeof(int32_t) * (size_t)ne);
    if (!eu || !ev) return -2;
    for (int64_t ch = 0; ch * chunk < ne; ++ch) {
        uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(ch + 1));
        g_rng r;
        g_seed(&r, g_mix(&x));
        for (int64_t e = ch * chunk; e < ne && e < (ch + 1) * chunk; ++e) {
            uint32_t u = 0, v = 0;
            for (int bit = 0; bit < scale; ++bit) {
                const double p = (double)(g_next(&r) >> 11) * 0x1.0p-53;
                if (p < a) continue;
                if (p < a + b) v |= 1u << bit;
                else if (p < a + b + c) u |= 1u << bit;
                else {
                    u |= 1u << bit;
                    v |= 1u << bit;
                }
            }
            eu[e] = (int32_t)u;
            ev[e] = (int32_t)v;
        }
    }
    if (permute) {
        int32_t *perm = malloc(sizeof(int32_t) * (size_t)n);
        if (!perm) return -2;
        for (int32_t i = 0; i < n; ++i) perm[i] = i;
        g_rng r;
        g_seed(&r, seed ^ 0x5EED5EED5EED5EEDull);
        for (int32_t i = n - 1; i > 0; --i) {
            const int32_t j = (int32_t)g_below(&r, (uint64_t)i + 1);
            const int32_t t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
        for (int64_t e = 0; e < ne; ++e) {
            eu[e] = perm[eu[e]];
            ev[e] = perm[ev[e]];
        }
        free(perm);
    }
    /* symmetric CSR: both directions of every non-loop edge, then sort and unique each list */
    int64_t *off = calloc((size_t)n + 1, sizeof(int64_t));
    if (!off) return -2;
    for (int64_t e = 0; e < ne; ++e)
        if (eu[e] != ev[e]) {
            off[eu[e] + 1]++;
            off[ev[e] + 1]++;
        }
    for (int32_t v = 0; v < n; ++v) off[v + 1] += off[v];
    int32_t *tmp = malloc(sizeof(int32_t) * (size_t)(off[n] > 0 ? off[n] : 1));
    int64_t *pos = malloc(sizeof(int64_t) * (size_t)n);
    if (!tmp || !pos) return -2;
    memcpy(pos, off, sizeof(int64_t) * (size_t)n);
    for (int64_t e = 0; e < ne; ++e)
        if (eu[e] != ev[e]) {
            tmp[pos[eu[e]]++] = ev[e];
            tmp[pos[ev[e]]++] = eu[e];
        }
    free(eu);
    free(ev);
    free(pos);
    int32_t *R = malloc(sizeof(int32_t) * ((size_t)n + 1));
    if (!R) return -2;
    int64_t m = 0;
    R[0] = 0;
    for (int32_t v = 0; v < n; ++v) {
        int32_t *lst = tmp + off[v];
        const int64_t len = off[v + 1] - off[v];
        qsort(lst, (size_t)len, sizeof(int32_t), g_cmp_i32);
        for (int64_t i = 0; i < len; ++i)
            if (i == 0 || lst[i] != lst[i - 1]) tmp[m++] = lst[i];  /* m <= off[v]: compaction in place */
        R[v + 1] = (int32_t)m;
    }
    free(off);
    *R_out = R;
    *C_out = tmp;
    *m_out = m;
    return 0;
}

int oracle_sources(int32_t n, int32_t k, uint64_t seed, int32_t *out)
{
    if (k < 0 || k > n) return -1;
    int32_t *idx = malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!idx) return -2;
    for (int32_t i = 0; i < n; ++i) idx[i] = i;
    g_rng r;
    g_seed(&r, seed);
    for (int32_t i = 0; i < k; ++i) {
        const int32_t j = i + (int32_t)g_below(&r, (uint64_t)(n - i));
        const int32_t t = idx[i];
        idx[i] = idx[j];
        idx[j] = t;
    }
    memcpy(out, idx, sizeof(int32_t) * (size_t)k);
    free(idx);
    return 0;
}

void oracle_free(void *p) { free(p); }
