// gen.cpp -- seeded synthetic graph generators and the host CSR builder.
//
// The reference ships no generator (it parses METIS / SNAP / MatrixMarket files,
// parse.cpp:115-441, into the hybrid CSR/COO host_graph of parse.h:15-35).  These
// generators define the synthetic workloads the library is measured on; every
// stream is a named PRNG (SplitMix64 seeding xoshiro256**), chunked so that the
// output does not depend on the number of host threads.
//
// Output CSR: R[n+1] int32 offsets, C[m] int32 neighbours, each adjacency list
// sorted ascending, duplicates and self-loops removed; undirected graphs store
// both directions (m = 2 * undirected edges), as parse_metis does (parse.cpp:162).
#include "gu_internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>

namespace gu {

static inline uint64_t splitmix64(uint64_t &x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Xoshiro256ss {
    uint64_t s[4];
    explicit Xoshiro256ss(uint64_t seed)
    {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next()
    {
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    // uniform double in [0,1) with 53 random bits (exact on every host)
    inline double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    // uniform integer in [0, bound) by rejection (no modulo bias)
    inline uint64_t below(uint64_t bound)
    {
        if (bound <= 1) return 0;
        uint64_t lim = (~0ull) - ((~0ull) % bound);
        uint64_t r;
        do { r = next(); } while (r >= lim);
        return r % bound;
    }
};

static uint64_t chunk_seed(uint64_t seed, uint64_t chunk)
{
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (chunk + 1));
    return splitmix64(x);
}

static int host_threads()
{
    unsigned h = std::thread::hardware_concurrency();
    if (h == 0) h = 1;
    if (h > 64) h = 64;
    return (int)h;
}

template <class F>
static void parallel_for(int64_t count, F fn)
{
    int nt = host_threads();
    if (count < 4096 || nt == 1) {
        fn(0, count);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        int64_t lo = count * t / nt, hi = count * (t + 1) / nt;
        th.emplace_back([=]() { fn(lo, hi); });
    }
    for (auto &x : th) x.join();
}

// Build a CSR from an edge list (u[i] -> v[i]); symmetric adds both directions.
// Removes self-loops and duplicate entries, sorts each adjacency list.
void build_csr(int32_t n, const std::vector<int32_t> &eu, const std::vector<int32_t> &ev, bool symmetric,
               std::vector<int32_t> &R, std::vector<int32_t> &C)
{
    const int64_t ne = (int64_t)eu.size();
    std::vector<int64_t> deg((size_t)n + 1, 0);
    for (int64_t i = 0; i < ne; ++i) {
        if (eu[i] == ev[i]) continue;
        deg[eu[i]]++;
        if (symmetric) deg[ev[i]]++;
    }
    std::vector<int64_t> off((size_t)n + 1, 0);
    for (int32_t v = 0; v < n; ++v) off[v + 1] = off[v] + deg[v];
    std::vector<int32_t> tmp((size_t)off[n]);
    std::vector<int64_t> pos(off.begin(), off.end() - 1);
    for (int64_t i = 0; i < ne; ++i) {
        int32_t a = eu[i], b = ev[i];
        if (a == b) continue;
        tmp[pos[a]++] = b;
        if (symmetric) tmp[pos[b]++] = a;
    }
    // sort + unique each list in parallel; record unique lengths
    std::vector<int64_t> ulen((size_t)n, 0);
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v) {
            int32_t *b = tmp.data() + off[v], *e = tmp.data() + off[v + 1];
            std::sort(b, e);
            ulen[v] = std::unique(b, e) - b;
        }
    });
    R.assign((size_t)n + 1, 0);
    int64_t total = 0;
    for (int32_t v = 0; v < n; ++v) {
        total += ulen[v];
        if (total > INT32_MAX) throw gu_error(GU_ERR_OVERFLOW, "graph has more than INT32_MAX CSR entries");
        R[v + 1] = (int32_t)total;
    }
    C.resize((size_t)total);
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v)
            std::memcpy(C.data() + R[v], tmp.data() + off[v], sizeof(int32_t) * (size_t)ulen[v]);
    });
}

static std::vector<int32_t> random_permutation(int32_t n, uint64_t seed)
{
    std::vector<int32_t> p((size_t)n);
    for (int32_t i = 0; i < n; ++i) p[i] = i;
    Xoshiro256ss rng(seed);
    for (int32_t i = n - 1; i > 0; --i) {
        int32_t j = (int32_t)rng.below((uint64_t)i + 1);
        std::swap(p[i], p[j]);
    }
    return p;
}

// R-MAT (Chakrabarti, Zhan, Faloutsos 2004): each of edge_factor * 2^scale edges
// descends `scale` levels of the adjacency matrix, picking quadrant
// (0,0),(0,1),(1,0),(1,1) with probabilities a,b,c,1-a-b-c.  Vertex labels are
// then relabelled by a seeded random permutation (Graph500 convention) when
// permute != 0.  The graph is symmetrised.
HostGraph gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, bool permute)
{
    if (scale < 1 || scale > 30) throw gu_error(GU_ERR_INVALID_ARGUMENT, "rmat scale must be in [1,30]");
    if (edge_factor < 1) throw gu_error(GU_ERR_INVALID_ARGUMENT, "rmat edge factor must be >= 1");
    if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0))
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "rmat probabilities must be non-negative and sum to <= 1");
    const int32_t n = (int32_t)(1u << scale);
    const int64_t ne = (int64_t)edge_factor << scale;
    std::vector<int32_t> eu((size_t)ne), ev((size_t)ne);
    const int64_t CH = 1 << 16;
    const int64_t nch = (ne + CH - 1) / CH;
    const double ab = a + b, abc = a + b + c;
    parallel_for(nch, [&](int64_t lo, int64_t hi) {
        for (int64_t ch = lo; ch < hi; ++ch) {
            Xoshiro256ss rng(chunk_seed(seed, (uint64_t)ch));
            int64_t e0 = ch * CH, e1 = std::min(ne, e0 + CH);
            for (int64_t e = e0; e < e1; ++e) {
                uint32_t u = 0, v = 0;
                for (int bit = 0; bit < scale; ++bit) {
                    double r = rng.uniform();
                    if (r < a) {
                    } else if (r < ab) {
                        v |= 1u << bit;
                    } else if (r < abc) {
                        u |= 1u << bit;
                    } else {
                        u |= 1u << bit;
                        v |= 1u << bit;
                    }
                }
                eu[e] = (int32_t)u;
                ev[e] = (int32_t)v;
            }
        }
    });
    if (permute) {
        std::vector<int32_t> p = random_permutation(n, seed ^ 0x5EED5EED5EED5EEDull);
        parallel_for(ne, [&](int64_t lo, int64_t hi) {
            for (int64_t e = lo; e < hi; ++e) {
                eu[e] = p[eu[e]];
                ev[e] = p[ev[e]];
            }
        });
    }
    HostGraph g;
    g.n = n;
    g.directed = false;
    build_csr(n, eu, ev, true, g.R, g.C);
    return g;
}

// Erdos-Renyi G(n, m): m distinct unordered pairs {u,v}, u != v, uniform.
HostGraph gen_er(int32_t n, int64_t m, uint64_t seed)
{
    if (n < 2 && m > 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "G(n,m) needs n >= 2");
    if ((double)m > 0.5 * (double)n * (double)(n - 1)) throw gu_error(GU_ERR_INVALID_ARGUMENT, "G(n,m): m too large");
    Xoshiro256ss rng(seed);
    std::unordered_set<uint64_t> seen;
    seen.reserve((size_t)m * 2);
    std::vector<int32_t> eu, ev;
    eu.reserve((size_t)m);
    ev.reserve((size_t)m);
    while ((int64_t)eu.size() < m) {
        int32_t u = (int32_t)rng.below((uint64_t)n), v = (int32_t)rng.below((uint64_t)n);
        if (u == v) continue;
        int32_t lo = std::min(u, v), hi = std::max(u, v);
        uint64_t key = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
        if (!seen.insert(key).second) continue;
        eu.push_back(lo);
        ev.push_back(hi);
    }
    HostGraph g;
    g.n = n;
    g.directed = false;
    build_csr(n, eu, ev, true, g.R, g.C);
    return g;
}

// rows x cols 4-neighbour grid, vertex id r*cols+c.  Every undirected edge is
// deleted independently with probability p_delete (Bernoulli per edge, one
// stream, horizontal edges in row-major order first, then vertical edges).
HostGraph gen_grid(int32_t rows, int32_t cols, double p_delete, uint64_t seed)
{
    if (rows < 1 || cols < 1 || (int64_t)rows * cols > INT32_MAX) throw gu_error(GU_ERR_INVALID_ARGUMENT, "bad grid size");
    Xoshiro256ss rng(seed);
    std::vector<int32_t> eu, ev;
    eu.reserve((size_t)2 * rows * cols);
    ev.reserve((size_t)2 * rows * cols);
    for (int32_t r = 0; r < rows; ++r)
        for (int32_t c = 0; c + 1 < cols; ++c) {
            bool del = rng.uniform() < p_delete;
            if (!del) { eu.push_back(r * cols + c); ev.push_back(r * cols + c + 1); }
        }
    for (int32_t r = 0; r + 1 < rows; ++r)
        for (int32_t c = 0; c < cols; ++c) {
            bool del = rng.uniform() < p_delete;
            if (!del) { eu.push_back(r * cols + c); ev.push_back((r + 1) * cols + c); }
        }
    HostGraph g;
    g.n = rows * cols;
    g.directed = false;
    build_csr(g.n, eu, ev, true, g.R, g.C);
    return g;
}

// Random DAG: a seeded random topological order pi; m edge draws, each picks two
// distinct ranks i < j uniformly and adds pi[i] -> pi[j]; duplicates removed.
HostGraph gen_dag(int32_t n, int64_t m, uint64_t seed)
{
    if (n < 2) throw gu_error(GU_ERR_INVALID_ARGUMENT, "DAG needs n >= 2");
    std::vector<int32_t> pi = random_permutation(n, seed ^ 0xDA6DA6DA6ull);
    std::vector<int32_t> eu((size_t)m), ev((size_t)m);
    const int64_t CH = 1 << 16;
    const int64_t nch = (m + CH - 1) / CH;
    parallel_for(nch, [&](int64_t lo, int64_t hi) {
        for (int64_t ch = lo; ch < hi; ++ch) {
            Xoshiro256ss rng(chunk_seed(seed, (uint64_t)ch));
            for (int64_t e = ch * CH; e < std::min(m, (ch + 1) * CH); ++e) {
                int32_t i, j;
                do {
                    i = (int32_t)rng.below((uint64_t)n);
                    j = (int32_t)rng.below((uint64_t)n);
                } while (i == j);
                if (i > j) std::swap(i, j);
                eu[e] = pi[i];
                ev[e] = pi[j];
            }
        }
    });
    HostGraph g;
    g.n = n;
    g.directed = true;
    build_csr(n, eu, ev, false, g.R, g.C);
    return g;
}

// k distinct vertices drawn uniformly without replacement (partial Fisher-Yates).
std::vector<int32_t> gen_sources(int32_t n, int32_t k, uint64_t seed)
{
    if (k < 0 || k > n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "need 0 <= k <= n sources");
    std::vector<int32_t> idx((size_t)n);
    for (int32_t i = 0; i < n; ++i) idx[i] = i;
    Xoshiro256ss rng(seed);
    for (int32_t i = 0; i < k; ++i) {
        int32_t j = i + (int32_t)rng.below((uint64_t)(n - i));
        std::swap(idx[i], idx[j]);
    }
    idx.resize((size_t)k);
    return idx;
}

// Reorders every adjacency list C[R[v]..R[v+1]) by descending key[neighbour]
// (ties by ascending id).  Search results do not depend on the order of a
// list; bottom-up levels stop scanning a list early once its first entries
// cover every missing source, and high-degree neighbours are the likeliest to.
void sort_adjacency_by_key(const int32_t *R, int32_t *C, int32_t n, const int32_t *key)
{
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v)
            std::sort(C + R[v], C + R[v + 1], [&](int32_t x, int32_t y) {
                return key[x] != key[y] ? key[x] > key[y] : x < y;
            });
    });
}

HostGraph transpose(const HostGraph &g)
{
    HostGraph t;
    t.n = g.n;
    t.directed = g.directed;
    t.R.assign((size_t)g.n + 1, 0);
    for (int32_t c : g.C) t.R[c + 1]++;
    for (int32_t v = 0; v < g.n; ++v) t.R[v + 1] += t.R[v];
    t.C.resize(g.C.size());
    std::vector<int32_t> pos(t.R.begin(), t.R.end() - 1);
    for (int32_t u = 0; u < g.n; ++u)
        for (int32_t k = g.R[u]; k < g.R[u + 1]; ++k) t.C[pos[g.C[k]]++] = u;
    return t;
}

} // namespace gu
