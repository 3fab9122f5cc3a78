// io.cpp -- graph files at the boundary: the reference's three text formats
// (parse.cpp:88-441) read fast, a binary CSR cache, and the reference's two
// host-graph utilities (parse.cpp:443-478).
//
// Each text reader reproduces the reference parser's result on the same file,
// quirks included, because a drop-in must build the same graph:
//   * lines are split at ' ' and '\t', but a separator met while no token is
//     open is kept as part of the next token (so "1  2" gives "1" and " 2"),
//     and '\r' stays in the token it ends;
//   * METIS ("dimacs"): '%' lines are comments; the first other line holds n and
//     the undirected edge count (a third field must be 0: no weights); line i
//     of the rest lists vertex i's neighbours, 1-based; a field that is not all
//     digits (a leading-space field, "12\r") is dropped; undirected.
//   * SNAP edge list ("edgelist", "edgelist_h": the header flag changes
//     nothing): '#' lines are comments; "u v [ignored...]" per line, 0-based,
//     kept in file order; n = number of distinct ids; R is induced from the
//     sources assuming they are sorted; directed.
//   * MatrixMarket ("market"): '%' lines are comments; the first line must be
//     "rows cols nnz"; every other line exactly "u v" (pattern), 1-based; both
//     directions stored, entries sorted by (row, column); undirected.
// Where the reference has undefined behaviour (more METIS lines or entries than
// the header announces, SNAP ids that are not dense, a line with one field) the
// reader reports GU_ERR_INVALID_ARGUMENT instead.  Files are read whole and
// parsed in place (no per-character string appends) by several threads, each
// over a range of whole lines, the ranges joined in file order -- the result is
// the sequential one.
#include "gu_internal.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace gu {

namespace {

std::vector<char> read_file(const char *path)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("cannot open graph file ") + path);
    std::vector<char> buf;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long sz = std::ftell(f);
        if (sz > 0) buf.reserve((size_t)sz);
        std::fseek(f, 0, SEEK_SET);
    }
    char tmp[1 << 16];
    size_t r;
    while ((r = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    std::fclose(f);
    return buf;
}

// One line's fields as [begin, end) ranges, split as the reference splits them.
struct Fields {
    std::vector<std::pair<const char *, const char *>> f;
    void split(const char *b, const char *e)
    {
        f.clear();
        const char *start = nullptr;  // open token
        for (const char *p = b; p < e; ++p) {
            const bool sep = *p == ' ' || *p == '\t';
            if (sep && start && start < p) {
                f.emplace_back(start, p);
                start = nullptr;
            } else if (!start) {
                start = p;  // a separator opens the token when none is open
            }
        }
        if (start && start < e) f.emplace_back(start, e);
    }
};

bool all_digits(const char *b, const char *e)
{
    if (b == e) return false;
    for (const char *p = b; p < e; ++p)
        if (*p < '0' || *p > '9') return false;
    return true;
}

// std::stoi semantics on a field: leading whitespace, optional sign, digits,
// trailing characters ignored; no digits is an error.
long long to_int(const char *b, const char *e, const char *what)
{
    const char *p = b;
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n' || *p == '\v' || *p == '\f')) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    if (p == e || *p < '0' || *p > '9') throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("not a number in ") + what);
    long long v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p++ - '0');
        if (v > 2147483647LL + 1) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("number out of range in ") + what);
    }
    v = neg ? -v : v;
    if (v > 2147483647LL || v < -2147483648LL) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("number out of range in ") + what);
    return v;
}

// Calls fn(b, e) for every line (without its '\n'), as std::getline yields them.
template <class Fn>
void for_lines(const std::vector<char> &buf, Fn fn)
{
    const char *p = buf.data(), *end = buf.data() + buf.size();
    while (p < end) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        const char *le = nl ? nl : end;
        fn(p, le);
        p = nl ? nl + 1 : end;
    }
}

// CSR offsets induced from COO sources as the reference does (parse.cpp:326-339,
// 417-433): offsets advance whenever a source larger than the last one appears.
void induce_offsets(const std::vector<int32_t> &F, int32_t n, std::vector<int32_t> &R)
{
    R.assign((size_t)n + 1, 0);
    int64_t last = 0;
    const int64_t m = (int64_t)F.size();
    for (int64_t i = 0; i < m; ++i) {
        if (F[i] >= n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "vertex ids are not dense 0..n-1");
        while (F[i] > last && last < (int64_t)n + 1) R[(size_t)++last] = (int32_t)i;
    }
    while (last < n) R[(size_t)++last] = (int32_t)m;
}

void check_columns(const std::vector<int32_t> &C, int32_t n)
{
    for (int32_t c : C)
        if (c < 0 || c >= n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "vertex id out of range");
}

// Splits [b, e) into up to `parts` ranges that end at line ends (each range but
// the last ends just after a '\n'), at least `min_bytes` each.
std::vector<std::pair<const char *, const char *>> line_ranges(const char *b, const char *e, unsigned parts,
                                                              size_t min_bytes)
{
    std::vector<std::pair<const char *, const char *>> r;
    const size_t len = (size_t)(e - b);
    parts = std::max(1u, std::min<unsigned>(parts, (unsigned)(len / std::max<size_t>(min_bytes, 1) + 1)));
    const char *s = b;
    for (unsigned i = 1; i <= parts && s < e; ++i) {
        const char *t = i == parts ? e : b + len * i / parts;
        if (t < s) t = s;
        if (t < e) {
            const char *nl = static_cast<const char *>(std::memchr(t, '\n', (size_t)(e - t)));
            t = nl ? nl + 1 : e;
        }
        r.emplace_back(s, t);
        s = t;
    }
    return r;
}

// Runs fn(i) for i in [0, n) on up to n threads; rethrows the first failure in
// index order after all have finished.
template <class Fn>
void parallel_for(size_t n, Fn fn)
{
    std::vector<std::exception_ptr> err(n);
    std::vector<std::thread> th;
    for (size_t i = 1; i < n; ++i)
        th.emplace_back([&, i] {
            try {
                fn(i);
            } catch (...) {
                err[i] = std::current_exception();
            }
        });
    if (n > 0) {
        try {
            fn(0);
        } catch (...) {
            err[0] = std::current_exception();
        }
    }
    for (auto &t : th) t.join();
    for (auto &x : err)
        if (x) std::rethrow_exception(x);
}

unsigned reader_threads()
{
    const unsigned hw = std::thread::hardware_concurrency();
    return std::max(1u, std::min(hw ? hw : 1u, 32u));
}

// METIS: the header is read first; the vertex lines are then parsed by several
// threads, each over a range of whole lines (its lines' entry counts and
// entries, in order), and joined in line order.  Same result as a sequential
// pass: line i of the body is vertex i whichever thread read it.
HostGraph parse_metis(const std::vector<char> &buf)
{
    HostGraph g;
    g.directed = false;
    Fields fl;
    int64_t m2 = 0;
    const char *p = buf.data(), *end = buf.data() + buf.size();
    bool have_header = false;
    while (p < end && !have_header) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        const char *le = nl ? nl : end;
        if (!(p < le && *p == '%')) {
            fl.split(p, le);
            if (fl.f.size() < 2) throw gu_error(GU_ERR_INVALID_ARGUMENT, "METIS header needs n and m");
            const long long n = to_int(fl.f[0].first, fl.f[0].second, "METIS header");
            m2 = 2 * to_int(fl.f[1].first, fl.f[1].second, "METIS header");
            if (fl.f.size() > 3 ||
                (fl.f.size() == 3 && to_int(fl.f[2].first, fl.f[2].second, "METIS header") != 0))
                throw gu_error(GU_ERR_UNSUPPORTED, "weighted graphs are not supported");
            if (n < 0 || m2 < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "negative size in METIS header");
            g.n = (int32_t)n;
            have_header = true;
        }
        p = nl ? nl + 1 : end;
    }
    if (!have_header) throw gu_error(GU_ERR_INVALID_ARGUMENT, "METIS file has no header");
    struct Part {
        std::vector<int32_t> cnt;  // entries of each vertex line
        std::vector<int32_t> c;    // the entries, 0-based
    };
    const auto ranges = line_ranges(p, end, reader_threads(), (size_t)1 << 20);
    std::vector<Part> parts(ranges.size());
    parallel_for(ranges.size(), [&](size_t i) {
        Part &pt = parts[i];
        Fields f;
        const char *q = ranges[i].first, *qe = ranges[i].second;
        while (q < qe) {
            const char *nl = static_cast<const char *>(std::memchr(q, '\n', (size_t)(qe - q)));
            const char *le = nl ? nl : qe;
            if (!(q < le && *q == '%')) {
                f.split(q, le);
                int32_t k = 0;
                for (const auto &t : f.f) {
                    if (!all_digits(t.first, t.second)) continue;  // dropped, as the reference drops it
                    pt.c.push_back((int32_t)(to_int(t.first, t.second, "METIS adjacency") - 1));
                    ++k;
                }
                pt.cnt.push_back(k);
            }
            q = nl ? nl + 1 : qe;
        }
    });
    // join in line order: the first n lines are the vertices; later lines must be empty
    g.R.assign((size_t)g.n + 1, 0);
    int64_t line = 0, total = 0;
    std::vector<int64_t> c_off(parts.size() + 1, 0);  // where each part's kept entries go
    std::vector<int64_t> keep(parts.size(), 0);       // entries of each part on vertex lines
    for (size_t i = 0; i < parts.size(); ++i) {
        c_off[i] = total;
        for (const int32_t k : parts[i].cnt) {
            if (line < g.n) {
                total += k;
                keep[i] += k;
                g.R[(size_t)++line] = (int32_t)std::min<int64_t>(total, 2147483647LL);
            } else if (k > 0) {
                throw gu_error(GU_ERR_INVALID_ARGUMENT, "more METIS vertex lines than the header's n");
            } else {
                ++line;  // blank line past the last vertex: ignored
            }
        }
    }
    for (int64_t v = std::min<int64_t>(line, g.n); v < g.n; ++v) g.R[(size_t)v + 1] = (int32_t)total;  // missing lines
    if (total > m2) throw gu_error(GU_ERR_INVALID_ARGUMENT, "more METIS entries than twice the header's m");
    g.C.resize((size_t)total);
    parallel_for(parts.size(), [&](size_t i) {
        std::memcpy(g.C.data() + c_off[i], parts[i].c.data(), sizeof(int32_t) * (size_t)keep[i]);
        for (int64_t j = 0; j < keep[i]; ++j) {
            const int32_t c = parts[i].c[(size_t)j];
            if (c < 0 || c >= g.n) throw gu_error(GU_ERR_INVALID_ARGUMENT, "vertex id out of range");
        }
    });
    return g;
}

// SNAP: lines parsed by several threads over ranges of whole lines (each keeps
// its edges in file order), the distinct ids marked in one shared bitset, the
// ranges' edges joined in file order.
HostGraph parse_snap(const std::vector<char> &buf)
{
    HostGraph g;
    g.directed = true;
    struct Part {
        std::vector<int32_t> u, v;
        int32_t max_id = -1;
    };
    const auto ranges = line_ranges(buf.data(), buf.data() + buf.size(), reader_threads(), (size_t)1 << 20);
    std::vector<Part> parts(ranges.size());
    parallel_for(ranges.size(), [&](size_t i) {
        Part &pt = parts[i];
        Fields fl;
        const char *q = ranges[i].first, *qe = ranges[i].second;
        while (q < qe) {
            const char *nl = static_cast<const char *>(std::memchr(q, '\n', (size_t)(qe - q)));
            const char *le = nl ? nl : qe;
            if (!(q < le && *q == '#')) {
                fl.split(q, le);
                if (!fl.f.empty()) {
                    if (fl.f.size() < 2) throw gu_error(GU_ERR_INVALID_ARGUMENT, "edge list line with one field");
                    const long long u = to_int(fl.f[0].first, fl.f[0].second, "edge list");
                    const long long v = to_int(fl.f[1].first, fl.f[1].second, "edge list");
                    if (u < 0 || v < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "negative vertex id");
                    pt.u.push_back((int32_t)u);
                    pt.v.push_back((int32_t)v);
                    pt.max_id = std::max(pt.max_id, (int32_t)std::max(u, v));
                }
            }
            q = nl ? nl + 1 : qe;
        }
    });
    int32_t max_id = -1;
    std::vector<size_t> off(parts.size() + 1, 0);
    for (size_t i = 0; i < parts.size(); ++i) {
        max_id = std::max(max_id, parts[i].max_id);
        off[i + 1] = off[i] + parts[i].u.size();
    }
    // n = number of distinct ids (dense 0..n-1 in a valid file)
    const size_t words = (size_t)(((int64_t)max_id + 64) / 64);
    std::vector<std::atomic<uint64_t>> seen(words);
    for (auto &w : seen) w.store(0, std::memory_order_relaxed);
    parallel_for(parts.size(), [&](size_t i) {
        for (const auto *a : {&parts[i].u, &parts[i].v})
            for (const int32_t x : *a) {
                const uint64_t bit = 1ull << (x & 63);
                if (!(seen[(size_t)x >> 6].load(std::memory_order_relaxed) & bit))
                    seen[(size_t)x >> 6].fetch_or(bit, std::memory_order_relaxed);
            }
    });
    int64_t distinct = 0;
    for (const auto &w : seen) distinct += __builtin_popcountll(w.load(std::memory_order_relaxed));
    if (distinct > 2147483647LL) throw gu_error(GU_ERR_INVALID_ARGUMENT, "too many vertices");
    g.n = (int32_t)distinct;
    std::vector<int32_t> F(off.back());
    g.C.resize(off.back());
    parallel_for(parts.size(), [&](size_t i) {
        std::memcpy(F.data() + off[i], parts[i].u.data(), sizeof(int32_t) * parts[i].u.size());
        std::memcpy(g.C.data() + off[i], parts[i].v.data(), sizeof(int32_t) * parts[i].v.size());
    });
    induce_offsets(F, g.n, g.R);
    check_columns(g.C, g.n);
    return g;
}

// MatrixMarket: the size line first, then the entry lines parsed by several
// threads over ranges of whole lines, joined in file order; both directions of
// every entry, counting-sorted by row and each row's columns sorted.
HostGraph parse_market(const std::vector<char> &buf)
{
    HostGraph g;
    g.directed = false;
    Fields fl;
    const char *p = buf.data(), *end = buf.data() + buf.size();
    bool have_size = false;
    while (p < end && !have_size) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        const char *le = nl ? nl : end;
        if (!(p < le && *p == '%')) {
            fl.split(p, le);
            if (fl.f.size() != 3) throw gu_error(GU_ERR_INVALID_ARGUMENT, "MatrixMarket size line must be: rows cols nnz");
            const long long n = to_int(fl.f[0].first, fl.f[0].second, "MatrixMarket size line");
            const long long nnz = to_int(fl.f[2].first, fl.f[2].second, "MatrixMarket size line");
            if (n < 0 || nnz < 0) throw gu_error(GU_ERR_INVALID_ARGUMENT, "negative size in MatrixMarket size line");
            g.n = (int32_t)n;
            have_size = true;
        }
        p = nl ? nl + 1 : end;
    }
    if (!have_size) throw gu_error(GU_ERR_INVALID_ARGUMENT, "MatrixMarket file has no size line");
    const auto ranges = line_ranges(p, end, reader_threads(), (size_t)1 << 20);
    std::vector<std::vector<std::pair<int32_t, int32_t>>> parts(ranges.size());
    parallel_for(ranges.size(), [&](size_t i) {
        Fields f;
        const char *q = ranges[i].first, *qe = ranges[i].second;
        while (q < qe) {
            const char *nl = static_cast<const char *>(std::memchr(q, '\n', (size_t)(qe - q)));
            const char *le = nl ? nl : qe;
            if (!(q < le && *q == '%')) {
                f.split(q, le);
                if (f.f.size() != 2)
                    throw gu_error(GU_ERR_INVALID_ARGUMENT, "only pattern MatrixMarket entries (u v) are accepted");
                const int32_t u = (int32_t)(to_int(f.f[0].first, f.f[0].second, "MatrixMarket entry") - 1);
                const int32_t v = (int32_t)(to_int(f.f[1].first, f.f[1].second, "MatrixMarket entry") - 1);
                if (u < 0 || u >= g.n || v < 0 || v >= g.n)
                    throw gu_error(GU_ERR_INVALID_ARGUMENT, "vertex id out of range");
                parts[i].emplace_back(u, v);
            }
            q = nl ? nl + 1 : qe;
        }
    });
    // entries in (row, column) order, as the reference's sort of the pairs leaves
    // them: a counting sort by row, then each row's columns sorted
    g.R.assign((size_t)g.n + 1, 0);
    for (const auto &pt : parts)
        for (const auto &e : pt) {
            g.R[(size_t)e.first + 1]++;
            g.R[(size_t)e.second + 1]++;
        }
    for (int32_t v = 0; v < g.n; ++v) g.R[(size_t)v + 1] += g.R[(size_t)v];
    g.C.resize((size_t)g.R[(size_t)g.n]);
    std::vector<int32_t> fill(g.R.begin(), g.R.end() - 1);
    for (const auto &pt : parts)
        for (const auto &e : pt) {
            g.C[(size_t)fill[(size_t)e.first]++] = e.second;
            g.C[(size_t)fill[(size_t)e.second]++] = e.first;
        }
    const unsigned nt = reader_threads();
    parallel_for(nt, [&](size_t t) {
        for (int64_t v = (int64_t)t; v < g.n; v += nt)
            std::sort(g.C.begin() + g.R[(size_t)v], g.C.begin() + g.R[(size_t)v + 1]);
    });
    return g;
}

constexpr char CSR_MAGIC[8] = {'G', 'U', 'C', 'S', 'R', '1', 0, 0};

HostGraph read_csr_cache(const std::vector<char> &buf)
{
    const size_t head = sizeof(CSR_MAGIC) + 4 + 8 + 4;
    if (buf.size() < head || std::memcmp(buf.data(), CSR_MAGIC, sizeof(CSR_MAGIC)) != 0)
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "not a binary CSR cache file");
    int32_t n, directed;
    int64_t m;
    const char *p = buf.data() + sizeof(CSR_MAGIC);
    std::memcpy(&n, p, 4);
    std::memcpy(&m, p + 4, 8);
    std::memcpy(&directed, p + 12, 4);
    if (n < 0 || m < 0 || buf.size() != head + 4 * ((size_t)n + 1 + (size_t)m))
        throw gu_error(GU_ERR_INVALID_ARGUMENT, "truncated binary CSR cache file");
    HostGraph g;
    g.n = n;
    g.directed = directed != 0;
    g.R.resize((size_t)n + 1);
    g.C.resize((size_t)m);
    std::memcpy(g.R.data(), buf.data() + head, 4 * ((size_t)n + 1));
    std::memcpy(g.C.data(), buf.data() + head + 4 * ((size_t)n + 1), 4 * (size_t)m);
    if (g.R[0] != 0 || g.R[(size_t)n] != m) throw gu_error(GU_ERR_INVALID_ARGUMENT, "inconsistent binary CSR cache");
    for (int32_t v = 0; v < n; ++v)
        if (g.R[(size_t)v + 1] < g.R[(size_t)v]) throw gu_error(GU_ERR_INVALID_ARGUMENT, "inconsistent binary CSR cache");
    check_columns(g.C, g.n);
    return g;
}

}  // namespace

HostGraph parse_graph_file(const char *path, const char *format)
{
    if (!path || !format) throw gu_error(GU_ERR_INVALID_ARGUMENT, "null path or format");
    const std::string f(format);
    const std::vector<char> buf = read_file(path);
    if (f == "dimacs" || f == "metis") return parse_metis(buf);
    if (f == "edgelist" || f == "edgelist_h") return parse_snap(buf);
    if (f == "market") return parse_market(buf);
    if (f == "csrbin") return read_csr_cache(buf);
    throw gu_error(GU_ERR_UNSUPPORTED, "unsupported graph file format " + f);
}

void write_csr_cache(const HostGraph &g, const char *path)
{
    FILE *f = path ? std::fopen(path, "wb") : nullptr;
    if (!f) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("cannot write ") + (path ? path : "(null)"));
    const int32_t n = g.n, directed = g.directed ? 1 : 0;
    const int64_t m = g.m();
    bool ok = std::fwrite(CSR_MAGIC, 1, sizeof(CSR_MAGIC), f) == sizeof(CSR_MAGIC) && std::fwrite(&n, 4, 1, f) == 1 &&
              std::fwrite(&m, 8, 1, f) == 1 && std::fwrite(&directed, 4, 1, f) == 1 &&
              std::fwrite(g.R.data(), 4, g.R.size(), f) == g.R.size() &&
              (g.C.empty() || std::fwrite(g.C.data(), 4, g.C.size(), f) == g.C.size());
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("short write to ") + path);
}

// host_graph::write_edgelist_to_file (parse.cpp:443-465): optional "n m" line,
// then "source target" per CSR entry.
void write_edgelist(const HostGraph &g, const char *path, bool header)
{
    FILE *f = path ? std::fopen(path, "w") : nullptr;
    if (!f) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("cannot write ") + (path ? path : "(null)"));
    std::string out;
    out.reserve(1 << 20);
    char line[32];
    if (header) out += std::to_string(g.n) + " " + std::to_string(g.m()) + "\n";
    bool ok = true;
    for (int32_t v = 0; v < g.n && ok; ++v) {
        for (int32_t e = g.R[(size_t)v]; e < g.R[(size_t)v + 1]; ++e) {
            const int len = std::snprintf(line, sizeof(line), "%d %d\n", v, g.C[(size_t)e]);
            out.append(line, (size_t)len);
        }
        if (out.size() > (1u << 20)) {
            ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
            out.clear();
        }
    }
    if (ok && !out.empty()) ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw gu_error(GU_ERR_INVALID_ARGUMENT, std::string("short write to ") + path);
}

// host_graph::count_degree_zero_vertices (parse.cpp:467-478).
uint64_t count_degree_zero(const HostGraph &g)
{
    uint64_t c = 0;
    for (int32_t v = 0; v < g.n; ++v) c += g.R[(size_t)v] == g.R[(size_t)v + 1];
    return c;
}

}  // namespace gu
