// Host-side graph and pattern I/O and CSR construction.
//
// Formats follow the reference loaders so its files load unchanged:
//  - text data graph: "n m" then m lines "u v" (relation/graph.cpp:255-314)
//  - binary data graph "BINGRPH": 7-byte magic, u32 n, u32 m, m × (u32 u, u32 v)
//    (DataGraph::saveBinaryGraph / loadBinaryGraph, relation/graph.cpp:316-419)
//  - pattern: "n m", m edges, then an optional orbit spec "1 v" or "2 u v"
//    that only relabels vertices (PatternGraph::loadPatternGraph, graph.cpp:661-770)
// The CSR is symmetric with each list sorted ascending (Graph::addDirectedEdges,
// graph.cpp:143-173).  Like the reference, the loaders do not clean input;
// sge_csr_from_edges(dedup=1) does, and sge_graph_create rejects unclean CSR.
#include "common.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace sge {
static thread_local std::string g_err;
void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}
const char *last_error() { return g_err.c_str(); }
sge_status fail(sge_status st, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}
}  // namespace sge

using namespace sge;

namespace {

struct FileBuf {
    std::vector<char> data;
    bool ok = false;
    explicit FileBuf(const char *path) {
        FILE *f = fopen(path, "rb");
        if (!f) return;
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        if (sz < 0) { fclose(f); return; }
        data.resize((size_t)sz + 1);
        size_t got = fread(data.data(), 1, (size_t)sz, f);
        fclose(f);
        data[got] = 0;
        data.resize(got + 1);
        ok = true;
    }
};

// Parses unsigned decimal integers separated by whitespace.
struct Tok {
    const char *p, *end;
    bool next(uint64_t &out) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
        if (p >= end || *p < '0' || *p > '9') return false;
        uint64_t v = 0;
        while (p < end && *p >= '0' && *p <= '9') { v = v * 10 + (uint64_t)(*p - '0'); ++p; }
        out = v;
        return true;
    }
};

// Builds a symmetric CSR from (u,v) pairs: counting sort by source, then a
// per-list sort (parallel over vertex ranges).
sge_status build_csr(const uint32_t *edges, uint64_t m, uint32_t n, int dedup, uint32_t **offsets_out,
                     uint32_t **nbrs_out, uint64_t *nnz_out) {
    if (2 * m >= (1ull << 32))
        return fail(SGE_BAD_INPUT, "graph has %llu directed edges; uint32 EdgeID limit is 2^32-1",
                    (unsigned long long)(2 * m));
    std::vector<uint64_t> deg(n + 1, 0);
    for (uint64_t i = 0; i < m; ++i) {
        uint32_t u = edges[2 * i], v = edges[2 * i + 1];
        if (u >= n || v >= n)
            return fail(SGE_BAD_INPUT, "edge %llu (%u,%u) out of range for n=%u", (unsigned long long)i, u, v, n);
        if (dedup && u == v) continue;
        deg[u]++;
        deg[v]++;
    }
    uint32_t *off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    if (!off) return fail(SGE_OOM, "host allocation of offsets failed");
    uint64_t acc = 0;
    for (uint32_t v = 0; v < n; ++v) { off[v] = (uint32_t)acc; acc += deg[v]; }
    off[n] = (uint32_t)acc;
    uint32_t *nb = (uint32_t *)malloc(sizeof(uint32_t) * (acc ? acc : 1));
    if (!nb) { free(off); return fail(SGE_OOM, "host allocation of %llu neighbours failed", (unsigned long long)acc); }
    std::vector<uint64_t> fill(off, off + n);
    for (uint64_t i = 0; i < m; ++i) {
        uint32_t u = edges[2 * i], v = edges[2 * i + 1];
        if (dedup && u == v) continue;
        nb[fill[u]++] = v;
        nb[fill[v]++] = u;
    }
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            for (uint64_t v = t; v < n; v += nt) std::sort(nb + off[v], nb + off[v + 1]);
        });
    for (auto &x : th) x.join();
    if (dedup) {
        // compact duplicates in place
        uint64_t w = 0;
        uint32_t prev_end = off[0];
        for (uint32_t v = 0; v < n; ++v) {
            uint32_t b = prev_end, e = off[v + 1];
            prev_end = e;
            off[v] = (uint32_t)w;
            for (uint32_t i = b; i < e; ++i)
                if (i == b || nb[i] != nb[i - 1]) nb[w++] = nb[i];
        }
        off[n] = (uint32_t)w;
        acc = w;
    }
    *offsets_out = off;
    *nbrs_out = nb;
    *nnz_out = acc;
    return SGE_OK;
}

}  // namespace

extern "C" {

const char *sge_last_error(void) { return sge::last_error(); }

size_t sge_struct_size(int which) {
    switch (which) {
        case 0: return sizeof(sge_plan_blob);
        case 1: return sizeof(sge_plan_opts);
        case 2: return sizeof(sge_count_opts);
        case 3: return sizeof(sge_stats);
        case 4: return sizeof(sge_graph_info);
        case 5: return sizeof(sge_graph_stats);
        case 6: return sizeof(sge_trie);
        case 7: return sizeof(sge_plan_tuning);
        default: return 0;
    }
}
void sge_free_host(void *p) { free(p); }

sge_status sge_csr_from_edges(const uint32_t *edges, uint64_t m, uint32_t num_vertices, int dedup,
                              uint32_t **offsets, uint32_t **nbrs, uint64_t *nnz) {
    if ((!edges && m) || !offsets || !nbrs || !nnz) return fail(SGE_BAD_INPUT, "sge_csr_from_edges: null argument");
    return build_csr(edges, m, num_vertices, dedup, offsets, nbrs, nnz);
}

sge_status sge_load_graph_file(const char *path, uint32_t **offsets, uint32_t **nbrs, uint32_t *num_vertices,
                               uint64_t *nnz) {
    if (!path || !offsets || !nbrs || !num_vertices || !nnz) return fail(SGE_BAD_INPUT, "sge_load_graph_file: null argument");
    FileBuf fb(path);
    if (!fb.ok) return fail(SGE_IO_ERROR, "Can not open file %s!", path);
    size_t sz = fb.data.size() - 1;
    std::vector<uint32_t> edges;
    uint32_t n = 0;
    uint64_t m = 0;
    if (sz >= 7 && memcmp(fb.data.data(), "BINGRPH", 7) == 0) {
        if (sz < 15) return fail(SGE_IO_ERROR, "%s: truncated BINGRPH header", path);
        uint32_t hdr[2];
        memcpy(hdr, fb.data.data() + 7, 8);
        n = hdr[0];
        m = hdr[1];
        if (sz < 15 + m * 8) return fail(SGE_IO_ERROR, "%s: truncated BINGRPH body (expected %llu edges)", path, (unsigned long long)m);
        edges.resize(2 * m);
        memcpy(edges.data(), fb.data.data() + 15, m * 8);
    } else {
        Tok t{fb.data.data(), fb.data.data() + sz};
        uint64_t nn, mm;
        if (!t.next(nn) || !t.next(mm)) return fail(SGE_IO_ERROR, "%s: missing 'n m' header", path);
        n = (uint32_t)nn;
        m = mm;
        edges.resize(2 * m);
        for (uint64_t i = 0; i < m; ++i) {
            uint64_t a, b;
            if (!t.next(a) || !t.next(b))
                return fail(SGE_IO_ERROR, "error: expecting %llu edges, getting %llu edges.", (unsigned long long)m,
                            (unsigned long long)i);
            edges[2 * i] = (uint32_t)a;
            edges[2 * i + 1] = (uint32_t)b;
        }
    }
    *num_vertices = n;
    return build_csr(edges.data(), m, n, 0, offsets, nbrs, nnz);
}

// "t n m", then "v id label degree" and "e u v" lines in any order
// (LabeledGraph::loadLabeldGraphFromText, relation/labeled_graph.cpp:63-143).
// The lists come out sorted by id (the reference sorts by (label, id); the
// executor keeps id order and checks labels itself).
sge_status sge_load_labeled_graph_file(const char *path, uint32_t **offsets, uint32_t **nbrs, uint32_t **labels,
                                       uint32_t *num_vertices, uint64_t *nnz) {
    if (!path || !offsets || !nbrs || !labels || !num_vertices || !nnz)
        return fail(SGE_BAD_INPUT, "sge_load_labeled_graph_file: null argument");
    FileBuf fb(path);
    if (!fb.ok) return fail(SGE_IO_ERROR, "Can not open file %s .", path);
    const char *q = fb.data.data(), *end = q + fb.data.size() - 1;
    auto tag = [&](char &c) {
        while (q < end && (*q == ' ' || *q == '\t' || *q == '\n' || *q == '\r')) ++q;
        if (q >= end) return false;
        c = *q++;
        return true;
    };
    Tok t{q, end};
    char c = 0;
    uint64_t n = 0, m = 0;
    if (!tag(c) || c != 't') return fail(SGE_IO_ERROR, "%s: expected a 't n m' header", path);
    t.p = q;
    if (!t.next(n) || !t.next(m)) return fail(SGE_IO_ERROR, "%s: expected a 't n m' header", path);
    if (n >= (1ull << 32)) return fail(SGE_BAD_INPUT, "%s: %llu vertices", path, (unsigned long long)n);
    q = t.p;
    std::vector<uint32_t> lab(n, 0), edges;
    std::vector<uint64_t> deg(n, 0);
    std::vector<char> seen(n, 0);
    edges.reserve(2 * m);
    while (tag(c)) {
        t.p = q;
        if (c == 'v') {
            uint64_t id, l, d;
            if (!t.next(id) || !t.next(l) || !t.next(d) || id >= n || l >= (1ull << 32))
                return fail(SGE_IO_ERROR, "%s: bad vertex line", path);
            lab[id] = (uint32_t)l;
            deg[id] = d;
            seen[id] = 1;
        } else if (c == 'e') {
            uint64_t a, b;
            if (!t.next(a) || !t.next(b) || a >= n || b >= n) return fail(SGE_IO_ERROR, "%s: bad edge line", path);
            edges.push_back((uint32_t)a);
            edges.push_back((uint32_t)b);
        } else {
            return fail(SGE_IO_ERROR, "%s: unexpected line type '%c'", path, c);
        }
        q = t.p;
    }
    if (edges.size() / 2 != m)
        return fail(SGE_IO_ERROR, "error: expecting %llu edges, getting %llu edges.", (unsigned long long)m,
                    (unsigned long long)(edges.size() / 2));
    for (uint64_t v = 0; v < n; ++v)
        if (!seen[v]) return fail(SGE_IO_ERROR, "%s: vertex %llu has no 'v' line", path, (unsigned long long)v);
    sge_status st = build_csr(edges.data(), m, (uint32_t)n, 0, offsets, nbrs, nnz);
    if (st != SGE_OK) return st;
    auto drop = [&]() {
        free(*offsets);
        free(*nbrs);
        *offsets = *nbrs = nullptr;
    };
    for (uint64_t v = 0; v < n; ++v) {
        const uint32_t have = (*offsets)[v + 1] - (*offsets)[v];
        if (have != deg[v]) {
            drop();
            return fail(SGE_IO_ERROR, "%s: vertex %llu declares degree %llu but has %u edges", path,
                        (unsigned long long)v, (unsigned long long)deg[v], have);
        }
    }
    *labels = static_cast<uint32_t *>(malloc(sizeof(uint32_t) * std::max<uint64_t>(n, 1)));
    if (!*labels) {
        drop();
        return fail(SGE_OOM, "host allocation of %llu labels failed", (unsigned long long)n);
    }
    memcpy(*labels, lab.data(), sizeof(uint32_t) * n);
    *num_vertices = (uint32_t)n;
    return SGE_OK;
}

sge_status sge_save_graph_binary(const char *path, const uint32_t *offsets, const uint32_t *nbrs, uint32_t n) {
    if (!path || !offsets || (!nbrs && offsets[n])) return fail(SGE_BAD_INPUT, "sge_save_graph_binary: null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(SGE_IO_ERROR, "Can not create file %s!", path);
    uint32_t m = offsets[n] / 2;
    fwrite("BINGRPH", 1, 7, f);
    fwrite(&n, 4, 1, f);
    fwrite(&m, 4, 1, f);
    std::vector<uint32_t> buf;
    buf.reserve(1 << 16);
    for (uint32_t u = 0; u < n; ++u)
        for (uint32_t e = offsets[u]; e < offsets[u + 1]; ++e)
            if (u < nbrs[e]) {
                buf.push_back(u);
                buf.push_back(nbrs[e]);
                if (buf.size() >= (1 << 16)) { fwrite(buf.data(), 4, buf.size(), f); buf.clear(); }
            }
    if (!buf.empty()) fwrite(buf.data(), 4, buf.size(), f);
    int rc = fclose(f);
    return rc == 0 ? SGE_OK : fail(SGE_IO_ERROR, "write to %s failed", path);
}

sge_status sge_load_pattern_file(const char *path, uint32_t *k, uint32_t *m, uint32_t *edges) {
    if (!path || !k || !m || !edges) return fail(SGE_BAD_INPUT, "sge_load_pattern_file: null argument");
    FileBuf fb(path);
    if (!fb.ok) return fail(SGE_IO_ERROR, "Can not open file %s!", path);
    Tok t{fb.data.data(), fb.data.data() + fb.data.size() - 1};
    uint64_t nn, mm;
    if (!t.next(nn) || !t.next(mm)) return fail(SGE_IO_ERROR, "%s: missing 'n m' header", path);
    if (nn < 2 || nn > SGE_MAX_K) return fail(SGE_UNSUPPORTED, "%s: pattern has %llu vertices (supported 2..%u)", path, (unsigned long long)nn, SGE_MAX_K);
    if (mm > nn * (nn - 1) / 2) return fail(SGE_BAD_INPUT, "%s: %llu edges exceed a simple graph on %llu vertices", path, (unsigned long long)mm, (unsigned long long)nn);
    std::vector<uint32_t> e(2 * mm);
    for (uint64_t i = 0; i < mm; ++i) {
        uint64_t a, b;
        if (!t.next(a) || !t.next(b))
            return fail(SGE_IO_ERROR, "error: expecting %llu edges, getting %llu edges.", (unsigned long long)mm, (unsigned long long)i);
        if (a >= nn || b >= nn || a == b) return fail(SGE_BAD_INPUT, "%s: bad edge (%llu,%llu)", path, (unsigned long long)a, (unsigned long long)b);
        e[2 * i] = (uint32_t)a;
        e[2 * i + 1] = (uint32_t)b;
    }
    // optional orbit spec: relabel so the orbit vertex is 0 / the orbit edge is (0,1)
    std::vector<uint32_t> map(nn);
    for (uint32_t i = 0; i < nn; ++i) map[i] = i;
    uint64_t type;
    if (t.next(type)) {
        if (type == 1) {
            uint64_t v;
            if (!t.next(v) || v >= nn) return fail(SGE_BAD_INPUT, "error: expecting a vertex orbit.");
            map[0] = (uint32_t)v;
            map[v] = 0;
        } else if (type == 2) {
            uint64_t a, b;
            if (!t.next(a) || !t.next(b) || a >= nn || b >= nn) return fail(SGE_BAD_INPUT, "error: expecting an edge orbit.");
            map[a] = 0;
            map[b] = 1;
            uint32_t i = 2;
            for (uint32_t j = 0; j < nn; ++j)
                if (j != a && j != b) map[j] = i++;
        } else {
            return fail(SGE_BAD_INPUT, "Scope currently supports vertex or edge orbit.");
        }
    }
    for (uint64_t i = 0; i < 2 * mm; ++i) edges[i] = map[e[i]];
    *k = (uint32_t)nn;
    *m = (uint32_t)mm;
    return SGE_OK;
}

}  // extern "C"
