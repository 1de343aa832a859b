/*
 * sge_oracle.c — CPU oracle for the subgraph-enumeration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * arm load liboracle.so, as the checker or as the timed CPU baseline.
 *
 * It holds three things:
 *  1. plain-C restatements of the reference's hot-path primitives, each citing
 *     the function it follows (paths relative to the reference project root);
 *  2. an independent brute-force counter (embeddings, |Aut|, instances) used to
 *     pin count semantics (instances for multi-bag plans, embeddings for
 *     single-bag plans);
 *  3. a CPU executor for sge_plan_blob built from the primitives in (1),
 *     following the reference's join structure (generateCandidates →
 *     MultiIntersection → DFS; traverse → numResults / choosec /
 *     numUniqueCombine at the leaf), parallel over root edges with OpenMP like
 *     parSharedJoin (matching/parallel.cpp:1154-1486);
 *  4. copies of the library's seeded generators and CSR build;
 *  5. the definition of the instrumented kernel's algorithmic-byte counter
 *     for plans whose leaf runs on the root edge, evaluated on the CPU.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sge.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define BST 32 /* BINARY_SEARCH_THRESHOLD, config/config.h:37 */

/* ---------------------------------------------------------------- 1 ---- */

/* choosec — utility/utils.cpp:80-94.  nom = n(n-1)…(n-k+1) accumulated in
 * uint64 (wrapping), denom = k!, result nom/denom.  Kept with the wrap so
 * tests can show where it departs from the exact binomial. */
uint64_t oracle_choosec_ref(uint64_t n, int k) {
    if ((uint64_t)k > n) return 0;
    if (k == 0) return 1;
    uint64_t nom = n, denom = 1;
    for (int i = 1; i < k; i++) {
        nom *= (n - (uint64_t)i);
        denom *= (uint64_t)(i + 1);
    }
    return nom / denom;
}

/* Exact C(n,k) mod 2^64 via 128-bit intermediates (what the executors use). */
uint64_t oracle_binom_exact(uint64_t n, int k) {
    if ((uint64_t)k > n) return 0;
    unsigned __int128 acc = 1;
    for (int i = 0; i < k; i++) acc = acc * (unsigned __int128)(n - (uint64_t)i) / (unsigned __int128)(i + 1);
    return (uint64_t)acc;
}

/* setBeginPos — utility/utils.cpp:581-597: first position with a[j] > maxCompared
 * (linear scan up to BINARY_SEARCH_THRESHOLD, else upper_bound). */
uint32_t oracle_set_begin_pos(const uint32_t *a, uint32_t count, uint32_t maxCompared) {
    uint32_t beginPos = 0;
    if (count <= BST) {
        for (uint32_t j = 0; j < count; ++j)
            if (a[j] > maxCompared) { beginPos = j; break; }
        if (beginPos == 0 && count > 0 && a[count - 1] <= maxCompared) beginPos = count;
    } else {
        uint32_t lo = 0, n = count;
        while (n > 0) {
            uint32_t h = n >> 1;
            if (a[lo + h] <= maxCompared) { lo += h + 1; n -= h + 1; } else n = h;
        }
        beginPos = lo;
    }
    return beginPos;
}

/* setEndPos — utility/utils.cpp:599-612: first position with a[j] >= minCompared. */
uint32_t oracle_set_end_pos(const uint32_t *a, uint32_t count, uint32_t minCompared) {
    uint32_t endPos = count;
    if (count <= BST) {
        for (uint32_t j = 0; j < count; ++j)
            if (a[j] >= minCompared) { endPos = j; break; }
    } else {
        uint32_t lo = 0, n = count;
        while (n > 0) {
            uint32_t h = n >> 1;
            if (a[lo + h] < minCompared) { lo += h + 1; n -= h + 1; } else n = h;
        }
        endPos = lo;
    }
    return endPos;
}

/* GallopingSearch — utility/compute_set_intersection.cpp:89-119: first index
 * in [begin, end) with src[i] >= val, by doubling steps then binary search. */
static uint32_t galloping_search(const uint32_t *src, uint32_t begin, uint32_t end, uint32_t target) {
    if (begin >= end || src[end - 1] < target) return end;
    if (src[begin] >= target) return begin;
    uint32_t offset = 1;
    while (begin + offset < end && src[begin + offset] < target) offset <<= 1;
    uint32_t lo = begin + (offset >> 1), hi = (begin + offset < end) ? begin + offset : end;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (src[mid] < target) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* ComputeCandidates (output) — utility/compute_set_intersection.cpp:10-45 with
 * the scalar kernels of :1136-1327: galloping when one list is more than 50×
 * the other, merge otherwise.  out may alias a. */
uint32_t oracle_intersect(const uint32_t *a, uint32_t na, const uint32_t *b, uint32_t nb, uint32_t *out) {
    uint32_t cnt = 0;
    if (na == 0 || nb == 0) return 0;
    if (na / nb > 50 || nb / na > 50) {
        const uint32_t *s = na < nb ? a : b, *l = na < nb ? b : a;
        uint32_t ns = na < nb ? na : nb, nl = na < nb ? nb : na;
        uint32_t li = 0;
        for (uint32_t si = 0; si < ns; ++si) {
            li = galloping_search(l, li, nl, s[si]);
            if (li >= nl) break;
            if (l[li] == s[si]) { out[cnt++] = s[si]; ++li; }
        }
        return cnt;
    }
    uint32_t i = 0, j = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else { out[cnt++] = a[i]; ++i; ++j; }
    }
    return cnt;
}

/* ComputeCandidates (count only) — compute_set_intersection.cpp:47-87: the
 * galloping switch happens above a 32× ratio. */
uint32_t oracle_intersect_count(const uint32_t *a, uint32_t na, const uint32_t *b, uint32_t nb) {
    uint32_t cnt = 0;
    if (na == 0 || nb == 0) return 0;
    if (na / nb > 32 || nb / na > 32) {
        const uint32_t *s = na < nb ? a : b, *l = na < nb ? b : a;
        uint32_t ns = na < nb ? na : nb, nl = na < nb ? nb : na;
        uint32_t li = 0;
        for (uint32_t si = 0; si < ns; ++si) {
            li = galloping_search(l, li, nl, s[si]);
            if (li >= nl) break;
            if (l[li] == s[si]) { ++cnt; ++li; }
        }
        return cnt;
    }
    uint32_t i = 0, j = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else { ++cnt; ++i; ++j; }
    }
    return cnt;
}

/* checkExists — relation/relation.cpp:206-232: position of target in
 * [begin, end) or end. */
static uint32_t check_exists(const uint32_t *a, uint32_t begin, uint32_t end, uint32_t target) {
    uint32_t lo = begin, hi = end;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] < target) lo = mid + 1; else hi = mid;
    }
    return (lo < end && a[lo] == target) ? lo : end;
}

/* TrieLevel::numResults — relation/relation.cpp:301-338: range after the
 * larger/smaller bounds, minus every already-matched vertex found inside it. */
uint64_t oracle_num_results(const uint32_t *values, uint32_t length, const uint32_t *partMatch,
                            const uint32_t *toCheck, uint32_t nCheck, const uint32_t *larger, uint32_t nLarger,
                            const uint32_t *smaller, uint32_t nSmaller) {
    uint32_t maxCompared = 0, minCompared = 0xFFFFFFFFu;
    for (uint32_t i = 0; i < nLarger; ++i) if (partMatch[larger[i]] > maxCompared) maxCompared = partMatch[larger[i]];
    for (uint32_t i = 0; i < nSmaller; ++i) if (partMatch[smaller[i]] < minCompared) minCompared = partMatch[smaller[i]];
    uint32_t beginPos = 0, endPos = length;
    if (nLarger) beginPos = oracle_set_begin_pos(values, length, maxCompared);
    if (nSmaller) endPos = oracle_set_end_pos(values, length, minCompared);
    if (endPos < beginPos) endPos = beginPos;
    uint64_t num = endPos - beginPos;
    for (uint32_t i = 0; i < nCheck; ++i)
        if (check_exists(values, beginPos, endPos, partMatch[toCheck[i]]) != endPos) --num;
    return num;
}

/* numUniqueCombine — utility/utils.cpp:290-350: number of tuples with one
 * element from each set and all elements distinct, by inclusion–exclusion over
 * subsets of the pairwise "equal" events; each chosen pair set is reduced with
 * a union-find and contributes Π |∩ sets of a component|.  Sets are sorted. */
static uint32_t uf_find(uint32_t *p, uint32_t x) { while (p[x] != x) x = p[x] = p[p[x]]; return x; }
uint64_t oracle_num_unique_combine(const uint32_t *const *sets, const uint32_t *lens, int nsets) {
    if (nsets <= 0) return 1;
    if (nsets > 6) return 0; /* 15 pairs → 2^15 subsets: enough for the tails here */
    uint64_t num = 1;
    for (int i = 0; i < nsets; ++i) num *= lens[i];
    int np = 0, pa[15], pb[15];
    for (int i = 0; i < nsets; ++i)
        for (int j = i + 1; j < nsets; ++j) { pa[np] = i; pb[np] = j; ++np; }
    uint32_t maxlen = 0;
    for (int i = 0; i < nsets; ++i) if (lens[i] > maxlen) maxlen = lens[i];
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (maxlen + 1));
    uint32_t *tmp2 = (uint32_t *)malloc(sizeof(uint32_t) * (maxlen + 1));
    for (uint32_t choice = 1; choice < (1u << np); ++choice) {
        uint32_t par[8];
        for (int i = 0; i < nsets; ++i) par[i] = (uint32_t)i;
        for (int q = 0; q < np; ++q)
            if ((choice >> q) & 1u) {
                uint32_t x = uf_find(par, (uint32_t)pa[q]), y = uf_find(par, (uint32_t)pb[q]);
                if (x != y) par[x] = y;
            }
        uint64_t term = 1;
        for (int r = 0; r < nsets; ++r) {
            if (uf_find(par, (uint32_t)r) != (uint32_t)r) continue;
            /* component rooted at r: intersect its sets */
            int first = 1;
            uint32_t n = 0;
            for (int i = 0; i < nsets; ++i) {
                if (uf_find(par, (uint32_t)i) != (uint32_t)r) continue;
                if (first) { memcpy(tmp, sets[i], sizeof(uint32_t) * lens[i]); n = lens[i]; first = 0; }
                else { n = oracle_intersect(tmp, n, sets[i], lens[i], tmp2); memcpy(tmp, tmp2, sizeof(uint32_t) * n); }
            }
            term *= n;
        }
        if (__builtin_popcount(choice) % 2 == 0) num += term; else num -= term;
    }
    free(tmp);
    free(tmp2);
    return num;
}

/* ---------------------------------------------------------------- 2 ---- */

static int pat_edge(const uint32_t *adj, uint32_t a, uint32_t b) { return (adj[a] >> b) & 1u; }

/* |Aut(P)| by enumerating adjacency-preserving permutations (k <= 10). */
uint64_t oracle_aut_size(uint32_t k, uint32_t m, const uint32_t *edges) {
    uint32_t adj[32] = {0};
    for (uint32_t i = 0; i < m; ++i) { adj[edges[2 * i]] |= 1u << edges[2 * i + 1]; adj[edges[2 * i + 1]] |= 1u << edges[2 * i]; }
    uint32_t map[32], used = 0, next[33];
    uint64_t cnt = 0;
    int i = 0;
    next[0] = 0;
    while (i >= 0) {
        if (i == (int)k) { ++cnt; --i; if (i >= 0) used &= ~(1u << map[i]); continue; }
        int placed = 0;
        for (uint32_t c = next[i]; c < k; ++c) {
            if ((used >> c) & 1u) continue;
            int ok = 1;
            for (int j = 0; j < i && ok; ++j) if (pat_edge(adj, (uint32_t)i, (uint32_t)j) != pat_edge(adj, c, map[j])) ok = 0;
            if (!ok) continue;
            map[i] = c; used |= 1u << c; next[i] = c + 1; ++i; if (i < (int)k) next[i] = 0; placed = 1; break;
        }
        if (!placed) { --i; if (i >= 0) used &= ~(1u << map[i]); }
    }
    return cnt;
}

/* As oracle_aut_size, counting only permutations that also preserve the
 * vertex labels lab (NULL: unlabeled). */
uint64_t oracle_aut_size_labeled(uint32_t k, uint32_t m, const uint32_t *edges, const uint32_t *lab) {
    uint32_t adj[32] = {0};
    for (uint32_t i = 0; i < m; ++i) { adj[edges[2 * i]] |= 1u << edges[2 * i + 1]; adj[edges[2 * i + 1]] |= 1u << edges[2 * i]; }
    uint32_t map[32], used = 0, next[33];
    uint64_t cnt = 0;
    int i = 0;
    next[0] = 0;
    while (i >= 0) {
        if (i == (int)k) { ++cnt; --i; if (i >= 0) used &= ~(1u << map[i]); continue; }
        int placed = 0;
        for (uint32_t c = next[i]; c < k; ++c) {
            if ((used >> c) & 1u) continue;
            if (lab && lab[c] != lab[i]) continue;
            int ok = 1;
            for (int j = 0; j < i && ok; ++j) if (pat_edge(adj, (uint32_t)i, (uint32_t)j) != pat_edge(adj, c, map[j])) ok = 0;
            if (!ok) continue;
            map[i] = c; used |= 1u << c; next[i] = c + 1; ++i; if (i < (int)k) next[i] = 0; placed = 1; break;
        }
        if (!placed) { --i; if (i >= 0) used &= ~(1u << map[i]); }
    }
    return cnt;
}

static int has_edge(const uint32_t *off, const uint32_t *nb, uint32_t u, uint32_t v) {
    uint32_t a = off[u], b = off[u + 1];
    return check_exists(nb, a, b, v) != b;
}

/* Injective homomorphisms (embeddings) of a connected pattern, by DFS over a
 * connected order; each new vertex ranges over the neighbours of its first
 * earlier neighbour and is checked against all other earlier neighbours. */
uint64_t oracle_bruteforce_embeddings_labeled(const uint32_t *off, const uint32_t *nb, uint32_t n, uint32_t k,
                                              uint32_t m, const uint32_t *edges, const uint32_t *plab,
                                              const uint32_t *glab, int threads);
uint64_t oracle_bruteforce_embeddings(const uint32_t *off, const uint32_t *nb, uint32_t n, uint32_t k, uint32_t m,
                                      const uint32_t *edges, int threads) {
    return oracle_bruteforce_embeddings_labeled(off, nb, n, k, m, edges, NULL, NULL, threads);
}

/* Embeddings of a labeled pattern: pattern vertex u maps only to data vertices
 * v with glab[v] == plab[u] (both NULL: unlabeled). */
uint64_t oracle_bruteforce_embeddings_labeled(const uint32_t *off, const uint32_t *nb, uint32_t n, uint32_t k,
                                              uint32_t m, const uint32_t *edges, const uint32_t *plab,
                                              const uint32_t *glab, int threads) {
    uint32_t adj[32] = {0};
    for (uint32_t i = 0; i < m; ++i) { adj[edges[2 * i]] |= 1u << edges[2 * i + 1]; adj[edges[2 * i + 1]] |= 1u << edges[2 * i]; }
    uint32_t order[32], pos[32], seen = 0;
    /* start at the max-degree vertex, then greedily most-connected */
    uint32_t best = 0;
    for (uint32_t u = 1; u < k; ++u) if (__builtin_popcount(adj[u]) > __builtin_popcount(adj[best])) best = u;
    order[0] = best; seen = 1u << best;
    for (uint32_t i = 1; i < k; ++i) {
        int bv = -1, bs = -1;
        for (uint32_t u = 0; u < k; ++u) {
            if ((seen >> u) & 1u) continue;
            int s = __builtin_popcount(adj[u] & seen);
            if (s > 0 && s > bs) { bs = s; bv = (int)u; }
        }
        if (bv < 0) return 0; /* disconnected */
        order[i] = (uint32_t)bv; seen |= 1u << bv;
    }
    for (uint32_t i = 0; i < k; ++i) pos[order[i]] = i;
    uint32_t back[32], first[32];
    for (uint32_t i = 0; i < k; ++i) {
        back[i] = 0;
        for (uint32_t j = 0; j < i; ++j) if (pat_edge(adj, order[i], order[j])) back[i] |= 1u << j;
        first[i] = back[i] ? (uint32_t)__builtin_ctz(back[i]) : 0;
    }
    (void)pos;
    uint64_t total = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
#endif
    for (int64_t r = 0; r < (int64_t)n; ++r) {
        uint32_t mm[32], it[32];
        int lv = 0;
        mm[0] = (uint32_t)r;
        if (plab && glab[r] != plab[order[0]]) continue;
        if (k == 1) { total += 1; continue; }
        lv = 1;
        it[1] = off[mm[first[1]]];
        while (lv >= 1) {
            uint32_t p = mm[first[lv]];
            if (it[lv] >= off[p + 1]) { --lv; continue; }
            uint32_t x = nb[it[lv]++];
            int ok = !plab || glab[x] == plab[order[lv]];
            for (int j = 0; j < lv && ok; ++j) if (mm[j] == x) ok = 0;
            for (uint32_t msk = back[lv] & ~(1u << first[lv]); msk && ok; msk &= msk - 1)
                if (!has_edge(off, nb, mm[__builtin_ctz(msk)], x)) ok = 0;
            if (!ok) continue;
            mm[lv] = x;
            if (lv + 1 == (int)k) { total += 1; continue; }
            ++lv;
            it[lv] = off[mm[first[lv]]];
        }
    }
    return total;
}

/* ---------------------------------------------------------------- 3 ---- */

typedef struct {
    const uint32_t *off, *nb;
    const sge_plan_blob *p;
    uint32_t maxdeg;
} exec_ctx;

/* Candidates of level i: bound-trim every parent list (setBeginPos /
 * setEndPos as in generateCandidates, matching/join.cpp:137-178), intersect
 * them pairwise shortest-first (MultiIntersection, compute_set_intersection.cpp:308-342),
 * then drop the matched vertices of check[i] (visited[]). */
static uint32_t level_candidates(const exec_ctx *c, uint32_t i, const uint32_t *mm, uint32_t *out, uint32_t *tmp) {
    const sge_plan_blob *p = c->p;
    uint32_t lo = 0, hi = 0xFFFFFFFFu;
    int has_lo = p->lower[i] != 0, has_hi = p->upper[i] != 0;
    for (uint32_t msk = p->lower[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] > lo) lo = mm[__builtin_ctz(msk)];
    for (uint32_t msk = p->upper[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] < hi) hi = mm[__builtin_ctz(msk)];
    const uint32_t *lists[32];
    uint32_t lens[32], nl = 0;
    for (uint32_t msk = p->parents[i]; msk; msk &= msk - 1) {
        uint32_t v = mm[__builtin_ctz(msk)];
        const uint32_t *a = c->nb + c->off[v];
        uint32_t len = c->off[v + 1] - c->off[v];
        if (has_lo) { uint32_t b = oracle_set_begin_pos(a, len, lo); a += b; len -= b; }
        if (has_hi) len = oracle_set_end_pos(a, len, hi);
        lists[nl] = a; lens[nl] = len; ++nl;
    }
    /* shortest first */
    for (uint32_t x = 0; x < nl; ++x)
        for (uint32_t y = x + 1; y < nl; ++y)
            if (lens[y] < lens[x]) {
                const uint32_t *t = lists[x]; lists[x] = lists[y]; lists[y] = t;
                uint32_t tl = lens[x]; lens[x] = lens[y]; lens[y] = tl;
            }
    uint32_t n = lens[0];
    memcpy(out, lists[0], sizeof(uint32_t) * n);
    for (uint32_t l = 1; l < nl && n; ++l) {
        n = oracle_intersect(out, n, lists[l], lens[l], tmp);
        memcpy(out, tmp, sizeof(uint32_t) * n);
    }
    uint32_t w = 0;
    for (uint32_t e = 0; e < n; ++e) {
        int ex = 0;
        for (uint32_t msk = p->check[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] == out[e]) ex = 1;
        if (!ex) out[w++] = out[e];
    }
    return w;
}

/* A tail level whose parents all precede the last enumerated level has a
 * candidate set that does not change while the last levels vary: like a bag
 * relation built once per binding of its prefix (nodeJoin + buildTrie,
 * matching/join.cpp:309-421,1713-1717), its intersection is computed when its
 * last parent is matched and reused (bounds and exclusions applied at the leaf). */
static int hoisted_level(const sge_plan_blob *p, uint32_t i) {
    const uint32_t par = p->parents[i];
    if (i < p->num_enum || __builtin_popcount(par) < 2) return 0;
    const uint32_t last = 31u - (uint32_t)__builtin_clz(par);
    return last + 1 < p->num_enum;
}
static uint32_t hoist_at_level(const sge_plan_blob *p, uint32_t i) {
    const uint32_t last = 31u - (uint32_t)__builtin_clz(p->parents[i]);
    return last < 1 ? 1u : last;
}

/* Intersection of the parents' lists of level i, no bounds, no exclusions. */
static uint32_t raw_intersection(const exec_ctx *c, uint32_t i, const uint32_t *mm, uint32_t *out, uint32_t *tmp) {
    const sge_plan_blob *p = c->p;
    const uint32_t *lists[32];
    uint32_t lens[32], nl = 0;
    for (uint32_t msk = p->parents[i]; msk; msk &= msk - 1) {
        uint32_t v = mm[__builtin_ctz(msk)];
        lists[nl] = c->nb + c->off[v];
        lens[nl] = c->off[v + 1] - c->off[v];
        ++nl;
    }
    for (uint32_t x = 0; x < nl; ++x)
        for (uint32_t y = x + 1; y < nl; ++y)
            if (lens[y] < lens[x]) {
                const uint32_t *t = lists[x]; lists[x] = lists[y]; lists[y] = t;
                uint32_t tl = lens[x]; lens[x] = lens[y]; lens[y] = tl;
            }
    uint32_t n = lens[0];
    memcpy(out, lists[0], sizeof(uint32_t) * n);
    for (uint32_t l = 1; l < nl && n; ++l) {
        n = oracle_intersect(out, n, lists[l], lens[l], tmp);
        memcpy(out, tmp, sizeof(uint32_t) * n);
    }
    return n;
}

/* Level i's candidates from a stored hoisted list: bound trim (setBeginPos /
 * setEndPos) and the matched vertices dropped (visited[]). */
static uint32_t from_hoisted(const exec_ctx *c, uint32_t i, const uint32_t *mm, const uint32_t *h, uint32_t hn,
                             uint32_t *out) {
    const sge_plan_blob *p = c->p;
    uint32_t lo = 0, hi = 0xFFFFFFFFu;
    for (uint32_t msk = p->lower[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] > lo) lo = mm[__builtin_ctz(msk)];
    for (uint32_t msk = p->upper[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] < hi) hi = mm[__builtin_ctz(msk)];
    uint32_t b = p->lower[i] ? oracle_set_begin_pos(h, hn, lo) : 0;
    uint32_t e = p->upper[i] ? oracle_set_end_pos(h, hn, hi) : hn;
    uint32_t w = 0;
    for (uint32_t x = b; x < e; ++x) {
        int ex = 0;
        for (uint32_t msk = p->check[i]; msk; msk &= msk - 1) if (mm[__builtin_ctz(msk)] == h[x]) ex = 1;
        if (!ex) out[w++] = h[x];
    }
    return w;
}

/* Leaf count (traverse, matching/join.cpp:1520-1691).  hoist[i]/hoist_n[i]
 * hold the stored list of hoisted tail levels (NULL otherwise). */
static uint64_t tail_count(const exec_ctx *c, const uint32_t *mm, uint32_t **bufs, uint32_t *tmp,
                           uint32_t *const *hoist, const uint32_t *hoist_n) {
    const sge_plan_blob *p = c->p;
    const uint32_t ne = p->num_enum, T = p->tail_len;
    #define TAIL_CANDS(i, out) (hoist[(i)] ? from_hoisted(c, (i), mm, hoist[(i)], hoist_n[(i)], (out)) \
                                           : level_candidates(c, (i), mm, (out), tmp))
    if (p->tail_mode == SGE_TAIL_SINGLE || p->tail_mode == SGE_TAIL_CHOOSE) {
        uint32_t n = TAIL_CANDS(ne, bufs[0]);
        if (p->tail_mode == SGE_TAIL_SINGLE) return (uint64_t)n;
        return p->choose_wrap ? oracle_choosec_ref(n, (int)T) : oracle_binom_exact(n, (int)T);
    }
    const uint32_t *sets[SGE_MAX_TAIL];
    uint32_t lens[SGE_MAX_TAIL];
    for (uint32_t t = 0; t < T; ++t) {
        lens[t] = TAIL_CANDS(ne + t, bufs[t]);
        sets[t] = bufs[t];
    }
    #undef TAIL_CANDS
    return oracle_num_unique_combine(sets, lens, (int)T);
}

/* Runs the plan over root tasks t ≡ offset (mod stride).  Returns the sum of
 * per-root counts (instances; multiply by count_multiplier for the
 * reference's number). */
static uint64_t count_plan_roots(const uint32_t *off, const uint32_t *nb, uint32_t maxdeg, const uint32_t *eu,
                                 const uint32_t *ev, uint64_t m, const sge_plan_blob *p, int threads, uint64_t stride,
                                 uint64_t offset, uint32_t root_max_degree, uint64_t *roots_done);

/* Root edges u<v in CSR order (the engine's root-task numbering). */
static uint64_t root_edges(const uint32_t *off, const uint32_t *nb, uint32_t n, uint32_t **eu, uint32_t **ev,
                           uint32_t *maxdeg) {
    uint64_t m = off[n] / 2, w = 0;
    *maxdeg = 0;
    for (uint32_t v = 0; v < n; ++v) if (off[v + 1] - off[v] > *maxdeg) *maxdeg = off[v + 1] - off[v];
    *eu = (uint32_t *)malloc(sizeof(uint32_t) * (m + 1));
    *ev = (uint32_t *)malloc(sizeof(uint32_t) * (m + 1));
    for (uint32_t u = 0; u < n; ++u)
        for (uint32_t e = off[u]; e < off[u + 1]; ++e)
            if (nb[e] > u) { (*eu)[w] = u; (*ev)[w] = nb[e]; ++w; }
    return m;
}

uint64_t oracle_count_plan(const uint32_t *off, const uint32_t *nb, uint32_t n, const sge_plan_blob *p, int threads,
                           uint64_t stride, uint64_t offset, uint64_t *roots_done) {
    uint32_t *eu, *ev, maxdeg;
    const uint64_t m = root_edges(off, nb, n, &eu, &ev, &maxdeg);
    const uint64_t r = count_plan_roots(off, nb, maxdeg, eu, ev, m, p, threads, stride, offset, 0, roots_done);
    free(eu);
    free(ev);
    return r;
}

/* Several plans over the same root sample, the root list built once:
 * counts[i] = instances of plan i over the sampled roots, roots[i] = the
 * root tasks it ran.  root_max_degree > 0 keeps only the roots whose two
 * endpoints both have at most that degree. */
void oracle_count_plans(const uint32_t *off, const uint32_t *nb, uint32_t n, const sge_plan_blob *plans,
                        uint32_t nplans, int threads, uint64_t stride, uint64_t offset, uint32_t root_max_degree,
                        uint64_t *counts, uint64_t *roots) {
    uint32_t *eu, *ev, maxdeg;
    const uint64_t m = root_edges(off, nb, n, &eu, &ev, &maxdeg);
    for (uint32_t i = 0; i < nplans; ++i)
        counts[i] = count_plan_roots(off, nb, maxdeg, eu, ev, m, &plans[i], threads, stride, offset, root_max_degree,
                                     &roots[i]);
    free(eu);
    free(ev);
}

/* A graph prepared once for many counting calls: the root edge list and the
 * largest degree (building them is a pass over every edge). */
typedef struct {
    const uint32_t *off, *nb;
    uint32_t n, maxdeg;
    uint32_t *eu, *ev;
    uint64_t m;
} oracle_ctx;

void *oracle_ctx_create(const uint32_t *off, const uint32_t *nb, uint32_t n) {
    oracle_ctx *c = (oracle_ctx *)malloc(sizeof(oracle_ctx));
    c->off = off;
    c->nb = nb;
    c->n = n;
    c->m = root_edges(off, nb, n, &c->eu, &c->ev, &c->maxdeg);
    return c;
}

void oracle_ctx_free(void *h) {
    oracle_ctx *c = (oracle_ctx *)h;
    if (!c) return;
    free(c->eu);
    free(c->ev);
    free(c);
}

/* oracle_count_plans on a prepared graph (the arrays it was made from must
 * still be alive). */
void oracle_ctx_count_plans(void *h, const sge_plan_blob *plans, uint32_t nplans, int threads, uint64_t stride,
                            uint64_t offset, uint32_t root_max_degree, uint64_t *counts, uint64_t *roots) {
    const oracle_ctx *c = (const oracle_ctx *)h;
    for (uint32_t i = 0; i < nplans; ++i)
        counts[i] = count_plan_roots(c->off, c->nb, c->maxdeg, c->eu, c->ev, c->m, &plans[i], threads, stride, offset,
                                     root_max_degree, &roots[i]);
}

/* Runs plan p over the sampled undirected root edges e ≡ offset (mod stride)
 * (both orientations when the root is unordered), in parallel like
 * parSharedJoin (matching/parallel.cpp:1154-1486), with one refinement: a root
 * with more than 64 level-2 candidates is split into up to 64 work items over
 * ranges of them, so one heavy root does not hold a single thread while the
 * others idle.  The counts are the same; only the CPU's time is shorter. */
static uint64_t count_plan_roots(const uint32_t *off, const uint32_t *nb, uint32_t maxdeg, const uint32_t *eu,
                                 const uint32_t *ev, uint64_t m, const sge_plan_blob *p, int threads, uint64_t stride,
                                 uint64_t offset, uint32_t root_max_degree, uint64_t *roots_done) {
    exec_ctx c;
    c.off = off; c.nb = nb; c.p = p; c.maxdeg = maxdeg;
    const int64_t nor = (p->root_kind == SGE_ROOT_ANY) ? 2 : 1;
    if (stride == 0) stride = 1;
    const uint32_t K = p->k, ne = p->num_enum;
    const int64_t nedge = offset < m ? (int64_t)((m - offset + stride - 1) / stride) : 0;
    const int64_t nroot = nedge * nor;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    /* the root task r -> (a, b) */
    #define ROOT_OF(r, a, b) do { \
        const uint64_t ei_ = offset + (uint64_t)((r) / nor) * stride; \
        a = eu[ei_]; b = ev[ei_]; \
        if ((p->root_kind == SGE_ROOT_ANY && ((r) % nor) == 1) || p->root_kind == SGE_ROOT_DESC) { uint32_t x_ = a; a = b; b = x_; } \
    } while (0)
    /* pass A: each root's level-2 list size and its number of work items */
    uint64_t *pre = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(nroot + 1));
    uint32_t *c2 = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nroot + 1));
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        uint32_t *buf = (uint32_t *)malloc(sizeof(uint32_t) * (c.maxdeg + 1));
        uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (c.maxdeg + 1));
        uint32_t mm[SGE_MAX_K];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t r = 0; r < nroot; ++r) {
            uint32_t a, b;
            ROOT_OF(r, a, b);
            if (root_max_degree && (off[a + 1] - off[a] > root_max_degree || off[b + 1] - off[b] > root_max_degree)) {
                c2[r] = 0xFFFFFFFFu;  /* dropped by the degree cap */
                continue;
            }
            if (ne == 2) { c2[r] = 0; continue; }
            mm[0] = a; mm[1] = b;
            c2[r] = level_candidates(&c, 2, mm, buf, tmp);
        }
        free(buf);
        free(tmp);
    }
    pre[0] = 0;
    for (int64_t r = 0; r < nroot; ++r) {
        const uint32_t n2 = c2[r];
        const uint64_t items = n2 == 0xFFFFFFFFu ? 0u : n2 <= 64 ? 1u : (n2 / 16 < 64 ? n2 / 16 : 64);
        pre[r + 1] = pre[r] + items;
    }
    const int64_t nitems = (int64_t)pre[nroot];
    uint64_t total = 0, done = 0;
#ifdef _OPENMP
#pragma omp parallel reduction(+ : total, done)
#endif
    {
        uint32_t *bufs[SGE_MAX_K + SGE_MAX_TAIL];
        for (uint32_t i = 0; i < SGE_MAX_K + SGE_MAX_TAIL; ++i) bufs[i] = (uint32_t *)malloc(sizeof(uint32_t) * (c.maxdeg + 1));
        uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (c.maxdeg + 1));
        uint32_t cnt[SGE_MAX_K], it[SGE_MAX_K], mm[SGE_MAX_K];
        uint32_t *hoist[SGE_MAX_K], hoist_n[SGE_MAX_K];
        for (uint32_t i = 0; i < SGE_MAX_K; ++i) {
            hoist[i] = NULL;
            hoist_n[i] = 0;
        }
        for (uint32_t i = ne; i < K; ++i)
            if (hoisted_level(p, i)) hoist[i] = (uint32_t *)malloc(sizeof(uint32_t) * (c.maxdeg + 1));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t q = 0; q < nitems; ++q) {
            /* the root holding item q: the last r with pre[r] <= q */
            int64_t lo = 0, hi = nroot;
            while (hi - lo > 1) { const int64_t mid = (lo + hi) / 2; if (pre[mid] <= (uint64_t)q) lo = mid; else hi = mid; }
            const int64_t r = lo;
            const uint64_t part = (uint64_t)q - pre[r], parts = pre[r + 1] - pre[r];
            uint32_t a, b;
            ROOT_OF(r, a, b);
            mm[0] = a; mm[1] = b;
            if (part == 0) ++done;
            if (ne == 2) { total += tail_count(&c, mm, bufs + SGE_MAX_K, tmp, hoist, hoist_n); continue; }
            for (uint32_t i = ne; i < K; ++i)
                if (hoist[i] && hoist_at_level(p, i) == 1) hoist_n[i] = raw_intersection(&c, i, mm, hoist[i], tmp);
            int lv = 2;
            const uint32_t n2 = level_candidates(&c, 2, mm, bufs[2], tmp);
            it[2] = (uint32_t)((uint64_t)n2 * part / parts);
            cnt[2] = (uint32_t)((uint64_t)n2 * (part + 1) / parts);
            while (lv >= 2) {
                if (it[lv] >= cnt[lv]) { --lv; continue; }
                mm[lv] = bufs[lv][it[lv]++];
                for (uint32_t i = ne; i < K; ++i)
                    if (hoist[i] && hoist_at_level(p, i) == (uint32_t)lv) hoist_n[i] = raw_intersection(&c, i, mm, hoist[i], tmp);
                if ((uint32_t)lv + 1 == ne) { total += tail_count(&c, mm, bufs + SGE_MAX_K, tmp, hoist, hoist_n); continue; }
                ++lv;
                cnt[lv] = level_candidates(&c, (uint32_t)lv, mm, bufs[lv], tmp);
                it[lv] = 0;
            }
        }
        for (uint32_t i = 0; i < SGE_MAX_K + SGE_MAX_TAIL; ++i) free(bufs[i]);
        for (uint32_t i = 0; i < SGE_MAX_K; ++i) free(hoist[i]);
        free(tmp);
    }
    #undef ROOT_OF
    free(pre);
    free(c2);
    if (roots_done) *roots_done = done;
    return total;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Lists every embedding (injective homomorphism) as k ids in pattern-vertex
 * order, by the same DFS as oracle_bruteforce_embeddings (single thread).
 * Returns the number of embeddings; rows past cap are not written. */
uint64_t oracle_list_embeddings(const uint32_t *off, const uint32_t *nb, uint32_t n, uint32_t k, uint32_t m,
                                const uint32_t *edges, uint32_t *out, uint64_t cap) {
    uint32_t adj[32] = {0};
    for (uint32_t i = 0; i < m; ++i) { adj[edges[2 * i]] |= 1u << edges[2 * i + 1]; adj[edges[2 * i + 1]] |= 1u << edges[2 * i]; }
    uint32_t order[32], seen = 0, best = 0;
    for (uint32_t u = 1; u < k; ++u) if (__builtin_popcount(adj[u]) > __builtin_popcount(adj[best])) best = u;
    order[0] = best; seen = 1u << best;
    for (uint32_t i = 1; i < k; ++i) {
        int bv = -1, bs = -1;
        for (uint32_t u = 0; u < k; ++u) {
            if ((seen >> u) & 1u) continue;
            int s = __builtin_popcount(adj[u] & seen);
            if (s > 0 && s > bs) { bs = s; bv = (int)u; }
        }
        if (bv < 0) return 0;
        order[i] = (uint32_t)bv; seen |= 1u << bv;
    }
    uint32_t back[32], first[32];
    for (uint32_t i = 0; i < k; ++i) {
        back[i] = 0;
        for (uint32_t j = 0; j < i; ++j) if (pat_edge(adj, order[i], order[j])) back[i] |= 1u << j;
        first[i] = back[i] ? (uint32_t)__builtin_ctz(back[i]) : 0;
    }
    uint64_t total = 0;
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t mm[32], it[32];
        int lv = 1;
        mm[0] = r;
        it[1] = off[mm[first[1]]];
        while (lv >= 1) {
            uint32_t p = mm[first[lv]];
            if (it[lv] >= off[p + 1]) { --lv; continue; }
            uint32_t x = nb[it[lv]++];
            int ok = 1;
            for (int j = 0; j < lv && ok; ++j) if (mm[j] == x) ok = 0;
            for (uint32_t msk = back[lv] & ~(1u << first[lv]); msk && ok; msk &= msk - 1)
                if (!has_edge(off, nb, mm[__builtin_ctz(msk)], x)) ok = 0;
            if (!ok) continue;
            mm[lv] = x;
            if (lv + 1 == (int)k) {
                if (total < cap)
                    for (uint32_t i = 0; i < k; ++i) out[total * k + order[i]] = mm[i];
                ++total;
                continue;
            }
            ++lv;
            it[lv] = off[mm[first[lv]]];
        }
    }
    return total;
}

/* ---------------------------------------------------------------- 4 ----
 * Seeded workloads without the library.  The library's seeded generators
 * (subgraph-enumeration_gb300/csrc/generators.cpp: sge_gen_rmat,
 * sge_gen_chung_lu) and its symmetric CSR build (sge_csr_from_edges) are
 * restated here, on the same splitmix64 streams and integer decisions, so a
 * CPU-only process (the timed CPU arm of bench.py) builds the very same data
 * graphs while loading nothing but this file's library.  tests/ pin the two
 * against each other. */

static uint64_t o_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

typedef struct { uint64_t s; } o_rng;
static void o_rng_init(o_rng *r, uint64_t seed) { r->s = o_splitmix64(seed ^ 0x5347454E5347454Eull); }
static uint64_t o_rng_next(o_rng *r) {
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static uint64_t o_rng_below(o_rng *r, uint64_t n) { return (uint64_t)(((unsigned __int128)o_rng_next(r) * n) >> 64); }

/* Set of distinct 64-bit edge keys (open addressing; ~0 marks a free slot),
 * remembering insertion order. */
typedef struct { uint64_t *slot, mask, *order, n; } o_keyset;
static int o_keyset_init(o_keyset *s, uint64_t cap) {
    uint64_t sz = 1;
    while (sz < 2 * cap + 16) sz <<= 1;
    s->slot = (uint64_t *)malloc(sizeof(uint64_t) * sz);
    s->order = (uint64_t *)malloc(sizeof(uint64_t) * (cap + 1));
    if (!s->slot || !s->order) { free(s->slot); free(s->order); return 0; }
    memset(s->slot, 0xFF, sizeof(uint64_t) * sz);
    s->mask = sz - 1;
    s->n = 0;
    return 1;
}
static void o_keyset_add(o_keyset *s, uint64_t key) {
    uint64_t h = (key * 0x9E3779B97F4A7C15ull) >> 20;
    for (;; ++h) {
        uint64_t *p = &s->slot[h & s->mask];
        if (*p == key) return;
        if (*p == ~0ull) { *p = key; s->order[s->n++] = key; return; }
    }
}

/* LSD radix sort of 64-bit keys (16-bit digits; digits that never vary are skipped). */
static void o_sort_u64(uint64_t *a, uint64_t n) {
    if (n < 2) return;
    uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * n);
    uint64_t *cnt = (uint64_t *)malloc(sizeof(uint64_t) * 65536);
    uint64_t *src = a, *dst = tmp;
    for (int sh = 0; sh < 64; sh += 16) {
        memset(cnt, 0, sizeof(uint64_t) * 65536);
        for (uint64_t i = 0; i < n; ++i) cnt[(src[i] >> sh) & 0xFFFF]++;
        if (cnt[(src[0] >> sh) & 0xFFFF] == n) continue;
        uint64_t acc = 0;
        for (int d = 0; d < 65536; ++d) { uint64_t c = cnt[d]; cnt[d] = acc; acc += c; }
        for (uint64_t i = 0; i < n; ++i) dst[cnt[(src[i] >> sh) & 0xFFFF]++] = src[i];
        uint64_t *t = src; src = dst; dst = t;
    }
    if (src != a) memcpy(a, src, sizeof(uint64_t) * n);
    free(tmp);
    free(cnt);
}

/* One R-MAT draw as generators.cpp's rmat_draw: `scale` quadrant choices,
 * two per 64-bit word; ~0 for a self-loop, else (min << 32) | max. */
static uint64_t o_rmat_draw(uint64_t seed, uint64_t idx, uint32_t scale, uint32_t ta, uint32_t tab, uint32_t tabc) {
    uint32_t u = 0, v = 0;
    uint64_t word = 0;
    for (uint32_t bit = 0; bit < scale; ++bit) {
        uint32_t r;
        if ((bit & 1) == 0) {
            word = o_splitmix64(seed * 0x100000001B3ull + idx * 64 + bit);
            r = (uint32_t)word;
        } else {
            r = (uint32_t)(word >> 32);
        }
        uint32_t ub, vb;
        if (r < ta) { ub = 0; vb = 0; }
        else if (r < tab) { ub = 0; vb = 1; }
        else if (r < tabc) { ub = 1; vb = 0; }
        else { ub = 1; vb = 1; }
        u = (u << 1) | ub;
        v = (v << 1) | vb;
    }
    if (u == v) return ~0ull;
    if (u > v) { uint32_t t = u; u = v; v = t; }
    return ((uint64_t)u << 32) | v;
}

static uint32_t o_ppm_threshold(uint64_t ppm) {
    uint64_t t = (ppm << 32) / 1000000u;
    return t > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)t;
}

/* sge_gen_rmat: the m distinct edges whose first draw comes earliest in the
 * draw stream (the library reaches the same set by drawing in rounds), as
 * sorted u<v pairs.  *edges is malloc'ed (2·m_out uint32). */
int oracle_gen_rmat(uint32_t scale, uint64_t m, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm, uint64_t seed,
                    uint32_t **edges, uint64_t *m_out) {
    if (scale < 1 || scale > 31) return 0;
    const uint32_t ta = o_ppm_threshold(a_ppm), tab = o_ppm_threshold((uint64_t)a_ppm + b_ppm),
                   tabc = o_ppm_threshold((uint64_t)a_ppm + b_ppm + c_ppm);
    o_keyset s;
    if (!o_keyset_init(&s, m)) return 0;
    const uint64_t CH = 1u << 22;
    uint64_t *buf = (uint64_t *)malloc(sizeof(uint64_t) * CH);
    for (uint64_t base = 0; s.n < m && base < (1ull << 34); base += CH) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < (int64_t)CH; ++i) buf[i] = o_rmat_draw(seed, base + (uint64_t)i, scale, ta, tab, tabc);
        for (uint64_t i = 0; i < CH && s.n < m; ++i)
            if (buf[i] != ~0ull) o_keyset_add(&s, buf[i]);
    }
    free(buf);
    free(s.slot);
    o_sort_u64(s.order, s.n);
    uint32_t *e = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (s.n ? s.n : 1));
    for (uint64_t i = 0; i < s.n; ++i) { e[2 * i] = (uint32_t)(s.order[i] >> 32); e[2 * i + 1] = (uint32_t)s.order[i]; }
    free(s.order);
    *edges = e;
    *m_out = s.n;
    return 1;
}

/* sge_gen_chung_lu: integer-rounded weights ∝ (i+1)^(-1/(gamma-1)) scaled to
 * mean degree 2m/n and capped at max_deg; draws until m distinct edges. */
int oracle_gen_chung_lu(uint32_t n, uint64_t m, uint32_t gamma_milli, uint32_t max_deg, uint64_t seed,
                        uint32_t **edges, uint64_t *m_out) {
    if (n < 2 || gamma_milli <= 1000) return 0;
    const double alpha = 1000.0 / ((double)gamma_milli - 1000.0);
    double *w = (double *)malloc(sizeof(double) * n);
    double sum = 0;
    for (uint32_t i = 0; i < n; ++i) { w[i] = pow((double)(i + 1), -alpha); sum += w[i]; }
    const double target = 2.0 * (double)m;
    const double cap = max_deg ? (double)max_deg : (double)(n - 1);
    double scale = target / sum;
    for (int it = 0; it < 8; ++it) {
        double capped = 0, free_sum = 0;
        for (uint32_t i = 0; i < n; ++i) {
            double x = w[i] * scale;
            if (x >= cap) capped += cap; else free_sum += w[i];
        }
        if (free_sum <= 0) break;
        scale = (target - capped) / free_sum;
    }
    uint64_t *cdf = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    cdf[0] = 0;
    for (uint32_t i = 0; i < n; ++i) {
        double x = w[i] * scale;
        if (x > cap) x = cap;
        uint64_t iw = (uint64_t)llround(x * 256.0);
        if (iw == 0) iw = 1;
        cdf[i + 1] = cdf[i] + iw;
    }
    free(w);
    const uint64_t total = cdf[n];
    o_rng rng;
    o_rng_init(&rng, seed);
    o_keyset s;
    if (!o_keyset_init(&s, m)) { free(cdf); return 0; }
    uint64_t guard = 0;
    while (s.n < m) {
        if (++guard > 200 * m + 100000) { free(cdf); free(s.slot); free(s.order); return 0; }
        uint32_t uv[2];
        for (int q = 0; q < 2; ++q) {
            uint64_t r = o_rng_below(&rng, total);
            uint32_t lo = 0, hi = n + 1;  /* upper_bound over cdf[0..n] */
            while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (cdf[mid] <= r) lo = mid + 1; else hi = mid; }
            uv[q] = lo - 1;
        }
        uint32_t u = uv[0], v = uv[1];
        if (u == v) continue;
        if (u > v) { uint32_t t = u; u = v; v = t; }
        o_keyset_add(&s, ((uint64_t)u << 32) | v);
    }
    free(cdf);
    free(s.slot);
    o_sort_u64(s.order, s.n);
    uint32_t *e = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (s.n ? s.n : 1));
    for (uint64_t i = 0; i < s.n; ++i) { e[2 * i] = (uint32_t)(s.order[i] >> 32); e[2 * i + 1] = (uint32_t)s.order[i]; }
    free(s.order);
    *edges = e;
    *m_out = s.n;
    return 1;
}

/* Symmetric CSR of m sorted, distinct u<v edges (relation/graph.cpp:143-173,
 * Graph::addDirectedEdges).  In (u, v) order, every vertex receives its
 * smaller neighbours before its larger ones, each in increasing order, so the
 * lists come out sorted.  off: n+1, nb: 2m (caller-allocated). */
void oracle_csr_from_sorted_edges(const uint32_t *edges, uint64_t m, uint32_t n, uint32_t *off, uint32_t *nb) {
    memset(off, 0, sizeof(uint32_t) * ((size_t)n + 1));
    for (uint64_t i = 0; i < m; ++i) { off[edges[2 * i] + 1]++; off[edges[2 * i + 1] + 1]++; }
    for (uint32_t v = 0; v < n; ++v) off[v + 1] += off[v];
    uint32_t *pos = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    memcpy(pos, off, sizeof(uint32_t) * ((size_t)n + 1));
    for (uint64_t i = 0; i < m; ++i) {
        const uint32_t u = edges[2 * i], v = edges[2 * i + 1];
        nb[pos[u]++] = v;
        nb[pos[v]++] = u;
    }
    free(pos);
}

void oracle_free(void *p) { free(p); }

/* ---------------------------------------------------------------- 5 ---- */
/* Algorithmic bytes (the instrumented device kernel's alg_bytes counter) of a
 * WCOJ plan with two enumerated levels, the root edge and its leaf, computed
 * on the CPU from the counter's definition so the device figure can be
 * checked.  The definition:
 *  - root tasks t = 0.. (undirected edge offset + (t/2)·stride, t odd the
 *    reversed orientation, for an unordered root; edge offset + t·stride
 *    otherwise) are taken in groups of 32 in task order, roots the degree cap
 *    drops removed from their group;
 *  - a tail level counted with a scan scans, for every root of the group, the
 *    same one of its lists: the one with the least Σ_roots len × (Σ of the
 *    other lists' probe costs + 1), the first on ties, where a list's probe
 *    cost is 1 for a list of at least hub_min entries (a hub bitmap) and
 *    2 + ⌊log2(len+1)⌋ otherwise.  A root then costs 4 B per element of the
 *    scanned list inside its bounds, plus for each other list 4 B per probe
 *    through a hub bitmap, or the whole list as a merge consumes it
 *    (8 + 4·len);
 *  - a tail level with a single list is counted directly (range size minus
 *    the matched vertices inside it): 4·(2 + |check|)·⌊log2(len'+1)⌋ with len'
 *    the list inside the bounds;
 *  - inclusion–exclusion passes go levels with several lists first, then
 *    single-list levels (each group in tail order); every pass but the last
 *    scans, the last one counts directly when its level has a single list.
 * Returns UINT64_MAX for any other plan shape. */
static uint32_t flog2p1(uint32_t len) {
    uint64_t x = (uint64_t)len + 1;
    uint32_t r = 0;
    while (x >>= 1) ++r;
    return r;
}

uint64_t oracle_alg_bytes_root_leaf(const uint32_t *off, const uint32_t *nb, uint32_t n, const sge_plan_blob *p,
                                    uint64_t stride, uint64_t offset, uint32_t root_max_degree, uint32_t hub_min) {
    if (p->num_enum != 2 || p->join_style != SGE_JOIN_WCOJ || p->tail_len == 0 || p->tail_len > SGE_MAX_TAIL)
        return UINT64_MAX;
    uint32_t *eu, *ev, maxdeg;
    const uint64_t m = root_edges(off, nb, n, &eu, &ev, &maxdeg);
    const uint64_t st = stride > 1 ? stride : 1, o0 = stride > 1 ? offset : 0;
    const uint64_t nedges = m > o0 ? (m - o0 + st - 1) / st : 0;
    const uint64_t ntasks = p->root_kind == SGE_ROOT_ANY ? 2 * nedges : nedges;
    const uint32_t T = p->tail_len;
    const uint32_t passes = p->tail_mode == SGE_TAIL_IEP ? T : 1;
    uint32_t ord[SGE_MAX_TAIL], no = 0;
    for (uint32_t pass = 0; pass < 2; ++pass)  /* several lists first, then one */
        for (uint32_t t = 0; t < passes; ++t)
            if ((__builtin_popcount(p->parents[2 + t]) == 1) == (pass == 1)) ord[no++] = t;
    uint64_t total = 0;
    for (uint64_t t0 = 0; t0 < ntasks; t0 += 32) {
        uint32_t cm[32][2], nc = 0;
        const uint64_t t1 = t0 + 32 < ntasks ? t0 + 32 : ntasks;
        for (uint64_t t = t0; t < t1; ++t) {
            uint32_t u, v;
            if (p->root_kind == SGE_ROOT_ANY) {
                const uint64_t e = o0 + (t >> 1) * st;
                u = eu[e]; v = ev[e];
                if (t & 1) { uint32_t x = u; u = v; v = x; }
            } else {
                const uint64_t e = o0 + t * st;
                u = eu[e]; v = ev[e];
                if (p->root_kind == SGE_ROOT_DESC) { uint32_t x = u; u = v; v = x; }
            }
            if (root_max_degree && (off[u + 1] - off[u] > root_max_degree || off[v + 1] - off[v] > root_max_degree))
                continue;
            cm[nc][0] = u; cm[nc][1] = v; ++nc;
        }
        for (uint32_t s = 0; s < passes; ++s) {
            const uint32_t i = 2 + ord[s];
            const uint32_t par = p->parents[i], nsrc = (uint32_t)__builtin_popcount(par);
            const int direct = (p->tail_mode != SGE_TAIL_IEP || s + 1 == T) && nsrc == 1;
            uint32_t slot[2], ns = 0;
            for (uint32_t j = 0; j < 2; ++j) if ((par >> j) & 1u) slot[ns++] = j;
            /* each root's lists and bounds */
            uint32_t len[32][2], trimmed[32][2];
            for (uint32_t l = 0; l < nc; ++l) {
                uint32_t lo = 0, hi = 0xFFFFFFFFu;
                for (uint32_t j = 0; j < 2; ++j) {
                    if ((p->lower[i] >> j) & 1u) lo = cm[l][j] > lo ? cm[l][j] : lo;
                    if ((p->upper[i] >> j) & 1u) hi = cm[l][j] < hi ? cm[l][j] : hi;
                }
                for (uint32_t q = 0; q < ns; ++q) {
                    const uint32_t v = cm[l][slot[q]];
                    const uint32_t *a = nb + off[v];
                    const uint32_t la = off[v + 1] - off[v];
                    uint32_t c = 0;
                    for (uint32_t e = 0; e < la; ++e)
                        c += (!p->lower[i] || a[e] > lo) && (!p->upper[i] || a[e] < hi);
                    len[l][q] = la;
                    trimmed[l][q] = c;
                }
            }
            if (direct) {
                for (uint32_t l = 0; l < nc; ++l)
                    total += 4ull * (2u + (uint32_t)__builtin_popcount(p->check[i])) * flog2p1(trimmed[l][0]);
                continue;
            }
            uint32_t bq = 0;
            unsigned long long best = ~0ull;
            for (uint32_t q = 0; q < ns; ++q) {
                unsigned long long cost = 0;
                for (uint32_t l = 0; l < nc; ++l) {
                    unsigned long long allp = 0, own = 0;
                    for (uint32_t r = 0; r < ns; ++r) {
                        const unsigned long long pc = len[l][r] >= hub_min ? 1u : 2u + flog2p1(len[l][r]);
                        allp += pc;
                        if (r == q) own = pc;
                    }
                    cost += (unsigned long long)len[l][q] * (allp - own + 1);
                }
                if (cost < best) { best = cost; bq = q; }
            }
            for (uint32_t l = 0; l < nc; ++l) {
                const uint64_t blen = trimmed[l][bq];
                total += 4ull * blen;
                for (uint32_t q = 0; q < ns; ++q)
                    if (q != bq) total += len[l][q] >= hub_min ? 4ull * blen : 8ull + 4ull * len[l][q];
            }
        }
    }
    free(eu);
    free(ev);
    return total;
}
