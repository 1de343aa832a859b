// Host planner: pattern → sge_plan_blob.
//
// Stands in for the reference's planning half (main.cpp:60-69): optCostPlan
// (plan/optimizer.cpp:217-300), HyperTree::selectSymmetry / setSymmetry
// (plan/decomposition.cpp:621-868), buildTraverseUnlabeled (:982-1259) and
// refineIntersectionInfo (:3031-3181).  Its output carries the same facts the
// reference's join reads: a matching order, each level's parents (the lists to
// intersect, attributesBefore), symmetry-breaking bounds (largerAttrs /
// smallerAttrs), candidate reuse (candidatesBefore), and how the last levels
// are counted instead of enumerated (symmLastLevel / groups with IEP).
//
// Count semantics follow the reference exactly:
//  - the reference runs a single-bag plan only when the pattern has no
//    degree<2 periphery (PatternGraph::buildCorePeripheral, relation/graph.cpp:1231-1305;
//    peripheral vertices become extra edge bags, HyperTree::addPeripheral,
//    plan/decomposition.cpp:1318+) and every minimal-width decomposition of
//    the core is one bag, i.e. the pattern is a clique (all_td.cpp:483-691
//    keeps only the smallest maximum bag size).  buildTraverseUnlabeled
//    returns before setSymmetry for one-bag plans (decomposition.cpp:983-986),
//    so those count embeddings; every other plan counts instances.
//  - here both are computed as instances (restrictions from the automorphism
//    group's stabilizer chain keep one embedding per class) times
//    count_multiplier = |Aut| for single-bag patterns, 1 otherwise.
#include "common.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstddef>
#include <vector>

using namespace sge;

// Implemented in engine.cu: the statistics a device graph keeps (host copy).
namespace sge {
bool graph_stats(const sge_graph *g, sge_graph_stats *out);
double sample_clustering(const uint32_t *off, const uint32_t *nb, uint32_t n);
}

namespace {

typedef std::array<uint8_t, SGE_MAX_K> Perm;

struct Pattern {
    uint32_t k = 0, m = 0;
    uint32_t adj[SGE_MAX_K] = {};
    uint32_t label[SGE_MAX_K] = {};  // vertex labels (all 0 when unlabeled)
    bool labeled = false;
    int deg(uint32_t u) const { return __builtin_popcount(adj[u]); }
    bool edge(uint32_t a, uint32_t b) const { return (adj[a] >> b) & 1u; }
};

sge_status make_pattern(uint32_t k, uint32_t m, const uint32_t *edges, Pattern &p) {
    if (k < 3 || k > SGE_MAX_K) return fail(SGE_UNSUPPORTED, "pattern has %u vertices (executor supports 3..%u)", k, SGE_MAX_K);
    if (!edges && m) return fail(SGE_BAD_INPUT, "pattern edges are null");
    p.k = k;
    p.m = 0;
    for (uint32_t i = 0; i < m; ++i) {
        uint32_t a = edges[2 * i], b = edges[2 * i + 1];
        if (a >= k || b >= k || a == b) return fail(SGE_BAD_INPUT, "pattern edge (%u,%u) invalid for k=%u", a, b, k);
        if (p.edge(a, b)) return fail(SGE_BAD_INPUT, "pattern edge (%u,%u) repeated", a, b);
        p.adj[a] |= 1u << b;
        p.adj[b] |= 1u << a;
        p.m++;
    }
    // connectivity
    uint32_t seen = 1, frontier = 1;
    while (frontier) {
        uint32_t nf = 0;
        for (uint32_t u = 0; u < k; ++u)
            if ((frontier >> u) & 1u) nf |= p.adj[u];
        nf &= ~seen;
        seen |= nf;
        frontier = nf;
    }
    if (seen != ((k == 32) ? 0xFFFFFFFFu : ((1u << k) - 1)))
        return fail(SGE_UNSUPPORTED, "pattern is disconnected (the executor needs a connected pattern)");
    return SGE_OK;
}

// All automorphisms by adjacency-preserving backtracking.
bool automorphisms(const Pattern &p, std::vector<Perm> &out, size_t limit) {
    out.clear();
    Perm map{};
    uint32_t used = 0;
    std::vector<uint32_t> cand_stack(p.k, 0);
    int i = 0;
    cand_stack[0] = 0;
    // iterative DFS: cand_stack[i] = next candidate image to try for vertex i
    while (i >= 0) {
        if (i == (int)p.k) {
            out.push_back(map);
            if (out.size() > limit) return false;
            --i;
            if (i >= 0) used &= ~(1u << map[i]);
            continue;
        }
        bool placed = false;
        for (uint32_t c = cand_stack[i]; c < p.k; ++c) {
            if ((used >> c) & 1u) continue;
            if (p.deg(c) != p.deg(i) || p.label[c] != p.label[i]) continue;
            bool ok = true;
            for (int j = 0; j < i && ok; ++j)
                if (p.edge(i, j) != p.edge(c, map[j])) ok = false;
            if (!ok) continue;
            map[i] = (uint8_t)c;
            used |= 1u << c;
            cand_stack[i] = c + 1;
            ++i;
            if (i < (int)p.k) cand_stack[i] = 0;
            placed = true;
            break;
        }
        if (!placed) {
            --i;
            if (i >= 0) used &= ~(1u << map[i]);
        }
    }
    return true;
}

bool is_single_bag(const Pattern &p) {
    // periphery: iterative peeling of degree<2 vertices (the 2-core)
    int deg[SGE_MAX_K];
    uint32_t alive = (1u << p.k) - 1;
    for (uint32_t u = 0; u < p.k; ++u) deg[u] = p.deg(u);
    bool changed = true;
    while (changed) {
        changed = false;
        for (uint32_t u = 0; u < p.k; ++u)
            if (((alive >> u) & 1u) && deg[u] < 2) {
                alive &= ~(1u << u);
                for (uint32_t w = 0; w < p.k; ++w)
                    if (((alive >> w) & 1u) && p.edge(u, w)) deg[w]--;
                changed = true;
            }
    }
    if (alive != (1u << p.k) - 1) return false;
    return p.m == p.k * (p.k - 1) / 2;
}

// Symmetry-breaking restrictions from the stabilizer chain along `seq`
// (pattern vertices): for the first vertex v of seq with a non-trivial orbit
// under the current group, require m[v] < m[u] for every other u in the orbit,
// then restrict the group to the stabilizer of v.  Exactly one embedding of
// every automorphism class satisfies the result (the role of selectSymmetry /
// setSymmetry, plan/decomposition.cpp:621-868).
std::vector<std::pair<uint32_t, uint32_t>> restrictions(const Pattern &p, const std::vector<Perm> &aut,
                                                        const uint32_t *seq) {
    std::vector<std::pair<uint32_t, uint32_t>> r;
    std::vector<const Perm *> group;
    for (auto &g : aut) group.push_back(&g);
    for (uint32_t i = 0; i < p.k && group.size() > 1; ++i) {
        uint32_t v = seq[i];
        uint32_t orbit = 0;
        for (auto *g : group) orbit |= 1u << (*g)[v];
        for (uint32_t u = 0; u < p.k; ++u)
            if (u != v && ((orbit >> u) & 1u)) r.emplace_back(v, u);
        std::vector<const Perm *> stab;
        for (auto *g : group)
            if ((*g)[v] == v) stab.push_back(g);
        group.swap(stab);
    }
    return r;
}

struct Moments {
    double M[SGE_MAX_K + 2];
    double n, nnz;
    double clustering = 0.05;
    bool have = false;
};

// Expected homomorphism count of the pattern induced by `mask` (over pattern
// vertices) in a Chung-Lu-like random graph with the data graph's degrees:
// Π_v M_{deg(v)} / W^{|E|}, W = Σ deg = 2m.  Used only to rank plans.
double expected_hom(const Pattern &p, uint32_t mask, const Moments &mo) {
    double lg = 0;
    int e2 = 0;
    for (uint32_t u = 0; u < p.k; ++u)
        if ((mask >> u) & 1u) {
            int d = __builtin_popcount(p.adj[u] & mask);
            e2 += d;
            lg += std::log(std::max(mo.M[d], 1e-300));
        }
    lg -= (e2 / 2) * std::log(std::max(mo.nnz, 1.0));
    return std::exp(lg);
}

struct Candidate {
    sge_plan_blob blob;
    double cost;
};

void set_partitions(uint32_t T, sge_plan_blob &b) {
    // restricted growth strings a[0]=0, a[i] <= 1+max(a[0..i-1])
    uint32_t a[SGE_MAX_TAIL] = {0};
    b.num_partitions = 0;
    while (true) {
        uint32_t nb = 0;
        for (uint32_t i = 0; i < T; ++i) nb = std::max(nb, a[i] + 1);
        uint32_t blocks[SGE_MAX_TAIL] = {0};
        for (uint32_t i = 0; i < T; ++i) blocks[a[i]] |= 1u << i;
        int64_t coef = 1;
        for (uint32_t x = 0; x < nb; ++x) {
            int s = __builtin_popcount(blocks[x]);
            int64_t f = 1;
            for (int t = 2; t < s; ++t) f *= t;  // (s-1)!
            coef *= ((s - 1) % 2 ? -1 : 1) * f;
        }
        uint32_t pi = b.num_partitions++;
        b.part_coef[pi] = (int32_t)coef;
        b.part_nblocks[pi] = nb;
        for (uint32_t x = 0; x < SGE_MAX_TAIL; ++x) b.part_block[pi][x] = x < nb ? blocks[x] : 0;
        // next RGS
        int i = (int)T - 1;
        while (i > 0) {
            uint32_t mx = 0;
            for (int j = 0; j < i; ++j) mx = std::max(mx, a[j]);
            if (a[i] <= mx) { a[i]++; for (uint32_t j = i + 1; j < T; ++j) a[j] = 0; break; }
            --i;
        }
        if (i <= 0) break;
    }
}

// Builds the blob for a fixed order, restriction set and tail length; returns
// false if the tail is not countable by one of the three modes.
bool build_blob(const Pattern &p, const uint32_t *order, const std::vector<std::pair<uint32_t, uint32_t>> &restr,
                uint32_t T, bool use_iep, uint32_t join_style, uint64_t aut_size, bool single_bag,
                sge_plan_blob &b) {
    const uint32_t k = p.k;
    memset(&b, 0, sizeof b);
    b.magic = SGE_PLAN_MAGIC;
    b.abi_version = SGE_ABI_VERSION;
    b.k = k;
    b.num_enum = k - T;
    b.tail_len = T;
    b.join_style = join_style;
    b.aut_size = aut_size;
    b.single_bag = single_bag ? 1u : 0u;
    b.labeled = p.labeled ? 1u : 0u;
    b.count_multiplier = single_bag ? aut_size : 1;
    b.num_restrictions = (uint32_t)restr.size();
    uint32_t lvl[SGE_MAX_K];
    for (uint32_t i = 0; i < k; ++i) { b.order[i] = order[i]; lvl[order[i]] = i; }
    for (uint32_t i = 0; i < k; ++i) b.base[i] = -1;
    for (uint32_t i = 0; i < k; ++i)
        for (uint32_t j = 0; j < i; ++j)
            if (p.edge(order[i], order[j])) b.parents[i] |= 1u << j;
    for (auto &r : restr) {  // m[a] < m[b]
        uint32_t la = lvl[r.first], lb = lvl[r.second];
        if (la < lb) b.lower[lb] |= 1u << la;  // at b's level: x > m[a]
        else b.upper[la] |= 1u << lb;          // at a's level: x < m[b]
    }
    const uint32_t ne = b.num_enum;
    if (ne < 2 || T < 1 || T > SGE_MAX_TAIL) return false;
    if (!((b.parents[1] >> 0) & 1u)) return false;  // root must be an edge
    for (uint32_t i = 1; i < k; ++i)
        if (b.parents[i] == 0) return false;  // connected order
    const uint32_t tail_mask_lv = ((1u << k) - 1) & ~((1u << ne) - 1);
    // tail: pairwise non-adjacent
    for (uint32_t i = ne; i < k; ++i)
        if (b.parents[i] & tail_mask_lv) return false;
    // restrictions among tail levels
    uint32_t intra = 0;
    for (uint32_t i = ne; i < k; ++i) intra |= (b.lower[i] | b.upper[i]) & tail_mask_lv;
    if (T == 1) {
        b.tail_mode = SGE_TAIL_SINGLE;
    } else {
        if (!use_iep) return false;
        if (intra == 0) {
            b.tail_mode = SGE_TAIL_IEP;
            set_partitions(T, b);
        } else {
            // CHOOSE: identical parents and identical non-tail bounds, and the
            // intra-tail restrictions totally order the tail.
            for (uint32_t i = ne + 1; i < k; ++i) {
                if (b.parents[i] != b.parents[ne]) return false;
                if (p.label[order[i]] != p.label[order[ne]]) return false;  // one candidate set
                if ((b.lower[i] & ~tail_mask_lv) != (b.lower[ne] & ~tail_mask_lv)) return false;
                if ((b.upper[i] & ~tail_mask_lv) != (b.upper[ne] & ~tail_mask_lv)) return false;
            }
            // transitive closure over tail positions
            bool less[SGE_MAX_TAIL][SGE_MAX_TAIL] = {};
            for (uint32_t i = ne; i < k; ++i)
                for (uint32_t j = ne; j < k; ++j) {
                    if ((b.lower[i] >> j) & 1u) less[j - ne][i - ne] = true;  // m[j] < m[i]
                    if ((b.upper[i] >> j) & 1u) less[i - ne][j - ne] = true;  // m[i] < m[j]
                }
            for (uint32_t x = 0; x < T; ++x)
                for (uint32_t a = 0; a < T; ++a)
                    for (uint32_t c = 0; c < T; ++c)
                        if (less[a][x] && less[x][c]) less[a][c] = true;
            for (uint32_t a = 0; a < T; ++a)
                for (uint32_t c = a + 1; c < T; ++c)
                    if (!(less[a][c] ^ less[c][a])) return false;
            b.tail_mode = SGE_TAIL_CHOOSE;
        }
        // intra-tail restrictions are accounted for by the counting mode
        for (uint32_t i = ne; i < k; ++i) {
            b.lower[i] &= ~tail_mask_lv;
            b.upper[i] &= ~tail_mask_lv;
        }
    }
    b.root_kind = ((b.lower[1] & 1u) ? SGE_ROOT_ASC : (b.upper[1] & 1u) ? 2u : SGE_ROOT_ANY);
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t below = (i < ne) ? ((1u << i) - 1) : ((1u << ne) - 1);
        b.check[i] = below & ~(b.parents[i] | b.lower[i] | b.upper[i]);
        b.first_parent[i] = b.parents[i] ? (uint32_t)__builtin_ctz(b.parents[i]) : 0;
        b.rest[i] = b.parents[i];
    }
    // candidate reuse (candidatesBefore): a stored enumerated level l >= 2
    // whose parents are a subset of level i's (the executor keeps a reused
    // level's list free of its bounds, so only the parents matter)
    for (uint32_t i = 3; i < k; ++i) {
        int best = -1, best_pc = 0;
        uint32_t lim = std::min(i, ne);
        // a tail level whose parents all precede the last enumerated level is
        // computed right after its last parent (hoisted): reuse only levels built by then
        const uint32_t lastp = 31u - (uint32_t)__builtin_clz(b.parents[i]);
        if (i >= ne && __builtin_popcount(b.parents[i]) >= 2 && lastp + 1 < ne) lim = std::min(lim, std::max(lastp, 1u) + 1);
        for (uint32_t l = 2; l < lim; ++l) {
            if ((b.parents[l] & ~b.parents[i]) != 0) continue;
            int pc = __builtin_popcount(b.parents[l]);
            if (pc >= 2 && pc >= best_pc) { best = (int)l; best_pc = pc; }
        }
        if (best >= 0) {
            b.base[i] = best;
            b.rest[i] = b.parents[i] & ~b.parents[best];
        }
    }
    return true;
}

// Cost model (ranks plans; the reference's counterpart is computeOrderCost,
// plan/optimizer.cpp:319-438).  Work is counted in list elements touched:
// each enumerated level multiplies the number of partial matches by its
// expected candidate-list size, which for a level with r parents is
// L·c^(r-1)/2^b (L = size-biased degree M2/M1, c = the graph's sampled
// clustering coefficient, b = symmetry bounds at that level); building a level
// costs its base list times one binary search per other parent list.
double plan_cost(const Pattern &p, const sge_plan_blob &b, const Moments &mo) {
    (void)p;
    const uint32_t k = b.k, ne = b.num_enum;
    const double L = std::max(1.0, mo.M[2] / std::max(mo.M[1], 1.0));
    const double c = std::min(0.9, std::max(1e-4, mo.clustering));
    const double lg = std::log2(L + 1.0);
    double cand[SGE_MAX_K];
    auto est_cand = [&](uint32_t i) {
        int r = __builtin_popcount(b.parents[i]);
        int nb = __builtin_popcount(b.lower[i] | b.upper[i]);
        return std::max(1e-3, L * std::pow(c, r - 1) / std::pow(2.0, nb));
    };
    // lists whose intersection gives level i (a reused stored list counts as one)
    auto lists = [&](uint32_t i) {
        return b.base[i] >= 0 ? 1 + __builtin_popcount(b.rest[i]) : __builtin_popcount(b.parents[i]);
    };
    auto full_len = [&](uint32_t l) { return std::max(1e-3, L * std::pow(c, __builtin_popcount(b.parents[l]) - 1)); };
    auto base_len = [&](uint32_t i) { return b.base[i] >= 0 ? std::min(full_len(b.base[i]), L) : L; };
    // the executor runs the last two enumerated levels as one flattened step
    // when it can (the pair step): its per-candidate overhead is amortised
    // over 32 candidates
    const ExecShape xs = exec_shape(b);
    const bool pair = xs.pair;
    double N = mo.nnz / ((b.root_kind == SGE_ROOT_ANY) ? 1.0 : 2.0);
    double cost = N * 4.0;
    double Nat[SGE_MAX_K];
    Nat[1] = N;
    for (uint32_t i = 2; i < ne; ++i) {
        cand[i] = est_cand(i);
        const double work = lists(i) > 1 ? base_len(i) * (1.0 + (lists(i) - 1) * lg) : lg;
        cost += N * (work + ((pair && i + 1 == ne) ? 4.0 : 16.0));
        N *= cand[i];
        Nat[i] = N;
        cost += N * (i + 1 == ne ? 4.0 : 8.0);  // last-level candidates go to the leaf in batches
    }
    for (uint32_t i = ne; i < k; ++i) {
        const uint32_t par = b.parents[i];
        const uint32_t last = 31u - (uint32_t)__builtin_clz(par);
        if (__builtin_popcount(par) >= 2 && last + 1 < ne) {
            const bool reuse = b.base[i] >= 0 && (uint32_t)b.base[i] <= std::max(last, 1u);
            const double work = reuse ? base_len(i) * (1.0 + __builtin_popcount(b.rest[i]) * lg)
                                      : L * (1.0 + (__builtin_popcount(par) - 1) * lg);
            cost += Nat[std::max(last, 1u)] * (work + 16.0);
        }
    }
    for (uint32_t i = ne; i < k; ++i) cand[i] = est_cand(i);
    // a tail level whose parents precede the last enumerated level is hoisted:
    // its intersection is computed once per match of its last parent
    // (WCOJ), or is the running list (exploration) — one list at the leaf
    auto hoisted = [&](uint32_t i) {
        const uint32_t par = b.parents[i];
        return __builtin_popcount(par) >= 2 && (31u - (uint32_t)__builtin_clz(par)) + 1 < ne;
    };
    auto leaf_lists = [&](uint32_t i) { return hoisted(i) ? 1 : lists(i); };
    double leaf = 0;
    const uint32_t yb = 1u << (ne - 1);
    if (xs.pair_direct && leaf_lists(ne) == 1) {
        // counted inline per pair: the candidate's count minus the pair's own vertex
        leaf = 1.0 + ((b.check[ne] & yb) ? 1.0 : 0.0);
    } else if (b.tail_mode != SGE_TAIL_IEP && leaf_lists(ne) == 1) {
        // a single list: range size minus matched vertices inside, by binary search
        leaf = 4.0 + 2.0 * __builtin_popcount(b.check[ne]) * lg;
    } else {
        const uint32_t passes = (b.tail_mode == SGE_TAIL_IEP) ? k - ne : 1u;
        for (uint32_t t = 0; t < passes; ++t) {
            const uint32_t i = ne + t;
            double probes = (leaf_lists(i) - 1) * lg;
            for (uint32_t u = i + 1; u < k && b.tail_mode == SGE_TAIL_IEP; ++u) probes += leaf_lists(u) * lg;
            const double bl = hoisted(i) ? std::max(1e-3, L * std::pow(c, __builtin_popcount(b.parents[i]) - 1))
                                         : base_len(i);
            leaf += bl * (1.0 + probes) + 4.0;
        }
    }
    cost += N * leaf;
    return cost;
}

bool next_perm(uint32_t *a, uint32_t n) { return std::next_permutation(a, a + n); }

}  // namespace

extern "C" {

sge_status sge_pattern_info(uint32_t k, uint32_t m, const uint32_t *edges, uint64_t *aut_size, uint32_t *single_bag) {
    Pattern p;
    sge_status st = make_pattern(k, m, edges, p);
    if (st != SGE_OK) return st;
    std::vector<Perm> aut;
    if (!automorphisms(p, aut, 1u << 22)) return fail(SGE_UNSUPPORTED, "automorphism group larger than 2^22");
    if (aut_size) *aut_size = aut.size();
    if (single_bag) *single_bag = is_single_bag(p) ? 1u : 0u;
    return SGE_OK;
}

sge_status sge_graph_stats_compute(const uint32_t *off, const uint32_t *nb, uint32_t n, sge_graph_stats *out) {
    if (!off || !out) return fail(SGE_BAD_INPUT, "sge_graph_stats_compute: null argument");
    memset(out, 0, sizeof *out);
    out->num_vertices = n;
    out->num_directed_edges = off[n];
    for (uint32_t v = 0; v < n; ++v) {
        double d = (double)(off[v + 1] - off[v]), p = 1.0;
        out->max_degree = std::max(out->max_degree, d);
        for (uint32_t j = 0; j < SGE_MAX_K + 2; ++j) { out->moments[j] += p; p *= d; }
    }
    out->clustering = sample_clustering(off, nb, n);
    return SGE_OK;
}

sge_status sge_plan_pattern(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph *g,
                            const sge_plan_opts *opts, sge_plan_blob *out) {
    sge_graph_stats st;
    if (g && graph_stats(g, &st)) return sge_plan_pattern_stats(k, m, edges, &st, opts, out);
    return sge_plan_pattern_stats(k, m, edges, nullptr, opts, out);
}

// Collects every valid plan of the pattern with its cost-model estimate,
// cheapest first, without duplicates.
static sge_status collect_candidates(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *gs,
                                     const sge_plan_opts *opts, std::vector<Candidate> &out) {
    Pattern p;
    sge_status st = make_pattern(k, m, edges, p);
    if (st != SGE_OK) return st;
    sge_plan_opts o{};
    o.join_style = SGE_JOIN_WCOJ;
    o.use_iep = 1;
    o.max_tail = SGE_MAX_TAIL;
    if (opts) o = *opts;
    if (o.max_tail == 0 || o.max_tail > SGE_MAX_TAIL) o.max_tail = SGE_MAX_TAIL;
    if (o.join_style > SGE_JOIN_EXPLORATION) return fail(SGE_BAD_INPUT, "unknown join style %u", o.join_style);
    if (o.vertex_labels) {
        // labeled matching: only label-preserving automorphisms restrict symmetry
        if (o.join_style != SGE_JOIN_WCOJ) return fail(SGE_UNSUPPORTED, "labeled plans use the WCOJ join style");
        p.labeled = true;
        for (uint32_t u = 0; u < k; ++u) p.label[u] = o.vertex_labels[u];
    }
    std::vector<Perm> aut;
    if (!automorphisms(p, aut, 1u << 22)) return fail(SGE_UNSUPPORTED, "automorphism group larger than 2^22");
    const bool single = is_single_bag(p);
    Moments mo;
    if (gs) {
        for (uint32_t d = 0; d < SGE_MAX_K + 2; ++d) mo.M[d] = gs->moments[d];
        mo.n = gs->num_vertices;
        mo.nnz = gs->num_directed_edges;
        mo.clustering = gs->clustering;
        mo.have = true;
    } else {
        // no graph: a regular graph with n=1e6, degree 16
        mo.n = 1e6;
        mo.nnz = 16e6;
        for (uint32_t d = 0; d < SGE_MAX_K + 2; ++d) mo.M[d] = 1e6 * std::pow(16.0, (double)d);
    }
    out.clear();
    if (o.symmetry_seq) {
        uint32_t seen = 0;
        for (uint32_t i = 0; i < k; ++i) {
            if (o.symmetry_seq[i] >= k || ((seen >> o.symmetry_seq[i]) & 1u))
                return fail(SGE_BAD_INPUT, "symmetry_seq is not a permutation");
            seen |= 1u << o.symmetry_seq[i];
        }
    }
    if (o.root_edge && (o.root_edge[0] >= k || o.root_edge[1] >= k || !p.edge(o.root_edge[0], o.root_edge[1])))
        return fail(SGE_BAD_INPUT, "root_edge is not an edge of the pattern");
    std::vector<std::pair<uint32_t, uint32_t>> fixed_restr;
    if (o.symmetry_seq) fixed_restr = restrictions(p, aut, o.symmetry_seq);
    auto consider = [&](const uint32_t *order) {
        if (o.root_edge && !((order[0] == o.root_edge[0] && order[1] == o.root_edge[1]) ||
                             (order[0] == o.root_edge[1] && order[1] == o.root_edge[0])))
            return;
        // two restriction schemes: stabilize in matching order, or in reverse
        // (one, from symmetry_seq, when that is given)
        for (int scheme = 0; scheme < (o.symmetry_seq ? 1 : 2); ++scheme) {
            uint32_t seq[SGE_MAX_K];
            for (uint32_t i = 0; i < k; ++i) seq[i] = scheme == 0 ? order[i] : order[k - 1 - i];
            auto restr = o.symmetry_seq ? fixed_restr : restrictions(p, aut, seq);
            uint32_t tmax = std::min<uint32_t>(o.use_iep ? o.max_tail : 1u, k - 2);
            for (uint32_t T = 1; T <= tmax; ++T) {
                Candidate c;
                if (!build_blob(p, order, restr, T, o.use_iep != 0, o.join_style, aut.size(), single, c.blob)) continue;
                c.cost = plan_cost(p, c.blob, mo);
                c.blob.est_cost = c.cost;
                out.push_back(c);
            }
        }
    };
    if (o.force_order) {
        uint32_t seen = 0;
        for (uint32_t i = 0; i < k; ++i) {
            if (o.force_order[i] >= k || ((seen >> o.force_order[i]) & 1u)) return fail(SGE_BAD_INPUT, "force_order is not a permutation");
            seen |= 1u << o.force_order[i];
        }
        consider(o.force_order);
        if (out.empty())
            return fail(SGE_BAD_INPUT, "force_order is not a connected order starting with an edge (or the root_edge)");
    } else if (k <= 8) {
        uint32_t order[SGE_MAX_K];
        for (uint32_t i = 0; i < k; ++i) order[i] = i;
        do {
            if (!p.edge(order[0], order[1])) continue;
            bool conn = true;
            uint32_t seen = (1u << order[0]) | (1u << order[1]);
            for (uint32_t i = 2; i < k && conn; ++i) {
                if (!(p.adj[order[i]] & seen)) conn = false;
                seen |= 1u << order[i];
            }
            if (conn) consider(order);
        } while (next_perm(order, k));
    } else {
        // greedy: start from each edge, add the vertex with the most edges into
        // the matched set (ties: higher pattern degree)
        for (uint32_t a = 0; a < k; ++a)
            for (uint32_t bb = 0; bb < k; ++bb) {
                if (!p.edge(a, bb)) continue;
                uint32_t order[SGE_MAX_K];
                order[0] = a;
                order[1] = bb;
                uint32_t seen = (1u << a) | (1u << bb);
                for (uint32_t i = 2; i < k; ++i) {
                    int bestv = -1, bs = -1;
                    for (uint32_t v = 0; v < k; ++v) {
                        if ((seen >> v) & 1u) continue;
                        int sc = __builtin_popcount(p.adj[v] & seen) * 64 + p.deg(v);
                        if (__builtin_popcount(p.adj[v] & seen) > 0 && sc > bs) { bs = sc; bestv = (int)v; }
                    }
                    order[i] = (uint32_t)bestv;
                    seen |= 1u << bestv;
                }
                consider(order);
            }
    }
    if (out.empty()) return fail(SGE_UNSUPPORTED, "no executable plan found for the pattern");
    std::stable_sort(out.begin(), out.end(), [](const Candidate &x, const Candidate &y) { return x.cost < y.cost; });
    // drop exact duplicates (same blob up to the cost field)
    std::vector<Candidate> uniq;
    for (auto &c : out) {
        bool dup = false;
        for (auto &u : uniq)
            if (u.blob.k == c.blob.k && memcmp(&u.blob, &c.blob, offsetof(sge_plan_blob, est_cost)) == 0) { dup = true; break; }
        if (!dup) uniq.push_back(c);
        if (uniq.size() >= 4096) break;
    }
    out.swap(uniq);
    return SGE_OK;
}

sge_status sge_plan_pattern_stats(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *gs,
                                  const sge_plan_opts *opts, sge_plan_blob *out) {
    if (!out) return fail(SGE_BAD_INPUT, "sge_plan_pattern: null output");
    std::vector<Candidate> cands;
    sge_status st = collect_candidates(k, m, edges, gs, opts, cands);
    if (st != SGE_OK) return st;
    *out = cands.front().blob;
    return SGE_OK;
}

sge_status sge_plan_candidates(uint32_t k, uint32_t m, const uint32_t *edges, const sge_graph_stats *gs,
                               const sge_plan_opts *opts, sge_plan_blob *out, uint32_t cap, uint32_t *n_out) {
    if (!out || !n_out || cap == 0) return fail(SGE_BAD_INPUT, "sge_plan_candidates: bad argument");
    std::vector<Candidate> cands;
    sge_status st = collect_candidates(k, m, edges, gs, opts, cands);
    if (st != SGE_OK) return st;
    uint32_t n = (uint32_t)std::min<size_t>(cap, cands.size());
    for (uint32_t i = 0; i < n; ++i) out[i] = cands[i].blob;
    *n_out = n;
    return SGE_OK;
}

sge_status sge_plan_features(const sge_plan_blob *b, const sge_graph_stats *gs, float *f) {
    if (!b || !f) return fail(SGE_BAD_INPUT, "sge_plan_features: null argument");
    for (uint32_t i = 0; i < SGE_FEATURES; ++i) f[i] = 0.f;
    auto lg2 = [](double x) { return (float)std::log2(x + 1.0); };
    if (gs) {
        f[0] = lg2(gs->num_vertices) / 32.f;
        f[1] = lg2(gs->num_directed_edges) / 32.f;
        f[2] = lg2(gs->moments[2] / std::max(gs->moments[1], 1.0)) / 16.f;
        f[3] = (float)gs->clustering;
        f[4] = lg2(gs->max_degree) / 24.f;
    }
    uint32_t medges = 0, tailpar = 0;
    for (uint32_t i = 0; i < b->k; ++i) medges += __builtin_popcount(b->parents[i]);
    for (uint32_t i = b->num_enum; i < b->k; ++i) tailpar += __builtin_popcount(b->parents[i]);
    f[5] = b->k / 16.f;
    f[6] = b->k > 1 ? (float)medges / (b->k * (b->k - 1) / 2) : 0.f;
    f[7] = lg2((double)b->aut_size) / 16.f;
    f[8] = b->num_enum / 16.f;
    f[9] = b->tail_len / 4.f;
    if (b->tail_mode >= 1 && b->tail_mode <= 3) f[9 + b->tail_mode] = 1.f;  // 10..12
    f[13] = (float)b->join_style;
    if (b->root_kind <= 2) f[14 + b->root_kind] = 1.f;  // 14..16
    f[17] = b->num_restrictions / 16.f;
    f[18] = (float)b->single_bag;
    f[19] = lg2(b->est_cost) / 64.f;
    for (uint32_t l = 2; l < 9 && l < b->k; ++l) {
        float *q = f + 20 + (l - 2) * 6;
        const uint32_t last = b->parents[l] ? 31u - (uint32_t)__builtin_clz(b->parents[l]) : 0u;
        q[0] = __builtin_popcount(b->parents[l]) / 8.f;
        q[1] = __builtin_popcount(b->lower[l] | b->upper[l]) / 4.f;
        q[2] = b->base[l] >= 0 ? 1.f : 0.f;
        q[3] = __builtin_popcount(b->rest[l]) / 8.f;
        q[4] = l >= b->num_enum ? 1.f : 0.f;
        q[5] = (l >= b->num_enum && __builtin_popcount(b->parents[l]) >= 2 && last + 1 < b->num_enum) ? 1.f : 0.f;
    }
    f[62] = tailpar / 16.f;
    f[63] = 1.f;
    return SGE_OK;
}

sge_status sge_plan_validate(const sge_plan_blob *b) {
    if (!b) return fail(SGE_BAD_INPUT, "plan is null");
    if (b->magic != SGE_PLAN_MAGIC) return fail(SGE_BAD_INPUT, "plan magic mismatch");
    if (b->abi_version != SGE_ABI_VERSION) return fail(SGE_BAD_INPUT, "plan ABI version %u (library %u)", b->abi_version, SGE_ABI_VERSION);
    const uint32_t k = b->k, ne = b->num_enum;
    if (k < 3 || k > SGE_MAX_K) return fail(SGE_BAD_INPUT, "plan k=%u outside 3..%u", k, SGE_MAX_K);
    if (ne < 2 || ne >= k || b->tail_len != k - ne || b->tail_len > SGE_MAX_TAIL)
        return fail(SGE_BAD_INPUT, "plan num_enum=%u tail_len=%u inconsistent with k=%u", ne, b->tail_len, k);
    if (b->tail_mode < SGE_TAIL_SINGLE || b->tail_mode > SGE_TAIL_IEP) return fail(SGE_BAD_INPUT, "bad tail mode %u", b->tail_mode);
    if (b->tail_mode == SGE_TAIL_SINGLE && b->tail_len != 1) return fail(SGE_BAD_INPUT, "SINGLE tail needs tail_len 1");
    if (b->join_style > SGE_JOIN_EXPLORATION) return fail(SGE_BAD_INPUT, "bad join style");
    if (b->root_kind > 2) return fail(SGE_BAD_INPUT, "bad root kind");
    if (b->count_multiplier == 0) return fail(SGE_BAD_INPUT, "count_multiplier is 0");
    if (b->choose_wrap > 1) return fail(SGE_BAD_INPUT, "choose_wrap must be 0 or 1");
    if (b->labeled > 1) return fail(SGE_BAD_INPUT, "labeled must be 0 or 1");
    if (b->labeled && b->join_style != SGE_JOIN_WCOJ) return fail(SGE_BAD_INPUT, "labeled plans use the WCOJ join style");
    uint32_t seen = 0;
    for (uint32_t i = 0; i < k; ++i) {
        if (b->order[i] >= k || ((seen >> b->order[i]) & 1u)) return fail(SGE_BAD_INPUT, "order is not a permutation");
        seen |= 1u << b->order[i];
    }
    if (b->parents[1] != 1u) return fail(SGE_BAD_INPUT, "level 1 must have exactly level 0 as parent");
    if ((b->lower[1] | b->upper[1]) & ~1u) return fail(SGE_BAD_INPUT, "level 1 bounds must refer to level 0");
    if (b->root_kind == SGE_ROOT_ASC && !(b->lower[1] & 1u)) return fail(SGE_BAD_INPUT, "ASC root without level-1 lower bound");
    if (b->root_kind == 2 && !(b->upper[1] & 1u)) return fail(SGE_BAD_INPUT, "DESC root without level-1 upper bound");
    if (b->root_kind == SGE_ROOT_ANY && ((b->lower[1] | b->upper[1]) & 1u)) return fail(SGE_BAD_INPUT, "ANY root with a level-1 bound");
    for (uint32_t i = 1; i < k; ++i) {
        uint32_t below = (i < ne) ? ((1u << i) - 1) : ((1u << ne) - 1);
        uint32_t all = b->parents[i] | b->lower[i] | b->upper[i] | b->check[i];
        if (all & ~below) return fail(SGE_BAD_INPUT, "level %u refers to a level it cannot see", i);
        if (all != below) return fail(SGE_BAD_INPUT, "level %u does not exclude every earlier level (injectivity)", i);
        if (b->parents[i] == 0) return fail(SGE_BAD_INPUT, "level %u has no parent", i);
        if (b->base[i] >= 0) {
            uint32_t l = (uint32_t)b->base[i];
            if (l < 2 || l >= i || l >= ne) return fail(SGE_BAD_INPUT, "level %u reuses level %u", i, l);
            if (b->parents[l] & ~b->parents[i])
                return fail(SGE_BAD_INPUT, "level %u reuse of level %u is not implied", i, l);
            if ((b->parents[l] | b->rest[i]) != b->parents[i]) return fail(SGE_BAD_INPUT, "level %u rest mask inconsistent", i);
        } else if (b->base[i] != -1) {
            return fail(SGE_BAD_INPUT, "level %u base %d", i, b->base[i]);
        }
    }
    if (b->tail_mode == SGE_TAIL_IEP) {
        if (b->num_partitions == 0 || b->num_partitions > SGE_MAX_PARTITIONS) return fail(SGE_BAD_INPUT, "bad partition count");
        const uint32_t full = (1u << b->tail_len) - 1;
        for (uint32_t pi = 0; pi < b->num_partitions; ++pi) {
            uint32_t acc = 0;
            if (b->part_nblocks[pi] == 0 || b->part_nblocks[pi] > b->tail_len) return fail(SGE_BAD_INPUT, "bad partition");
            for (uint32_t x = 0; x < b->part_nblocks[pi]; ++x) {
                uint32_t blk = b->part_block[pi][x];
                if (blk == 0 || (blk & acc) || (blk & ~full)) return fail(SGE_BAD_INPUT, "bad partition block");
                acc |= blk;
            }
            if (acc != full) return fail(SGE_BAD_INPUT, "partition does not cover the tail");
        }
    }
    return SGE_OK;
}

}  // extern "C"

extern "C" sge_status sge_plan_pattern_learned(uint32_t k, uint32_t m, const uint32_t *edges,
                                               const sge_graph_stats *gs, const sge_plan_opts *opts, sge_mlp *scorer,
                                               uint32_t shortlist, sge_plan_blob *out) {
    if (!out || !scorer) return fail(SGE_BAD_INPUT, "sge_plan_pattern_learned: null argument");
    std::vector<Candidate> cands;
    sge_status st = collect_candidates(k, m, edges, gs, opts, cands);
    if (st != SGE_OK) return st;
    const uint32_t n = (uint32_t)std::min<size_t>(shortlist ? shortlist : 64u, cands.size());
    std::vector<float> feats((size_t)n * SGE_FEATURES), pred(n);
    for (uint32_t i = 0; i < n; ++i) sge_plan_features(&cands[i].blob, gs, &feats[(size_t)i * SGE_FEATURES]);
    st = sge_mlp_forward_bf16(scorer, feats.data(), n, pred.data());
    if (st != SGE_OK) return st;
    uint32_t best = 0;
    for (uint32_t i = 1; i < n; ++i)
        if (pred[i] < pred[best]) best = i;
    *out = cands[best].blob;
    return SGE_OK;
}

extern "C" sge_status sge_pattern_automorphisms(uint32_t k, uint32_t m, const uint32_t *edges, uint8_t *out,
                                                uint32_t cap, uint32_t *naut) {
    if (!out || !naut) return fail(SGE_BAD_INPUT, "sge_pattern_automorphisms: null argument");
    Pattern p;
    sge_status st = make_pattern(k, m, edges, p);
    if (st != SGE_OK) return st;
    std::vector<Perm> aut;
    if (!automorphisms(p, aut, cap)) return fail(SGE_UNSUPPORTED, "more than %u automorphisms", cap);
    for (size_t a = 0; a < aut.size(); ++a)
        for (uint32_t j = 0; j < k; ++j) out[a * k + j] = aut[a][j];
    *naut = (uint32_t)aut.size();
    return SGE_OK;
}

// The reference's plan as text: the block HyperTree::writeToStream prints
// ("num bags: N" then one comma-separated attribute order per bag, global bag
// last; plan/decomposition.cpp:537-552, printed by main.cpp:66) or an order
// file in buildTreesFromOrderFile's format (one order per line,
// plan/optimizer.cpp:724-752).  Other lines of a reference log (timings,
// counts) and symmetry-rule lines ("a < b,c,") are skipped.
static bool parse_order_line(const char *s, const char *e, std::vector<uint32_t> &out) {
    out.clear();
    bool any = false;
    uint64_t cur = 0;
    bool in_num = false;
    for (const char *q = s; q < e; ++q) {
        const char ch = *q;
        if (ch >= '0' && ch <= '9') {
            cur = cur * 10 + (uint64_t)(ch - '0');
            if (cur > 0xFFFFu) return false;
            in_num = any = true;
        } else if (ch == ',' || ch == ' ' || ch == '\t' || ch == '\r') {
            if (in_num) { out.push_back((uint32_t)cur); cur = 0; in_num = false; }
        } else {
            return false;
        }
    }
    if (in_num) out.push_back((uint32_t)cur);
    return any && !out.empty();
}

sge_status sge::parse_bag_text(uint32_t k, const char *text, std::vector<std::vector<uint32_t>> &bags) {
    bags.clear();
    long want = -1;  // from "num bags: N"
    std::vector<uint32_t> row;
    for (const char *s = text; *s;) {
        const char *e = s;
        while (*e && *e != '\n') ++e;
        if (strncmp(s, "num bags:", 9) == 0) {
            want = strtol(s + 9, nullptr, 10);
            bags.clear();
        } else if (parse_order_line(s, e, row)) {
            if (want < 0 || (long)bags.size() < want) bags.push_back(row);
        }
        s = *e ? e + 1 : e;
        if (want >= 0 && (long)bags.size() == want) break;
    }
    if (bags.empty()) return fail(SGE_BAD_INPUT, "plan text holds no bag order");
    if (want >= 0 && (long)bags.size() != want)
        return fail(SGE_BAD_INPUT, "plan text announces %ld bags but holds %zu orders", want, bags.size());
    // every attribute is a pattern vertex, once per bag; the bags cover the vertices
    uint32_t covered = 0;
    for (size_t b = 0; b < bags.size(); ++b) {
        uint32_t mask = 0;
        for (uint32_t u : bags[b]) {
            if (u >= k) return fail(SGE_BAD_INPUT, "bag %zu names vertex %u of a %u-vertex pattern", b, u, k);
            if ((mask >> u) & 1u) return fail(SGE_BAD_INPUT, "bag %zu names vertex %u twice", b, u);
            mask |= 1u << u;
        }
        covered |= mask;
    }
    if (covered != ((1u << k) - 1u)) return fail(SGE_BAD_INPUT, "the bags do not cover every pattern vertex");
    return SGE_OK;
}

extern "C" sge_status sge_plan_from_order_text(uint32_t k, uint32_t m, const uint32_t *edges, const char *text,
                                               const sge_graph_stats *stats, const sge_plan_opts *opts,
                                               sge_plan_blob *out, uint32_t *num_bags) {
    if (!text || !out || !edges) return fail(SGE_BAD_INPUT, "sge_plan_from_order_text: null argument");
    if (k < 3 || k > SGE_MAX_K) return fail(SGE_BAD_INPUT, "pattern k=%u outside 3..%u", k, SGE_MAX_K);
    Pattern p;
    sge_status st = make_pattern(k, m, edges, p);
    if (st != SGE_OK) return st;
    std::vector<std::vector<uint32_t>> bags;
    st = parse_bag_text(k, text, bags);
    if (st != SGE_OK) return st;
    // every pattern edge lies inside some bag (a decomposition)
    std::vector<uint32_t> bag_mask(bags.size(), 0);
    for (size_t b = 0; b < bags.size(); ++b)
        for (uint32_t u : bags[b]) bag_mask[b] |= 1u << u;
    for (uint32_t a = 0; a < k; ++a)
        for (uint32_t c = a + 1; c < k; ++c) {
            if (!p.edge(a, c)) continue;
            bool in = false;
            for (uint32_t msk : bag_mask) in |= ((msk >> a) & 1u) && ((msk >> c) & 1u);
            if (!in) return fail(SGE_BAD_INPUT, "pattern edge (%u,%u) lies in no bag", a, c);
        }
    // Execution order of the reference's join: the global bag's attributes in
    // its order (the prefix shared by the bags comes first in every order),
    // then each other bag's own attributes in its order (matched in its trie
    // and counted at the leaf).  The device DFS needs each vertex to have an
    // earlier neighbour and the first two to be an edge, so a vertex that has
    // none yet waits for the first point where it does (the sequence is
    // otherwise kept).
    std::vector<uint32_t> seq;
    uint32_t in_seq = 0;
    auto take = [&](const std::vector<uint32_t> &o) {
        for (uint32_t u : o)
            if (!((in_seq >> u) & 1u)) { seq.push_back(u); in_seq |= 1u << u; }
    };
    take(bags.back());
    for (size_t b = 0; b + 1 < bags.size(); ++b) take(bags[b]);
    uint32_t order[SGE_MAX_K], placed = 0;
    std::vector<bool> used(seq.size(), false);
    for (uint32_t i = 0; i < k; ++i) {
        size_t pick = seq.size();
        for (size_t j = 0; j < seq.size() && pick == seq.size(); ++j) {
            if (used[j]) continue;
            if (i == 0 || (p.adj[seq[j]] & placed)) pick = j;
        }
        if (pick == seq.size()) return fail(SGE_BAD_INPUT, "the pattern is not connected");
        used[pick] = true;
        order[i] = seq[pick];
        placed |= 1u << seq[pick];
    }
    sge_plan_opts o{};
    o.join_style = SGE_JOIN_WCOJ;
    o.use_iep = 1;
    o.max_tail = SGE_MAX_TAIL;
    if (opts) o = *opts;
    o.force_order = order;
    std::vector<Candidate> cands;
    st = collect_candidates(k, m, edges, stats, &o, cands);
    if (st != SGE_OK) return st;
    // sharedJoin matches the global bag and counts the other bags' own
    // attributes at the leaf (join.cpp:1520-1691): the tail is as long as the
    // attributes outside the global bag allow (cheapest such candidate; the
    // candidates come sorted by cost)
    uint32_t outside = k - (uint32_t)__builtin_popcount(bag_mask.back());
    size_t pick = 0;
    for (size_t i = 0; i < cands.size(); ++i)
        if (cands[i].blob.tail_len <= std::max<uint32_t>(outside, 1u) &&
            cands[i].blob.tail_len > cands[pick].blob.tail_len)
            pick = i;
    *out = cands[pick].blob;
    // "Number of matches" follows the imported plan's shape: embeddings for a
    // one-bag plan, instances otherwise (relation/graph.cpp:910-1077,
    // plan/decomposition.cpp:983-986)
    out->choose_wrap = 1u;  // the reference's choosec arithmetic
    out->single_bag = bags.size() == 1 ? 1u : 0u;
    out->count_multiplier = bags.size() == 1 ? out->aut_size : 1u;
    if (num_bags) *num_bags = (uint32_t)bags.size();
    return SGE_OK;
}
