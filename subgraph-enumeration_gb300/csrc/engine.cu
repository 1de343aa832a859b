// GB300 (sm_103a) execution engine: device graph, compiled plans, and the
// persistent counting kernel behind sge_count.
//
// Replaces the reference's join drivers: sharedJoin / globalJoin / traverse
// (matching/join.cpp:812-1691) and their OpenMP split parSharedJoin /
// subtreeSharedJoin (matching/parallel.cpp:167-1844).  The reference gives one
// OpenMP task per root (a candidate of the first shared attribute, or a data
// edge, parallel.cpp:1272,1414); here one warp owns one root edge at a time,
// taken from a per-plan atomic queue, and runs the plan's depth-first search:
//   - candidate generation = bound trimming (setBeginPos/setEndPos,
//     utility/utils.cpp:581-612) + k-way intersection (ComputeCandidates /
//     MultiIntersection, utility/compute_set_intersection.cpp:10-87,308-342),
//     done as a warp-parallel membership test of one list against the others:
//     shared-memory bitmap/hash probes for the root's pinned lists, binary
//     search otherwise, compacted with ballot/popc;
//   - the last two enumerated levels run as one step flattened over
//     (candidate, element) pairs across the lanes ("pair step");
//   - the last tail_len levels are counted, not enumerated, 32 candidates at
//     a time with their list scans flattened across the lanes: numResults
//     (relation/relation.cpp:290-338), choosec (utils.cpp:80-94) and the
//     inclusion–exclusion of numUniqueCombine (utils.cpp:290-350);
//   - exploration style (-i) keeps running candidate lists per later level,
//     updated as soon as a parent is matched (join.cpp:266-307).
// The DFS is latency-bound, so the per-warp state is kept small enough for 28
// resident warps per SM.  Counts are exact uint64 (wrapping like the
// reference's size_t).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "common.hpp"
#include "device_util.hpp"

using namespace sge;

#define FULL_MASK 0xFFFFFFFFu
#define SGE_MAX_BUFS 32
// exploration version slots: at most Σ_{i<16} (i-1) = 105 for k <= 16
#define SGE_MAX_VSLOTS 112

namespace {

struct DevGraph {
    const uint32_t *off;    // n+1
    const uint32_t *adj;    // nnz
    const uint2 *edges;     // m undirected edges (u<v)
    uint32_t n;
    uint64_t m;
    // Hub index: every vertex of degree >= hub_min has a bitmap of its
    // neighbours (hub_words words over all vertex ids) at hub_slot[v], so a
    // membership test in its list is one load instead of a binary search
    // (hub_min = 0xFFFFFFFF: no index).
    const uint32_t *hub_bits;
    const int32_t *hub_slot;
    uint32_t hub_words, hub_min;
};

// A bag relation's trie on the device (sge_trie levels): key columns
// 0..nkeys-1, the bag's own attribute in column nkeys.  The first key level
// is dense over vertex ids: [first[v], first[v+1]) are the level-1 nodes
// under key v (empty when v heads no tuple).  Below it, node p of level l
// owns children [child[l][p], child[l][p+1]) of level l+1; val[l] are the
// values of level l (val[0] and child[0] are unused).
struct DevTrie {
    const unsigned long long *first;
    const uint32_t *val[4];
    const unsigned long long *child[3];
    uint32_t nkeys, pad_;
};

// Range [off, off+len) of val[nkeys] under the key tuple key[0..nkeys-1]
// (len = 0 when the tuple is absent): one dense step, then one binary search
// per further key within its parent's children.
__device__ __forceinline__ void trie_range(const DevTrie &T, const uint32_t *key, uint32_t &off, uint32_t &len) {
    unsigned long long lo = __ldg(T.first + key[0]), hi = __ldg(T.first + key[0] + 1);
    for (uint32_t c = 1; c < T.nkeys && lo < hi; ++c) {
        const uint32_t *v = T.val[c] + lo;
        const uint32_t n = (uint32_t)(hi - lo);
        uint32_t a = 0, w = n;
        while (w > 0) {
            const uint32_t half = w >> 1;
            if (__ldg(v + a + half) < key[c]) { a += half + 1; w -= half + 1; }
            else w = half;
        }
        if (a == n || __ldg(v + a) != key[c]) { lo = hi; break; }
        const unsigned long long p = lo + a;
        lo = __ldg(T.child[c] + p);
        hi = __ldg(T.child[c] + p + 1);
    }
    off = (uint32_t)lo;
    len = (uint32_t)(hi - lo);
}

// Compact device form of sge_plan_blob (+ batch bookkeeping).
struct DevPlan {
    // level masks fit 16 bits (k <= SGE_MAX_K = 16); small fields are bytes,
    // which keeps the per-warp shared-memory copy of the plan small
    uint16_t parents[SGE_MAX_K], lower[SGE_MAX_K], upper[SGE_MAX_K], check[SGE_MAX_K], rest[SGE_MAX_K];
    uint16_t after[SGE_MAX_K];          // exploration: later levels having this level as a parent
    int8_t base[SGE_MAX_K];
    uint8_t order_[SGE_MAX_K];          // pattern vertex of each level (enumeration output order)
    uint8_t hoist_at[SGE_MAX_K];        // level after whose match a hoisted list is computed
    int8_t slot[SGE_MAX_K][SGE_MAX_K];  // exploration: buffer slot of version (j, i), -1 = direct N(m[j])
    int8_t part_coef[SGE_MAX_PARTITIONS];
    uint8_t part_nblocks[SGE_MAX_PARTITIONS];
    uint8_t part_block[SGE_MAX_PARTITIONS][SGE_MAX_TAIL];
    uint8_t pad_[2];
    uint32_t k, ne, T, tail_mode, join_style, root_kind, nparts, nbufs;
    unsigned long long task_begin, ntasks;        // this batch's task range for the plan
    unsigned long long root_stride, root_offset;  // task j of the plan = root root_offset + j*root_stride
    unsigned long long mult;                      // count multiplier (|Aut| for single-bag plans)
    uint32_t chunk;                               // root tasks per queue grab
    uint32_t pin_mask;                            // levels 0/1 whose lists are pinned in shared memory
    uint32_t keep_full;                           // levels whose bound-free list later levels reuse
    uint32_t hoist_mask;                          // tail levels whose list is computed early (WCOJ)
    uint32_t split_par;                           // level 2's parents (levels 0/1): bounds its list by degree
    uint32_t split_H;                             // roots whose level-2 bound exceeds this are deferred
    uint32_t split_S;                             // level-2 candidates per deferred task (0 = never defer)
    uint32_t split_P3;                            // parts of each level-3 list per deferred task (1 = none)
    uint32_t pair;                                // 1: the last two enumerated levels run as one flattened step
    uint32_t pair_direct;                         // pair step may count a single-list tail per pair inline
    uint32_t epin;                                // exploration: tail level whose root-level running list is pinned
    uint32_t tail_par;                            // union of the tail levels' parents
    uint32_t choose_wrap;                         // CHOOSE leaves use the reference's wrapping choosec
    uint32_t root_maxdeg;                         // roots with an endpoint of larger degree are skipped (0 = none)
    uint32_t no_hubs;                             // this plan probes lists by binary search only
    // bag relations (sge_plan_use_bags): up to 2 tail levels read their
    // candidates from a trie; tri[i] = slot 0/1 of tail level i, -1 = none
    const DevTrie *tries;                         // the bag set's device array
    int8_t tri[SGE_MAX_K];
    uint8_t trel[2];                              // relation of slot j in `tries`
    uint8_t tkey[2][3];                           // key levels of slot j, in the trie's key order
    uint8_t ntrie, pad2_[3];
    // labeled matching (sge_plan_set_labels): vlab = the data graph's vertex
    // labels (null: unlabeled), lab[i] = the label of level i's pattern vertex
    const uint32_t *vlab;
    uint32_t lab[SGE_MAX_K];
};
static_assert(sizeof(DevPlan) % 4 == 0, "DevPlan is copied as 32-bit words");

struct DevStats {
    unsigned long long set_ops, alg_bytes, partial, roots;
};

// Flags written by kernels (never trapped on): bit0 overflow, bit1 timeout.
// bit2: a CHOOSE leaf's falling product reached 2^64 (informational).
enum { FLAG_OVERFLOW = 1u, FLAG_TIMEOUT = 2u, FLAG_CHOOSE_WRAP = 4u };

// Per-warp DFS state (shared memory).
struct WarpState {
    uint32_t m[SGE_MAX_K];
    uint32_t pos[SGE_MAX_K];
    uint32_t cnt[SGE_MAX_K];
    const uint32_t *list[SGE_MAX_K];
    const uint32_t *flist[SGE_MAX_K];     // level's full (bound-free) list, for reuse by later levels
    uint32_t fcnt[SGE_MAX_K];
    const uint32_t *lptr[SGE_MAX_K];      // N(m[j]) of the matched levels
    uint32_t llen[SGE_MAX_K];
    int32_t hs[SGE_MAX_K];                // hub bitmap slot of m[j], -1 = none
    uint32_t pmode[3];                    // pinned N(m[0]), N(m[1]), level-2 list: 0 none, 1 bitmap, 2 hash
    uint32_t hcnt[SGE_MAX_K];             // hoisted tail lists (buffer slot = level)
    uint32_t hpin;                        // tail level whose hoisted list is pinned in table 2 (0 = none)
    unsigned long long t_root;            // globaltimer at the start of the current root (per-plan busy time)
};

// One tail level's candidate set as the leaf probes it: its lists (a pinned
// table, a sorted list, or the CSR list of a candidate's own level = slot),
// the bound and exclusion values from the levels below the leaf's first
// candidate level, and which slots add bounds or exclusions.
struct TailDesc {
    const uint32_t *ptr[SGE_MAX_K];
    const uint32_t *vlab;     // labeled plans: the data graph's labels (null: unlabeled)
    uint32_t len[SGE_MAX_K];
    uint32_t exv[SGE_MAX_K];
    uint32_t lo, hi, lab;     // lab: the level's pattern label
    uint8_t kind[SGE_MAX_K];  // 0..2 pinned table; 3 sorted list; 4/5 CSR list of slot 0/1
    int8_t lvl[SGE_MAX_K];    // kind 3: the matched level whose CSR list it is, -1 = a stored list
    uint8_t nsrc, nex, has_lo, has_hi, lo_slots, hi_slots, ex_slots, pad;
};

// Leaf state (shared memory): up to 32 candidates of the last enumerated
// level, each with its own matched values for the levels from L0 on.
struct LeafState {
    uint32_t cm[32][2];
    const uint32_t *bptr[32];
    uint32_t pref[32];
    // per slot s and candidate l: (offset, length) of a per-candidate list.
    // Slots 0/1: the CSR lists of the candidate's own levels; slots 2/3: its
    // ranges of the bag-relation tries.  Slots 2/3 are last so that a warp's
    // shared memory holds them only in launches whose plans use tries.
    uint2 ol[4][32];
};
// Shared-memory bytes of a warp's LeafState with ntr trie slots (0..2).
__host__ __device__ constexpr size_t leaf_bytes(uint32_t ntr) {
    return sizeof(LeafState) - (2u - ntr) * 32u * sizeof(uint2);
}

// Pair step (shared memory): level a = ne-2 of the DFS is processed 32
// candidates x at a time; level a+1's candidates y of all 32 are generated in
// one flattened scan, and the (x, y) pairs go to the leaf 32 at a time.
struct PairState {
    const uint32_t *sptr[SGE_MAX_K];  // level a+1's lists that do not depend on x
    uint32_t slen[SGE_MAX_K];
    int32_t stab[SGE_MAX_K];          // pinned table holding the list, -1 = none
    int32_t shub[SGE_MAX_K];          // hub bitmap slot when the list is a hub's CSR list, -1 = none
    uint32_t ns;                      // number of such lists
    uint32_t xpar;                    // 1: N(x) is also one of level a+1's lists
    uint32_t exv[SGE_MAX_K];          // matched values below a that level a+1 excludes
    uint32_t nex;
    uint32_t x[32];                   // this batch's level-a candidates
    uint32_t xo[32];                  // N(x): CSR offset
    uint32_t xl[32];
    const uint32_t *bp[32];           // list scanned for candidate x (trimmed by bounds)
    uint32_t pref[32];
    uint32_t qx[64], qy[64];          // (x, y) pairs waiting for the leaf
    uint32_t tr[32];                  // inline tail: x's count before y's own exclusion
    TailDesc ptd;                     // inline tail: the tail level as seen from level a
};

constexpr uint32_t PIN_EMPTY = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Lists searched here may be per-warp scratch written earlier in the same
// launch, so these use ordinary (coherent) loads, never the read-only path.
// first index with a[i] >= x  (std::lower_bound)
__device__ __forceinline__ uint32_t lb(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        uint32_t half = n >> 1;
        if (a[lo + half] < x) { lo += half + 1; n -= half + 1; }
        else n = half;
    }
    return lo;
}
// first index with a[i] > x  (std::upper_bound)
__device__ __forceinline__ uint32_t ub(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0;
    while (n > 0) {
        uint32_t half = n >> 1;
        if (a[lo + half] <= x) { lo += half + 1; n -= half + 1; }
        else n = half;
    }
    return lo;
}
__device__ __forceinline__ bool contains(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t i = lb(a, n, x);
    return i < n && a[i] == x;
}

// y ∈ N(hub) through the hub's bitmap (read-only for the whole launch).
__device__ __forceinline__ bool hub_has(const DevGraph &g, int32_t slot, uint32_t y) {
    return (__ldg(g.hub_bits + (size_t)slot * g.hub_words + (y >> 5)) >> (y & 31u)) & 1u;
}
// Bitmap slot of v given its degree (-1 below the hub threshold).
__device__ __forceinline__ int32_t hub_slot_of(const DevGraph &g, uint32_t v, uint32_t deg) {
    return deg >= g.hub_min ? __ldg(g.hub_slot + v) : -1;
}
// y ∈ N(v) for the CSR list (p, len) of vertex v.
__device__ __forceinline__ bool csr_has(const DevGraph &g, uint32_t v, const uint32_t *p, uint32_t len, uint32_t y) {
    const int32_t s = hub_slot_of(g, v, len);
    return s >= 0 ? hub_has(g, s, y) : contains(p, len, y);
}
// Probe cost of a sorted list of len elements searched by bisection (a table
// or bitmap probe costs 1).
__device__ __forceinline__ uint32_t search_cost(uint32_t len) { return 2u + (31u - __clz(len + 1u)); }
// Algorithmic bytes of probing a list of len elements nprobe times (the
// instrumented kernel's counters): through a table or hub bitmap each probe
// reads one word; by bisection the list counts as a merge would consume it,
// plus its offset pair.
__device__ __forceinline__ unsigned long long probe_bytes(unsigned long long nprobe, uint32_t len, bool table) {
    return table ? 4ull * nprobe : 8ull + 4ull * len;
}

__device__ __forceinline__ unsigned long long binom_exact(unsigned long long n, uint32_t r) {
    if (n < r) return 0ull;
    unsigned __int128 acc = 1;
    for (uint32_t i = 0; i < r; ++i) acc = acc * (unsigned __int128)(n - i) / (unsigned __int128)(i + 1);
    return (unsigned long long)acc;
}

// CHOOSE leaf: C(n, r) for the r symmetric last levels (symmLastLevel,
// matching/join.cpp:1534-1538).  The reference's choosec
// (utility/utils.cpp:80-94) multiplies n(n-1)…(n-r+1) in uint64 before
// dividing by r!, so it wraps once that product reaches 2^64; wrap selects
// its arithmetic, otherwise the exact binomial.  A product past 2^64 is
// reported through the flags either way.
__device__ __forceinline__ unsigned long long choose_leaf(unsigned long long n, uint32_t r, uint32_t wrap,
                                                          uint32_t *flags) {
    if (n < r) return 0ull;
    unsigned long long nom = n, denom = 1;
    unsigned __int128 wide = n;
    for (uint32_t i = 1; i < r; ++i) {
        nom *= n - i;
        denom *= i + 1;
        wide *= (unsigned __int128)(n - i);
    }
    if ((unsigned long long)(wide >> 64)) atomicOr(flags, FLAG_CHOOSE_WRAP);
    return wrap ? nom / denom : binom_exact(n, r);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    // three 32-bit warp reductions (redux.sync) instead of five 64-bit
    // shuffle steps: the high words (only their sum mod 2^32 matters) and the
    // low words in 16-bit halves (each half's sum stays below 2^21)
    const uint32_t lo = (uint32_t)v;
    const uint32_t hi = __reduce_add_sync(FULL_MASK, (uint32_t)(v >> 32));
    const uint32_t a = __reduce_add_sync(FULL_MASK, lo >> 16);
    const uint32_t b = __reduce_add_sync(FULL_MASK, lo & 0xFFFFu);
    return ((unsigned long long)hi << 32) + ((unsigned long long)a << 16) + b;
}

// Bounds of level i from the current partial match: keep lo < x < hi.
struct Bounds {
    uint32_t lo, hi;
    bool has_lo, has_hi;
};
__device__ __forceinline__ Bounds level_bounds(const DevPlan &P, const WarpState &W, uint32_t i) {
    Bounds b;
    b.lo = 0;
    b.hi = 0xFFFFFFFFu;
    b.has_lo = P.lower[i] != 0;
    b.has_hi = P.upper[i] != 0;
    for (uint32_t msk = P.lower[i]; msk; msk &= msk - 1) b.lo = max(b.lo, W.m[__ffs(msk) - 1]);
    for (uint32_t msk = P.upper[i]; msk; msk &= msk - 1) b.hi = min(b.hi, W.m[__ffs(msk) - 1]);
    return b;
}

__device__ __forceinline__ bool excluded(const DevPlan &P, const WarpState &W, uint32_t i, uint32_t x) {
    bool ex = false;
    for (uint32_t msk = P.check[i]; msk; msk &= msk - 1) ex |= (W.m[__ffs(msk) - 1] == x);
    return ex;
}
// x may not be level i's match: an earlier match (injectivity) or, for a
// labeled plan, a vertex of another label.  (Stored lists are filtered by
// excluded() alone: a later level with another label may reuse them.)
__device__ __forceinline__ bool rejected(const DevPlan &P, const WarpState &W, uint32_t i, uint32_t x) {
    if (P.vlab && __ldg(P.vlab + x) != P.lab[i]) return true;
    return excluded(P, W, i, x);
}

__device__ __forceinline__ void nbr(const DevGraph &g, uint32_t v, const uint32_t *&p, uint32_t &len) {
    uint32_t a = __ldg(g.off + v), b = __ldg(g.off + v + 1);
    p = g.adj + a;
    len = b - a;
}

__device__ __forceinline__ void nbr_off(const DevGraph &g, uint32_t v, uint32_t &off, uint32_t &len) {
    const uint32_t a = __ldg(g.off + v), b = __ldg(g.off + v + 1);
    off = a;
    len = b - a;
}

// Trim a sorted list to (lo, hi).
__device__ __forceinline__ void trim(const uint32_t *&p, uint32_t &len, const Bounds &b) {
    if (b.has_lo) { uint32_t s = ub(p, len, b.lo); p += s; len -= s; }
    if (b.has_hi) { len = lb(p, len, b.hi); }
}

template <bool STATS>
struct Ctx {
    DevGraph g;
    uint32_t *buf;    // this warp's scratch: nbufs × cap
    uint32_t cap;
    uint32_t *flags;
    uint32_t *tab;    // this warp's three pinned-list tables (shared memory), tw words each
    uint32_t tw;
    uint32_t tmode;   // 0 none, 1 bitmap over all vertices, 2 open-addressing hash
    LeafState *L;
    PairState *PS;
    TailDesc *td;     // this warp's tail descriptors (one per inclusion–exclusion pass)
    uint32_t *vs;     // exploration: length of the version list in each buffer slot
    uint32_t *cnt;    // per-candidate counters S[subset]: cnt[l * cs + subset]
    uint32_t cs;
    unsigned long long tstart, deadline;  // globaltimer of the warp's start; budget in ns (0 = none)
    unsigned long long set_ops, alg_bytes, partial;
};

// Membership in a pinned table.
__device__ __forceinline__ bool pin_has(const uint32_t *t, uint32_t mode, uint32_t tw, uint32_t y) {
    if (mode == 1) return (t[y >> 5] >> (y & 31u)) & 1u;
    uint32_t h = (y * 2654435761u) & (tw - 1u);
    while (true) {  // load factor <= 1/2: an empty slot always ends the probe
        uint32_t k = t[h];
        if (k == y) return true;
        if (k == PIN_EMPTY) return false;
        h = (h + 1u) & (tw - 1u);
    }
}

// y ∈ N(m[j]) for a shared level j (pinned table when present).
template <bool STATS>
__device__ __forceinline__ bool in_level_list(const WarpState &W, const Ctx<STATS> &c, uint32_t j, uint32_t y) {
    if (j < 2 && W.pmode[j]) return pin_has(c.tab + j * c.tw, W.pmode[j], c.tw, y);
    if (W.hs[j] >= 0) return hub_has(c.g, W.hs[j], y);
    return contains(W.lptr[j], W.llen[j], y);
}

// Approximate probe cost of a shared level's list (for choosing base lists).
__device__ __forceinline__ uint32_t probe_cost(const WarpState &W, uint32_t j, uint32_t len) {
    if ((j < 2 && W.pmode[j]) || W.hs[j] >= 0) return 1u;
    return search_cost(len);
}

// Pins a sorted list into table ti (a bitmap over all vertices, or an
// open-addressing hash when it is at most half full); records the mode.
template <bool STATS>
__device__ void pin_list(WarpState &W, Ctx<STATS> &c, uint32_t ti, const uint32_t *p, uint32_t len) {
    const uint32_t lane = lane_id();
    uint32_t mode = c.tmode;
    if (mode == 2 && len * 2u > c.tw) mode = 0;
    uint32_t *t = c.tab + ti * c.tw;
    if (mode == 1) {
        for (uint32_t e = lane; e < len; e += 32) { uint32_t y = p[e]; atomicOr(&t[y >> 5], 1u << (y & 31u)); }
    } else if (mode == 2) {
        for (uint32_t e = lane; e < len; e += 32) {
            uint32_t y = p[e], h = (y * 2654435761u) & (c.tw - 1u);
            while (true) {
                uint32_t old = atomicCAS(&t[h], PIN_EMPTY, y);
                if (old == PIN_EMPTY || old == y) break;
                h = (h + 1u) & (c.tw - 1u);
            }
        }
    }
    if (STATS && mode) c.alg_bytes += 4ull * len;
    __syncwarp();
    if (lane == 0) W.pmode[ti] = mode;
    __syncwarp();
}

template <bool STATS>
__device__ void unpin_list(WarpState &W, Ctx<STATS> &c, uint32_t ti, const uint32_t *p, uint32_t len) {
    const uint32_t lane = lane_id();
    const uint32_t mode = W.pmode[ti];
    uint32_t *t = c.tab + ti * c.tw;
    if (mode == 1) {
        if (len * 2u < c.tw) {
            for (uint32_t e = lane; e < len; e += 32) { uint32_t y = p[e]; atomicAnd(&t[y >> 5], ~(1u << (y & 31u))); }
        } else {
            for (uint32_t w = lane; w < c.tw; w += 32) t[w] = 0u;
        }
    } else if (mode == 2) {
        for (uint32_t w = lane; w < c.tw; w += 32) t[w] = PIN_EMPTY;
    }
    __syncwarp();
    if (lane == 0) W.pmode[ti] = 0;
    __syncwarp();
}

// Pins N(m[0]) and N(m[1]) (levels probed inside the DFS).
template <bool STATS>
__device__ void pin_root(const DevPlan &P, WarpState &W, Ctx<STATS> &c) {
    for (uint32_t j = 0; j < 2; ++j)
        if ((P.pin_mask >> j) & 1u) pin_list(W, c, j, W.lptr[j], W.llen[j]);
}

// Exploration: version (j, i) list length and pointer.  The first parent's
// version is N(m[j]) itself; the others live in buffer slot[j][i].
template <bool STATS>
__device__ __forceinline__ uint32_t version_len(const DevPlan &P, const WarpState &W, const Ctx<STATS> &c, uint32_t j,
                                                uint32_t i) {
    const int s = P.slot[j][i];
    return s < 0 ? W.llen[j] : c.vs[s];
}

template <bool STATS>
__device__ __forceinline__ const uint32_t *version_ptr(const DevPlan &P, const WarpState &W, const Ctx<STATS> &c,
                                                       uint32_t j, uint32_t i) {
    int s = P.slot[j][i];
    if (s < 0) return W.lptr[j];
    return c.buf + (size_t)s * c.cap;
}

template <bool STATS>
__device__ void unpin_root(const DevPlan &P, WarpState &W, Ctx<STATS> &c) {
    for (uint32_t j = 0; j < 2; ++j)
        if (W.pmode[j]) unpin_list(W, c, j, W.lptr[j], W.llen[j]);
    if (W.pmode[2]) {
        if (W.hpin && P.join_style == SGE_JOIN_EXPLORATION)
            unpin_list(W, c, 2, version_ptr(P, W, c, 1, W.hpin), version_len(P, W, c, 1, W.hpin));
        else if (W.hpin) unpin_list(W, c, 2, c.buf + (size_t)W.hpin * c.cap, W.hcnt[W.hpin]);
        else unpin_list(W, c, 2, W.flist[2], W.fcnt[2]);
    }
    __syncwarp();
    if (lane_id() == 0) W.hpin = 0;
    __syncwarp();
}

__device__ __forceinline__ void set_match(const DevGraph &g, WarpState &W, uint32_t lv, uint32_t x) {
    // all lanes compute; lane 0 stores
    const uint32_t *p;
    uint32_t len;
    nbr(g, x, p, len);
    __syncwarp();
    if (lane_id() == 0) { W.m[lv] = x; W.lptr[lv] = p; W.llen[lv] = len; W.hs[lv] = hub_slot_of(g, x, len); }
    __syncwarp();
}

// Base list of level i for WCOJ: a reused stored list, or the parent list that
// is cheapest to scan while probing the others; `rest` returns the parents
// still to test.
template <bool STATS>
__device__ __forceinline__ void wcoj_base(const DevPlan &P, const WarpState &W, Ctx<STATS> &c, uint32_t i,
                                          const uint32_t *&bp, uint32_t &blen, uint32_t &rest) {
    if (P.base[i] >= 0) {
        uint32_t l = (uint32_t)P.base[i];
        bp = W.flist[l];
        blen = W.fcnt[l];
        rest = P.rest[i];
        return;
    }
    uint32_t best = 0;
    unsigned long long bestcost = ~0ull;
    for (uint32_t msk = P.parents[i]; msk; msk &= msk - 1) {
        uint32_t j = __ffs(msk) - 1;
        unsigned long long probes = 0;
        for (uint32_t o = P.parents[i] & ~(1u << j); o; o &= o - 1) {
            uint32_t q = __ffs(o) - 1;
            probes += probe_cost(W, q, W.llen[q]);
        }
        unsigned long long cost = (unsigned long long)W.llen[j] * (probes + 1);
        if (cost < bestcost) { bestcost = cost; best = j; }
    }
    bp = W.lptr[best];
    blen = W.llen[best];
    rest = P.parents[i] & ~(1u << best);
}

// Warp-cooperative filter of [bp, bp+blen) by membership in all parent lists
// of `rest` and by the exclusion set of level i; stores the survivors (in
// order) to out when STORE.  Returns the survivor count (warp-uniform).
template <bool STATS, bool STORE, bool EXCLUDE = true>
__device__ __forceinline__ uint32_t setop(const DevPlan &P, const WarpState &W, Ctx<STATS> &c, uint32_t i,
                                          const uint32_t *bp, uint32_t blen, uint32_t rest, uint32_t *out) {
    const uint32_t lane = lane_id();
    if (STATS) {
        c.set_ops += 1;
        c.alg_bytes += 4ull * blen;
        for (uint32_t msk = rest; msk; msk &= msk - 1) {
            const uint32_t j = __ffs(msk) - 1;
            c.alg_bytes += probe_bytes(blen, W.llen[j], (j < 2 && W.pmode[j]) || W.hs[j] >= 0);
        }
    }
    uint32_t total = 0;
    for (uint32_t off = 0; off < blen; off += 32) {
        uint32_t idx = off + lane;
        bool ok = idx < blen;
        uint32_t x = ok ? bp[idx] : 0u;
        for (uint32_t msk = rest; msk && ok; msk &= msk - 1) ok = in_level_list(W, c, __ffs(msk) - 1, x);
        if (EXCLUDE && ok) ok = !excluded(P, W, i, x);
        uint32_t bal = __ballot_sync(FULL_MASK, ok);
        if (STORE) {
            uint32_t p = total + __popc(bal & ((1u << lane) - 1u));
            if (ok && p < c.cap) out[p] = x;
        }
        total += __popc(bal);
    }
    return total;
}

// Builds level i's candidate list (WCOJ).  Returns false on overflow.
// A level that later levels reuse keeps its full intersection (bounds not
// applied); its own iteration range is that list trimmed by its bounds.
template <bool STATS>
__device__ __forceinline__ bool build_level_wcoj(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t i) {
    const uint32_t *bp;
    uint32_t blen, rest;
    wcoj_base(P, W, c, i, bp, blen, rest);
    const Bounds b = level_bounds(P, W, i);
    const bool keep = (P.keep_full >> i) & 1u;
    if (!keep) trim(bp, blen, b);
    const uint32_t *fp = bp;
    uint32_t fl = blen;
    if (rest != 0) {
        uint32_t *out = c.buf + (size_t)i * c.cap;
        uint32_t n = setop<STATS, true>(P, W, c, i, bp, blen, rest, out);
        if (n > c.cap) {
            if (lane_id() == 0) atomicOr(c.flags, FLAG_OVERFLOW);
            return false;
        }
        fp = out;
        fl = n;
    }
    // (a list taken without intersection keeps the exclusions for iteration time)
    const uint32_t *ip = fp;
    uint32_t il = fl;
    if (keep) trim(ip, il, b);
    __syncwarp();
    if (lane_id() == 0) { W.flist[i] = fp; W.fcnt[i] = fl; W.list[i] = ip; W.cnt[i] = il; }
    __syncwarp();
    return true;
}

// Hoisting: a tail level whose parents are all matched before the last
// enumerated level gets its full intersection computed once, right after its
// last parent is matched (bounds and exclusions are applied at the leaf).
template <bool STATS>
__device__ __forceinline__ bool hoist_after(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t j) {
    for (uint32_t msk = P.hoist_mask; msk; msk &= msk - 1) {
        const uint32_t i = __ffs(msk) - 1;
        if (P.hoist_at[i] != j) continue;
        const uint32_t *bp;
        uint32_t blen, rest;
        if (P.base[i] >= 0 && (uint32_t)P.base[i] <= j) {
            // a reused level's full list (built when that level was entered)
            bp = W.flist[P.base[i]];
            blen = W.fcnt[P.base[i]];
            rest = P.rest[i];
        } else {
            uint32_t best = 0;
            unsigned long long bestcost = ~0ull;
            for (uint32_t pm = P.parents[i]; pm; pm &= pm - 1) {
                const uint32_t q = __ffs(pm) - 1;
                unsigned long long probes = 0;
                for (uint32_t o = P.parents[i] & ~(1u << q); o; o &= o - 1)
                    probes += probe_cost(W, __ffs(o) - 1, W.llen[__ffs(o) - 1]);
                const unsigned long long cost = (unsigned long long)W.llen[q] * (probes + 1);
                if (cost < bestcost) { bestcost = cost; best = q; }
            }
            bp = W.lptr[best];
            blen = W.llen[best];
            rest = P.parents[i] & ~(1u << best);
        }
        uint32_t *out = c.buf + (size_t)i * c.cap;
        const uint32_t n = setop<STATS, true, false>(P, W, c, i, bp, blen, rest, out);
        __syncwarp();
        if (lane_id() == 0) W.hcnt[i] = n;
        __syncwarp();
        if (n > c.cap) {
            if (lane_id() == 0) atomicOr(c.flags, FLAG_OVERFLOW);
            return false;
        }
        // a list hoisted once per root is probed for every candidate below it:
        // pin it in the third table when that table is free
        if (j == 1 && c.tmode && !((P.pin_mask >> 2) & 1u) && W.hpin == 0u && W.pmode[2] == 0u) {
            pin_list(W, c, 2, out, n);
            __syncwarp();
            if (lane_id() == 0 && W.pmode[2]) W.hpin = i;
            __syncwarp();
        }
    }
    return true;
}


// Exploration: after level j is matched, intersect N(m[j]) into the running
// list of every later level that has j as a parent.  false = prune (empty) or
// overflow.  Levels past `upto` are left to the leaf.
template <bool STATS>
__device__ __forceinline__ bool explore_update(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t j) {
    const uint32_t lane = lane_id();
    for (uint32_t msk = P.after[j]; msk; msk &= msk - 1) {
        uint32_t i = __ffs(msk) - 1;
        uint32_t below = P.parents[i] & ((1u << j) - 1u);
        if (below == 0) {
            __syncwarp();
            __syncwarp();
            if (W.llen[j] == 0) return false;
            continue;
        }
        uint32_t pj = 31 - __clz(below);  // previous parent of i
        const uint32_t *prev = version_ptr(P, W, c, pj, i);
        uint32_t plen = version_len(P, W, c, pj, i);
        uint32_t *out = c.buf + (size_t)P.slot[j][i] * c.cap;
        uint32_t total = 0;
        // scan the running list, probe N(m[j]) (pinned table when present)
        const bool pinned = j < 2 && W.pmode[j];
        const bool scan_prev = pinned || plen <= W.llen[j];
        if (STATS) {
            c.set_ops += 1;
            c.alg_bytes += scan_prev ? 4ull * plen + probe_bytes(plen, W.llen[j], pinned || W.hs[j] >= 0)
                                     : 8ull + 4ull * (plen + W.llen[j]);
        }
        const uint32_t *sp = scan_prev ? prev : W.lptr[j];
        const uint32_t sl = scan_prev ? plen : W.llen[j];
        for (uint32_t off = 0; off < sl; off += 32) {
            uint32_t idx = off + lane;
            bool ok = idx < sl;
            uint32_t x = ok ? sp[idx] : 0u;
            if (ok) ok = scan_prev ? in_level_list(W, c, j, x) : contains(prev, plen, x);
            uint32_t bal = __ballot_sync(FULL_MASK, ok);
            uint32_t p = total + __popc(bal & ((1u << lane) - 1u));
            if (ok && p < c.cap) out[p] = x;
            total += __popc(bal);
        }
        __syncwarp();
        if (lane == 0) c.vs[P.slot[j][i]] = total;
        __syncwarp();
        if (total > c.cap) {
            if (lane == 0) atomicOr(c.flags, FLAG_OVERFLOW);
            return false;
        }
        if (total == 0) return false;
    }
    return true;
}

// Exploration: level i's candidates = its running list (last parent's version), trimmed.
template <bool STATS>
__device__ __forceinline__ void explore_level(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t i) {
    uint32_t lastp = 31 - __clz(P.parents[i]);
    const uint32_t *bp = version_ptr(P, W, c, lastp, i);
    uint32_t blen = version_len(P, W, c, lastp, i);
    Bounds b = level_bounds(P, W, i);
    __syncwarp();
    if (lane_id() == 0) { W.flist[i] = bp; W.fcnt[i] = blen; }
    trim(bp, blen, b);
    if (lane_id() == 0) { W.list[i] = bp; W.cnt[i] = blen; }
    __syncwarp();
}

// ---------------------------------------------------------------- leaf ----
// The leaf counts the tail levels [ne, k) for up to 32 candidates of the last
// enumerated level at once.  The candidates' (base element) work is flattened
// across the lanes, so a candidate with a long list does not stall the warp,
// and every probe into the root's lists is a shared-memory table lookup.
// Candidate l's value of level p is L.cm[l][p-L0] for p >= L0, W.m[p] below.

// List identity used by the leaf for the pinned stored list of level 2
// (distinct from the level numbers that name CSR lists).
constexpr int SRC_LEVEL2_LIST = 40;
constexpr int SRC_HOISTED = 41;

struct LeafCtx {
    uint32_t L0;
    bool explore;  // exploration: shared parents of a tail level are one running list
};

// Visits the lists whose intersection is tail level i's candidate set for
// candidate l: f(ptr, len, src, pinned) with src = level of the list, or -1 for
// the shared running list (exploration).  f returns false to stop.
template <bool STATS, class F>
__device__ __forceinline__ void for_tail_lists(const DevPlan &P, const WarpState &W, const LeafState &L,
                                               const Ctx<STATS> &c, const LeafCtx &lc, uint32_t l, uint32_t i, F f) {
    const uint32_t below = (1u << lc.L0) - 1u;
    uint32_t shared = P.parents[i] & below, cand = P.parents[i] & ~below;
    if (!lc.explore && ((P.hoist_mask >> i) & 1u)) {
        f(c.buf + (size_t)i * c.cap, W.hcnt[i], SRC_HOISTED, W.hpin == i);
        return;
    }
    if (lc.explore && shared) {
        // one running list for the shared parents; a first-parent version is
        // N(m[j]) itself, pinned when j is a root level
        const uint32_t lastp = 31 - __clz(shared);
        if (P.slot[lastp][i] < 0 && lastp < 2 && W.pmode[lastp]) {
            if (!f(W.lptr[lastp], W.llen[lastp], (int)lastp, true)) return;
        } else if (lastp == 1 && W.hpin == i) {
            if (!f(version_ptr(P, W, c, 1, i), version_len(P, W, c, 1, i), SRC_HOISTED, true)) return;
        } else if (!f(version_ptr(P, W, c, lastp, i), version_len(P, W, c, lastp, i), -1, false)) {
            return;
        }
        shared = 0;
    } else if (!lc.explore && P.base[i] >= 0) {
        // the stored list of an enumerated level (candidatesBefore) replaces its parents
        const uint32_t bl = (uint32_t)P.base[i];
        if (bl == 2 && W.pmode[2]) {
            if (!f(W.flist[bl], W.fcnt[bl], SRC_LEVEL2_LIST, true)) return;
        } else if (!f(W.flist[bl], W.fcnt[bl], -1, false)) {
            return;
        }
        shared &= P.rest[i];
        cand &= P.rest[i];
    }
    for (uint32_t msk = shared; msk; msk &= msk - 1) {
        const uint32_t j = __ffs(msk) - 1;
        if (!f(W.lptr[j], W.llen[j], (int)j, j < 2 && W.pmode[j] != 0)) return;
    }
    for (uint32_t msk = cand; msk; msk &= msk - 1) {
        const uint32_t j = __ffs(msk) - 1;
        if (!f(c.g.adj + L.ol[j - lc.L0][l].x, L.ol[j - lc.L0][l].y, (int)j, false)) return;
    }
}

// Lists, bounds and exclusions of one tail level, described once per leaf
// call: the same for every candidate except the lists of the candidates' own
// levels (slots), which are looked up per candidate.
__device__ __forceinline__ Bounds td_bounds(const TailDesc &D, const LeafState &L, uint32_t l) {
    Bounds b;
    b.lo = D.lo;
    b.hi = D.hi;
    b.has_lo = D.has_lo;
    b.has_hi = D.has_hi;
    if (D.lo_slots & 1u) b.lo = max(b.lo, L.cm[l][0]);
    if (D.lo_slots & 2u) b.lo = max(b.lo, L.cm[l][1]);
    if (D.hi_slots & 1u) b.hi = min(b.hi, L.cm[l][0]);
    if (D.hi_slots & 2u) b.hi = min(b.hi, L.cm[l][1]);
    return b;
}

// Bag relations: candidate l's key tuple selects its range of each trie's
// last level (the tail level's whole candidate list), stored in slot 2 + j.
// Returns the lookups' algorithmic bytes: the dense pair of offsets, then
// one probe word and one offset pair per further key.  (Inlined: a call
// would make every leaf save its live registers around it.)
__device__ __forceinline__ unsigned long long trie_lookups(const DevPlan &P, const WarpState &W, LeafState &L,
                                                        uint32_t L0, uint32_t l) {
    unsigned long long bytes = 0;
    for (uint32_t j = 0; j < P.ntrie; ++j) {
        const DevTrie &Tr = P.tries[P.trel[j]];
        uint32_t key[3];
        for (uint32_t q = 0; q < Tr.nkeys; ++q) {
            const uint32_t lv = P.tkey[j][q];
            key[q] = lv < L0 ? W.m[lv] : L.cm[l][lv - L0];
        }
        trie_range(Tr, key, L.ol[2 + j][l].x, L.ol[2 + j][l].y);
        bytes += 16ull + 20ull * (Tr.nkeys - 1u);
    }
    return bytes;
}

// Kinds 4..7 are per-candidate lists: slot k-4 of LeafState.ol, relative to
// D.ptr (the CSR neighbour array for slots 0/1, a trie's last level for 2/3).
__device__ __forceinline__ const uint32_t *td_ptr(const TailDesc &D, const LeafState &L, uint32_t q, uint32_t l) {
    const uint32_t k = D.kind[q];
    return k >= 4 ? D.ptr[q] + L.ol[k - 4][l].x : D.ptr[q];
}
__device__ __forceinline__ uint32_t td_len(const TailDesc &D, const LeafState &L, uint32_t q, uint32_t l) {
    const uint32_t k = D.kind[q];
    return k >= 4 ? L.ol[k - 4][l].y : D.len[q];
}

// y ∈ list q of the level for candidate l.
template <bool STATS>
__device__ __forceinline__ bool td_has(const TailDesc &D, const LeafState &L, const WarpState &W,
                                       const Ctx<STATS> &c, uint32_t q, uint32_t l, uint32_t y) {
    const uint32_t k = D.kind[q];
    if (k < 3) return pin_has(c.tab + k * c.tw, W.pmode[k], c.tw, y);
    if (k == 3) {
        const int32_t hs = D.lvl[q] >= 0 ? W.hs[D.lvl[q]] : -1;
        return hs >= 0 ? hub_has(c.g, hs, y) : contains(D.ptr[q], D.len[q], y);
    }
    const uint32_t sl = k - 4;
    const uint2 r = L.ol[sl][l];
    const int32_t hs = sl < 2 ? hub_slot_of(c.g, L.cm[l][sl], r.y) : -1;  // (a trie range has no bitmap)
    return hs >= 0 ? hub_has(c.g, hs, y) : contains(D.ptr[q] + r.x, r.y, y);
}

// Cost of probing list q for candidate l (1: pinned table or hub bitmap).
__device__ __forceinline__ uint32_t td_probe_cost(const TailDesc &D, const LeafState &L, const WarpState &W,
                                                  const DevGraph &g, uint32_t q, uint32_t l) {
    const uint32_t k = D.kind[q];
    if (k < 3) return 1u;
    if (k == 3) return (D.lvl[q] >= 0 && W.hs[D.lvl[q]] >= 0) ? 1u : search_cost(D.len[q]);
    const uint32_t len = L.ol[k - 4][l].y;
    return (k < 6 && len >= g.hub_min) ? 1u : search_cost(len);
}

__device__ __forceinline__ bool td_excluded(const TailDesc &D, const LeafState &L, uint32_t l, uint32_t y) {
    bool ex = false;
    for (uint32_t e = 0; e < D.nex; ++e) ex |= D.exv[e] == y;
    if (D.ex_slots & 1u) ex |= L.cm[l][0] == y;
    if (D.ex_slots & 2u) ex |= L.cm[l][1] == y;
    return ex;
}

// y ∈ the level's candidate set for candidate l (bounds, every list, exclusions).
template <bool STATS>
__device__ __forceinline__ bool td_member(const TailDesc &D, const LeafState &L, const WarpState &W,
                                          const Ctx<STATS> &c, uint32_t l, uint32_t y) {
    const Bounds b = td_bounds(D, L, l);
    if ((b.has_lo && y <= b.lo) || (b.has_hi && y >= b.hi)) return false;
    for (uint32_t q = 0; q < D.nsrc; ++q)
        if (!td_has(D, L, W, c, q, l, y)) return false;
    if (D.vlab && __ldg(D.vlab + y) != D.lab) return false;  // labeled plans
    return !td_excluded(D, L, l, y);
}

// Fills D for tail level i from the lists for_tail_lists visits.
template <bool STATS>
__device__ void tail_desc(const DevPlan &P, const WarpState &W, const LeafState &L, const Ctx<STATS> &c,
                          const LeafCtx &lc, uint32_t i, TailDesc &D) {
    uint32_t n = 0;
    if (P.ntrie && P.tri[i] >= 0) {
        // the bag relation's trie: each candidate's child range (looked up at
        // the start of the leaf) is the whole candidate list
        const uint32_t j = (uint32_t)P.tri[i];
        const DevTrie &T = P.tries[P.trel[j]];
        D.kind[0] = (uint8_t)(6 + j);
        D.lvl[0] = -1;
        D.ptr[0] = T.val[T.nkeys];
        D.len[0] = 0;
        n = 1;
    } else
    for_tail_lists(P, W, L, c, lc, 0, i, [&](const uint32_t *p, uint32_t len, int src, bool pinned) {
        uint32_t k = 3;
        if (pinned) k = (src == SRC_LEVEL2_LIST || src == SRC_HOISTED) ? 2u : (uint32_t)src;
        else if (src >= (int)lc.L0 && src < SRC_LEVEL2_LIST) k = 4u + (uint32_t)src - lc.L0;
        D.kind[n] = (uint8_t)k;
        D.lvl[n] = (int8_t)((k == 3 && src >= 0 && src < (int)lc.L0) ? src : -1);
        D.ptr[n] = k >= 4 ? c.g.adj : p;
        D.len[n] = len;
        ++n;
        return true;
    });
    D.nsrc = (uint8_t)n;
    D.vlab = P.vlab;
    D.lab = P.lab[i];
    D.has_lo = P.lower[i] != 0;
    D.has_hi = P.upper[i] != 0;
    uint32_t lo = 0, hi = 0xFFFFFFFFu, los = 0, his = 0, exs = 0, nex = 0;
    for (uint32_t msk = P.lower[i]; msk; msk &= msk - 1) {
        const uint32_t q = __ffs(msk) - 1;
        if (q >= lc.L0) los |= 1u << (q - lc.L0);
        else lo = max(lo, W.m[q]);
    }
    for (uint32_t msk = P.upper[i]; msk; msk &= msk - 1) {
        const uint32_t q = __ffs(msk) - 1;
        if (q >= lc.L0) his |= 1u << (q - lc.L0);
        else hi = min(hi, W.m[q]);
    }
    for (uint32_t msk = P.check[i]; msk; msk &= msk - 1) {
        const uint32_t q = __ffs(msk) - 1;
        if (q >= lc.L0) exs |= 1u << (q - lc.L0);
        else D.exv[nex++] = W.m[q];
    }
    D.lo = lo;
    D.hi = hi;
    D.lo_slots = (uint8_t)los;
    D.hi_slots = (uint8_t)his;
    D.ex_slots = (uint8_t)exs;
    D.nex = (uint8_t)nex;
}

template <bool STATS>
__device__ unsigned long long leaf_chunk(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t L0,
                                         uint32_t ncand) {
    LeafState &L = *c.L;
    const uint32_t lane = lane_id();
    const uint32_t ne = P.ne, T = P.T;
    LeafCtx lc{L0, P.join_style == SGE_JOIN_EXPLORATION && L0 > 0};
    const uint32_t passes = (P.tail_mode == SGE_TAIL_IEP) ? T : 1u;
    // lane t describes tail level ne+t (IEP passes probe the later levels too)
    __syncwarp();
    if (lane < passes) tail_desc(P, W, L, c, lc, ne + lane, c.td[lane]);
    unsigned long long tbytes = 0;
    if (P.ntrie && lane < ncand) tbytes = trie_lookups(P, W, L, L0, lane);
    if (P.tail_mode != SGE_TAIL_SINGLE) {
        for (uint32_t q = 0; q < c.cs; ++q) c.cnt[lane * c.cs + q] = 0;
    }
    __syncwarp();
    // inclusion–exclusion: S[A] (A a set of tail positions) is counted in the
    // pass of A's first position in pass order, probing the later ones; the
    // sums do not depend on the order, so levels with one list go last (the
    // last pass is then a plain count and the earlier passes probe them
    // through a pinned table or one search, not a scan)
    uint32_t ord = 0;  // 4 bits per pass: tail position
    if (passes > 1) {
        uint32_t n = 0;
        for (uint32_t q = 0; q < passes; ++q)
            if (c.td[q].nsrc != 1) ord |= q << (4 * n++);
        for (uint32_t q = 0; q < passes; ++q)
            if (c.td[q].nsrc == 1) ord |= q << (4 * n++);
    }
    unsigned long long single = 0, bytes = tbytes;
    for (uint32_t t = 0; t < passes; ++t) {
        const uint32_t tp = (ord >> (4 * t)) & 15u;
        const TailDesc &D = c.td[tp];
        // a tail level with a single list (after reuse) is counted without a
        // scan: range size minus the matched vertices inside it (numResults)
        // (the last inclusion–exclusion pass probes no other tail level, so it
        // is a plain count too)
        const bool direct = (P.tail_mode != SGE_TAIL_IEP || t + 1 == T) && D.nsrc == 1 && !P.vlab;
        if (direct) {
            if (lane < ncand) {
                const uint32_t *fp = td_ptr(D, L, 0, lane);
                const uint32_t fl = td_len(D, L, 0, lane);
                const Bounds b = td_bounds(D, L, lane);
                const uint32_t *bp = fp;
                uint32_t blen = fl;
                trim(bp, blen, b);
                uint32_t cnt = blen;
                auto drop = [&](uint32_t v) {
                    if ((!b.has_lo || v > b.lo) && (!b.has_hi || v < b.hi) && td_has(D, L, W, c, 0, lane, v)) --cnt;
                };
                for (uint32_t e = 0; e < D.nex; ++e) drop(D.exv[e]);
                if (D.ex_slots & 1u) drop(L.cm[lane][0]);
                if (D.ex_slots & 2u) drop(L.cm[lane][1]);
                if (P.tail_mode == SGE_TAIL_SINGLE) single += cnt;
                else if (P.tail_mode == SGE_TAIL_CHOOSE) c.cnt[(lane) * c.cs + (1)] = cnt;
                else c.cnt[(lane) * c.cs + (1u << tp)] = cnt;
                if (STATS) bytes += 4ull * (2u + __popc(P.check[ne + tp])) * (31u - __clz(blen + 1u));
            }
            __syncwarp();
            continue;
        }
        // 1. the warp scans one source per candidate, the one with the least
        // cost summed over the candidates (scan length × probes of the
        // others), trimmed by each candidate's bounds; the others are probed
        uint32_t bq = 0;
        {
            unsigned long long allp = 0, best = ~0ull;
            if (lane < ncand)
                for (uint32_t q = 0; q < D.nsrc; ++q) allp += td_probe_cost(D, L, W, c.g, q, lane);
            for (uint32_t q = 0; q < D.nsrc; ++q) {
                unsigned long long cost = 0;
                if (lane < ncand) {
                    const uint32_t len = td_len(D, L, q, lane);
                    const unsigned long long own = td_probe_cost(D, L, W, c.g, q, lane);
                    cost = (unsigned long long)len * (allp - own + 1);
                }
                cost = warp_sum_u64(cost);
                if (cost < best) { best = cost; bq = q; }
            }
        }
        const uint32_t *bp = nullptr;
        uint32_t blen = 0;
        if (lane < ncand) {
            bp = td_ptr(D, L, bq, lane);
            blen = td_len(D, L, bq, lane);
            trim(bp, blen, td_bounds(D, L, lane));
            if (STATS) {  // the scanned range, and each other list probed once per element of it
                bytes += 4ull * blen;
                for (uint32_t q = 0; q < D.nsrc; ++q)
                    if (q != bq) bytes += probe_bytes(blen, td_len(D, L, q, lane), td_probe_cost(D, L, W, c.g, q, lane) == 1);
            }
        }
        L.bptr[lane] = bp;
        uint32_t incl = blen;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl += v;
        }
        L.pref[lane] = incl;
        const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
        __syncwarp();
        const uint32_t ns = D.nsrc;
        const uint32_t nu = (P.tail_mode == SGE_TAIL_IEP) ? (T - 1 - t) : 0u;
        // 2. flattened scan: element j belongs to the candidate l with
        // pref[l-1] <= j < pref[l].  A lane's elements of one candidate are
        // consecutive, so it counts S[{tp}] (and, with one later level,
        // S[{tp, up}]) in registers and adds them when its candidate changes
        uint32_t l = 0;
        const uint32_t i0 = (P.tail_mode == SGE_TAIL_CHOOSE) ? 1u : (1u << tp);
        const uint32_t up1 = nu ? (ord >> (4 * (t + 1))) & 15u : 0u;
        const uint32_t i1 = i0 | (1u << up1);
        uint32_t al = 0, a0 = 0, a1 = 0;
        auto flush = [&]() {
            if (a0) atomicAdd(&c.cnt[al * c.cs + i0], a0);
            if (a1) atomicAdd(&c.cnt[al * c.cs + i1], a1);
            a0 = a1 = 0;
        };
        // (a warp-uniform loop, so the periodic time check's shuffle is converged)
        for (uint32_t j0 = 0; j0 < total; j0 += 32) {
            if (j0 && (j0 & 0x3FFFu) == 0 && out_of_time(c)) break;
            const uint32_t j = j0 + lane;
            if (j >= total) break;
            while (L.pref[l] <= j) ++l;
            const uint32_t start = l ? L.pref[l - 1] : 0u;
            const uint32_t y = L.bptr[l][j - start];
            bool ok = true;
            for (uint32_t q = 0; q < ns && ok; ++q)
                if (q != bq) ok = td_has(D, L, W, c, q, l, y);
            if (ok) ok = !td_excluded(D, L, l, y);
            if (ok && P.vlab) ok = __ldg(P.vlab + y) == D.lab;
            if (!ok) continue;
            if (P.tail_mode == SGE_TAIL_SINGLE) {
                ++single;
                continue;
            }
            if (l != al) {
                flush();
                al = l;
            }
            ++a0;
            if (nu == 1) {
                a1 += td_member(c.td[up1], L, W, c, l, y) ? 1u : 0u;
            } else if (nu > 1) {
                uint32_t fm = 0;
                for (uint32_t q = t + 1; q < t + 1 + nu; ++q) {
                    const uint32_t up = (ord >> (4 * q)) & 15u;
                    fm |= (uint32_t)td_member(c.td[up], L, W, c, l, y) << up;
                }
                // every nonempty subset s of the later positions y belongs to: S[{tp} ∪ s] += 1
                for (uint32_t sub = fm; sub; sub = (sub - 1) & fm) atomicAdd(&c.cnt[l * c.cs + (i0 | sub)], 1u);
            }
        }
        if (P.tail_mode != SGE_TAIL_SINGLE) flush();
        __syncwarp();
    }
    // 3. per-candidate results
    unsigned long long r = 0;
    if (P.tail_mode == SGE_TAIL_SINGLE) {
        r = single;
    } else if (lane < ncand) {
        if (P.tail_mode == SGE_TAIL_CHOOSE) {
            r = choose_leaf(c.cnt[(lane) * c.cs + (1)], T, P.choose_wrap, c.flags);
        } else {
            for (uint32_t p = 0; p < P.nparts; ++p) {
                unsigned long long term = (unsigned long long)(long long)P.part_coef[p];
                for (uint32_t bk = 0; bk < P.part_nblocks[p]; ++bk) term *= c.cnt[lane * c.cs + P.part_block[p][bk]];
                r += term;
            }
        }
    }
    if (STATS) {
        c.alg_bytes += warp_sum_u64(bytes);
        c.set_ops += (unsigned long long)ncand * passes;
    }
    __syncwarp();
    return warp_sum_u64(r);
}

// Leaf over up to 32 root edges (plans with only two enumerated levels):
// lane l < n holds root (u, v).
template <bool STATS>
__device__ unsigned long long leaf_roots(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t n, uint32_t u,
                                         uint32_t v) {
    LeafState &L = *c.L;
    const uint32_t lane = lane_id();
    if (lane < n) {
        L.cm[lane][0] = u;
        L.cm[lane][1] = v;
        nbr_off(c.g, u, L.ol[0][lane].x, L.ol[0][lane].y);
        nbr_off(c.g, v, L.ol[1][lane].x, L.ol[1][lane].y);
    }
    __syncwarp();
    return leaf_chunk(P, W, c, 0, n);
}

// Pair step helpers.  The leaf takes up to 32 queued (x, y) pairs as its
// candidates with L0 = a: cm[l][0] = x (level a), cm[l][1] = y (level a+1).
template <bool STATS>
__device__ __forceinline__ unsigned long long pair_flush(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t a,
                                                         uint32_t nq) {
    LeafState &L = *c.L;
    PairState &S = *c.PS;
    const uint32_t lane = lane_id();
    if (lane < nq) {
        const uint32_t x = S.qx[lane], y = S.qy[lane];
        L.cm[lane][0] = x;
        L.cm[lane][1] = y;
        if ((P.tail_par >> a) & 1u) nbr_off(c.g, x, L.ol[0][lane].x, L.ol[0][lane].y);
        if ((P.tail_par >> (a + 1)) & 1u) nbr_off(c.g, y, L.ol[1][lane].x, L.ol[1][lane].y);
    }
    __syncwarp();
    return leaf_chunk(P, W, c, a, nq);
}

// Level a+1's lists that are the same for every candidate x of level a
// (matched levels below a only), its exclusion values, and whether N(x) is
// one of its lists.  Mirrors build_level_wcoj / explore_level for level a+1.
template <bool STATS>
__device__ __forceinline__ void pair_sources(const DevPlan &P, const WarpState &W, const Ctx<STATS> &c,
                                             uint32_t a) {
    PairState &S = *c.PS;
    const uint32_t i = a + 1;
    if (lane_id() == 0) {
        uint32_t ns = 0, xpar = (P.parents[i] >> a) & 1u;
        if (P.join_style == SGE_JOIN_EXPLORATION) {
            const uint32_t shared = P.parents[i] & ((1u << a) - 1u);
            if (shared) {
                const uint32_t lastp = 31 - __clz(shared);
                S.shub[ns] = -1;
                if (P.slot[lastp][i] < 0 && lastp < 2 && W.pmode[lastp]) {
                    S.sptr[ns] = W.lptr[lastp]; S.slen[ns] = W.llen[lastp]; S.stab[ns] = (int32_t)lastp;
                } else {
                    S.sptr[ns] = version_ptr(P, W, c, lastp, i); S.slen[ns] = version_len(P, W, c, lastp, i); S.stab[ns] = -1;
                    if (P.slot[lastp][i] < 0) S.shub[ns] = W.hs[lastp];
                }
                ++ns;
            }
        } else {
            uint32_t rem = P.parents[i];
            if (P.base[i] >= 0) {
                const uint32_t bl = (uint32_t)P.base[i];
                S.sptr[ns] = W.flist[bl];
                S.slen[ns] = W.fcnt[bl];
                S.stab[ns] = (bl == 2 && ((P.pin_mask >> 2) & 1u) && W.pmode[2]) ? 2 : -1;
                S.shub[ns] = -1;
                ++ns;
                rem = P.rest[i];
            }
            for (uint32_t msk = rem & ((1u << a) - 1u); msk; msk &= msk - 1) {
                const uint32_t j = __ffs(msk) - 1;
                S.sptr[ns] = W.lptr[j];
                S.slen[ns] = W.llen[j];
                S.stab[ns] = (j < 2 && W.pmode[j]) ? (int32_t)j : -1;
                S.shub[ns] = W.hs[j];
                ++ns;
            }
            xpar = (rem >> a) & 1u;
        }
        uint32_t nex = 0;
        for (uint32_t msk = P.check[i] & ((1u << a) - 1u); msk; msk &= msk - 1) S.exv[nex++] = W.m[__ffs(msk) - 1];
        S.ns = ns;
        S.xpar = xpar;
        S.nex = nex;
    }
    __syncwarp();
}

// y ∈ list q of level a+1 (shared list q, or N(x) for q = -1).
template <bool STATS>
__device__ __forceinline__ bool pair_in(const WarpState &W, const Ctx<STATS> &c, const PairState &S, int q,
                                        uint32_t l, uint32_t y) {
    if (q < 0) return csr_has(c.g, S.x[l], c.g.adj + S.xo[l], S.xl[l], y);
    if (S.stab[q] >= 0) return pin_has(c.tab + S.stab[q] * c.tw, W.pmode[S.stab[q]], c.tw, y);
    if (S.shub[q] >= 0) return hub_has(c.g, S.shub[q], y);
    return contains(S.sptr[q], S.slen[q], y);
}

// v ∈ the inline tail's single list for batch candidate l.
template <bool STATS>
__device__ __forceinline__ bool pair_tail_has(const WarpState &W, const Ctx<STATS> &c, const PairState &S,
                                              uint32_t l, uint32_t v) {
    const TailDesc &D = S.ptd;
    const uint32_t k = D.kind[0];
    if (k < 3) return pin_has(c.tab + k * c.tw, W.pmode[k], c.tw, v);
    if (k == 3) {
        const int32_t hs = D.lvl[0] >= 0 ? W.hs[D.lvl[0]] : -1;
        return hs >= 0 ? hub_has(c.g, hs, v) : contains(D.ptr[0], D.len[0], v);
    }
    return csr_has(c.g, S.x[l], c.g.adj + S.xo[l], S.xl[l], v);
}

// The last two enumerated levels as one step: for 32 candidates x of level
// a = ne-2 at a time, level a+1's candidate sets are generated by one scan
// flattened over (x, element) like the leaf's, and every surviving (x, y)
// joins a queue the leaf drains 32 pairs at a time.  Same pairs as entering
// level a+1 once per x (build_level_wcoj / explore_update + explore_level),
// without one warp-wide set operation and one short leaf call per x.
// Returns false on timeout.
template <bool STATS>
__device__ bool pair_level(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t a, unsigned long long &acc) {
    PairState &S = *c.PS;
    const uint32_t lane = lane_id();
    const uint32_t i = a + 1;
    const uint32_t n = W.cnt[a];
    const uint32_t *lst = W.list[a];
    pair_sources(P, W, c, a);
    // inline tail: the tail level's single list does not depend on y, so the
    // pair's count is x's count minus y itself when y is in x's range and list
    bool inl = false;
    if (P.pair_direct) {
        if (lane == 0) {
            const LeafCtx lc{a, P.join_style == SGE_JOIN_EXPLORATION};
            tail_desc(P, W, *c.L, c, lc, P.ne, S.ptd);
        }
        __syncwarp();
        inl = S.ptd.nsrc == 1;
    }
    const TailDesc &D = S.ptd;
    const uint32_t ns = S.ns, xpar = S.xpar, nex = S.nex;
    const bool ex_x = (P.check[i] >> a) & 1u;
    uint32_t qn = 0;
    unsigned long long isum = 0;
    bool ok = true;
    for (uint32_t b0 = W.pos[a]; b0 < n && ok; b0 += 32) {
        if (out_of_time(c)) { ok = false; break; }
        // 1. this batch's level-a candidates, compacted
        const uint32_t idx = b0 + lane;
        bool valid = idx < n;
        const uint32_t xv = valid ? lst[idx] : 0u;
        if (valid) valid = !excluded(P, W, a, xv);  // (labeled plans take no pair step)
        const uint32_t bal = __ballot_sync(FULL_MASK, valid);
        const uint32_t nc = __popc(bal);
        if (valid) S.x[__popc(bal & ((1u << lane) - 1u))] = xv;
        __syncwarp();
        if (STATS) { c.partial += nc; c.set_ops += nc; }
        // 2. per candidate: N(x); the warp scans one source for every
        // candidate (the least cost summed over the batch: scan length ×
        // probes of the others), trimmed by level a+1's bounds
        const uint32_t *bp = nullptr;
        uint32_t blen = 0;
        int32_t bsrc = -1;
        uint32_t x = 0, xl = 0;
        unsigned long long pbytes = 0;  // this lane's algorithmic bytes (instrumented kernel)
        const uint32_t *xp = nullptr;
        if (lane < nc) {
            x = S.x[lane];
            nbr(c.g, x, xp, xl);
            S.xo[lane] = (uint32_t)(xp - c.g.adj);
            S.xl[lane] = xl;
        }
        {
            unsigned long long allp = 0;
            for (uint32_t q = 0; q < ns; ++q) allp += (S.stab[q] >= 0 || S.shub[q] >= 0) ? 1u : search_cost(S.slen[q]);
            const unsigned long long xcost = xl >= c.g.hub_min ? 1u : search_cost(xl);
            if (xpar) allp += xcost;
            unsigned long long best = ~0ull;
            for (uint32_t q = 0; q < ns; ++q) {
                const unsigned long long own = (S.stab[q] >= 0 || S.shub[q] >= 0) ? 1u : search_cost(S.slen[q]);
                const unsigned long long cost =
                    warp_sum_u64(lane < nc ? (unsigned long long)S.slen[q] * (allp - own + 1) : 0ull);
                if (cost < best) { best = cost; bsrc = (int32_t)q; }
            }
            if (xpar) {
                const unsigned long long cost = warp_sum_u64(lane < nc ? (unsigned long long)xl * (allp - xcost + 1) : 0ull);
                if (cost < best) { best = cost; bsrc = -1; }
            }
        }
        if (lane < nc) {
            bp = bsrc < 0 ? xp : S.sptr[bsrc];
            blen = bsrc < 0 ? xl : S.slen[bsrc];
            if (STATS) {
                unsigned long long by = 4ull * blen;
                for (uint32_t q = 0; q < ns; ++q)
                    if ((int32_t)q != bsrc) by += probe_bytes(blen, S.slen[q], S.stab[q] >= 0 || S.shub[q] >= 0);
                if (xpar && bsrc != -1) by += probe_bytes(blen, xl, xl >= c.g.hub_min);
                pbytes += by;
            }
            Bounds b;
            b.lo = 0;
            b.hi = 0xFFFFFFFFu;
            b.has_lo = P.lower[i] != 0;
            b.has_hi = P.upper[i] != 0;
            for (uint32_t msk = P.lower[i]; msk; msk &= msk - 1) {
                const uint32_t p = __ffs(msk) - 1;
                b.lo = max(b.lo, p == a ? x : W.m[p]);
            }
            for (uint32_t msk = P.upper[i]; msk; msk &= msk - 1) {
                const uint32_t p = __ffs(msk) - 1;
                b.hi = min(b.hi, p == a ? x : W.m[p]);
            }
            trim(bp, blen, b);
            if (inl) {
                // x's tail count (range of the single list minus the matched values inside)
                const uint32_t *fp = D.kind[0] == 4 ? xp : D.ptr[0];
                const uint32_t fl = D.kind[0] == 4 ? xl : D.len[0];
                Bounds tb;
                tb.lo = D.lo;
                tb.hi = D.hi;
                tb.has_lo = D.has_lo;
                tb.has_hi = D.has_hi;
                if (D.lo_slots & 1u) tb.lo = max(tb.lo, x);
                if (D.hi_slots & 1u) tb.hi = min(tb.hi, x);
                const uint32_t *tp = fp;
                uint32_t tl = fl;
                trim(tp, tl, tb);
                uint32_t cnt = tl;
                for (uint32_t e = 0; e < D.nex + ((D.ex_slots & 1u) ? 1u : 0u); ++e) {
                    const uint32_t v = e < D.nex ? D.exv[e] : x;
                    if ((!tb.has_lo || v > tb.lo) && (!tb.has_hi || v < tb.hi) && pair_tail_has(W, c, S, lane, v))
                        --cnt;
                }
                S.tr[lane] = cnt;
                if (STATS) pbytes += 4ull * (2u + D.nex) * (31u - __clz(fl + 1u));
            }
        }
        S.bp[lane] = bp;
        if (STATS) c.alg_bytes += warp_sum_u64(pbytes);  // all lanes, after the per-candidate branch
        uint32_t incl = blen;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl += v;
        }
        S.pref[lane] = incl;
        const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
        __syncwarp();
        // 3. flattened scan; survivors are appended to the pair queue
        uint32_t l = 0;
        for (uint32_t j0 = 0; j0 < total; j0 += 32) {
            if (j0 && (j0 & 0x1FFFu) == 0 && out_of_time(c)) { ok = false; break; }
            const uint32_t j = j0 + lane;
            bool keep = j < total;
            uint32_t y = 0;
            if (keep) {
                while (S.pref[l] <= j) ++l;
                const uint32_t start = l ? S.pref[l - 1] : 0u;
                y = S.bp[l][j - start];
                for (uint32_t q = 0; q < ns && keep; ++q)
                    if ((int32_t)q != bsrc) keep = pair_in(W, c, S, (int)q, l, y);
                if (keep && xpar && bsrc != -1) keep = pair_in(W, c, S, -1, l, y);
                for (uint32_t e = 0; e < nex && keep; ++e) keep = y != S.exv[e];
                if (keep && ex_x) keep = y != S.x[l];
            }
            if (inl) {
                if (keep) {
                    uint32_t r = S.tr[l];
                    // y itself, when the tail excludes it and it lies in x's range and list
                    const uint32_t xl0 = S.x[l];
                    const uint32_t tlo = (D.lo_slots & 1u) ? max(D.lo, xl0) : D.lo;
                    const uint32_t thi = (D.hi_slots & 1u) ? min(D.hi, xl0) : D.hi;
                    if ((D.ex_slots & 2u) && (!D.has_lo || y > tlo) && (!D.has_hi || y < thi) &&
                        pair_tail_has(W, c, S, l, y))
                        --r;
                    isum += r;
                }
                if (STATS) {
                    const uint32_t kb = __ballot_sync(FULL_MASK, keep);
                    c.partial += __popc(kb);
                    c.set_ops += __popc(kb);
                }
                continue;
            }
            const uint32_t kb = __ballot_sync(FULL_MASK, keep);
            if (keep) {
                const uint32_t p = qn + __popc(kb & ((1u << lane) - 1u));
                S.qx[p] = S.x[l];
                S.qy[p] = y;
            }
            qn += __popc(kb);
            if (STATS) c.partial += __popc(kb);
            __syncwarp();
            if (qn >= 32) {
                acc += pair_flush(P, W, c, a, 32u);
                // move the remainder (< 32 pairs) to the front of the queue
                const uint32_t rx = S.qx[32 + lane], ry = S.qy[32 + lane];
                __syncwarp();
                if (lane < qn - 32) { S.qx[lane] = rx; S.qy[lane] = ry; }
                qn -= 32;
                __syncwarp();
            }
        }
    }
    if (ok && qn) acc += pair_flush(P, W, c, a, qn);
    if (inl) acc += warp_sum_u64(isum);
    return ok;
}

// One root edge: DFS over levels 2..ne-2; the candidates of level ne-1 go to
// the leaf 32 at a time.
// Past the time budget?  (all lanes agree: lane 0 reads the clock)
template <bool STATS>
__device__ __forceinline__ bool out_of_time(Ctx<STATS> &c) {
    if (!c.deadline) return false;
    unsigned long long now = 0;
    if (lane_id() == 0) now = globaltimer_ns();
    now = __shfl_sync(FULL_MASK, now, 0);
    if (now - c.tstart <= c.deadline) return false;
    if (lane_id() == 0) atomicOr(c.flags, FLAG_TIMEOUT);
    return true;
}

// r2b/r2e restrict the level-2 candidates processed, and p3 of np3 the part
// of each level-3 list (a heavy root is split into tasks over ranges of its
// level-2 list and equal parts of the level-3 lists below them).
template <bool STATS>
__device__ unsigned long long run_root(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t u, uint32_t v,
                                       uint32_t r2b = 0u, uint32_t r2e = 0xFFFFFFFFu, uint32_t p3 = 0u,
                                       uint32_t np3 = 1u) {
    const uint32_t lane = lane_id();
    const uint32_t ne = P.ne;
    if (ne == 2) return leaf_roots(P, W, c, 1u, u, v);
    const bool explore = P.join_style == SGE_JOIN_EXPLORATION;
    const uint32_t L0 = ne - 1;
    const uint32_t Lt = P.pair ? ne - 2 : L0;  // level whose candidates end the DFS
    LeafState &L = *c.L;
    set_match(c.g, W, 0, u);
    set_match(c.g, W, 1, v);
    if (P.pin_mask) pin_root(P, W, c);
    unsigned long long acc = 0;
    bool ok = true;
    if (explore) {
        ok = explore_update(P, W, c, 0) && explore_update(P, W, c, 1);
        if (ok && P.epin && c.tmode && W.pmode[2] == 0u) {
            pin_list(W, c, 2, version_ptr(P, W, c, 1, P.epin), version_len(P, W, c, 1, P.epin));
            __syncwarp();
            if (lane == 0 && W.pmode[2]) W.hpin = P.epin;
            __syncwarp();
        }
    } else if (P.hoist_mask) {
        ok = hoist_after(P, W, c, 1);
    }
    uint32_t lv = 2;
    if (ok) {
        if (explore) explore_level(P, W, c, lv);
        else ok = build_level_wcoj(P, W, c, lv);
        // level 2's list is built once per root; pin it when later levels reuse it
        if (ok && ((P.pin_mask >> 2) & 1u)) pin_list(W, c, 2, W.flist[2], W.fcnt[2]);
    }
    if (ok) {
        __syncwarp();
        if (lane == 0) {
            W.cnt[2] = min(W.cnt[2], r2e);
            W.pos[2] = min(r2b, W.cnt[2]);
        }
        __syncwarp();
    }
    while (ok) {
        if (lv == Lt && P.pair) {
            ok = pair_level(P, W, c, lv, acc);
            if (lv == 2) break;
            --lv;
            continue;
        }
        if (lv == L0) {
            const uint32_t n = W.cnt[lv];
            const uint32_t *lst = W.list[lv];
            for (uint32_t b0 = W.pos[lv]; b0 < n; b0 += 32) {
                if (out_of_time(c)) { ok = false; break; }
                const uint32_t idx = b0 + lane;
                bool valid = idx < n;
                const uint32_t x = valid ? lst[idx] : 0u;
                if (valid) valid = !rejected(P, W, lv, x);
                const uint32_t bal = __ballot_sync(FULL_MASK, valid);
                const uint32_t nc = __popc(bal);
                if (valid) {
                    const uint32_t rk = __popc(bal & ((1u << lane) - 1u));
                    L.cm[rk][0] = x;
                    if ((P.tail_par >> L0) & 1u) nbr_off(c.g, x, L.ol[0][rk].x, L.ol[0][rk].y);
                }
                __syncwarp();
                if (nc) acc += leaf_chunk(P, W, c, L0, nc);
                if (STATS) c.partial += nc;
            }
            if (lv == 2) break;
            --lv;
            continue;
        }
        const uint32_t pos = W.pos[lv];
        if (pos >= W.cnt[lv]) {
            if (lv == 2) break;
            --lv;
            continue;
        }
        if (out_of_time(c)) { ok = false; break; }
        const uint32_t x = W.list[lv][pos];
        __syncwarp();
        if (lane == 0) W.pos[lv] = pos + 1;
        __syncwarp();
        if (rejected(P, W, lv, x)) continue;
        set_match(c.g, W, lv, x);
        if (STATS) c.partial += 1;
        if (explore && !explore_update(P, W, c, lv)) continue;
        if (!explore && P.hoist_mask && !hoist_after(P, W, c, lv)) { ok = false; break; }
        ++lv;
        if (explore) explore_level(P, W, c, lv);
        else if (!build_level_wcoj(P, W, c, lv)) { ok = false; break; }
        __syncwarp();
        if (lane == 0) {
            W.pos[lv] = 0;
            if (lv == 3 && np3 > 1) {  // this task's part of the level-3 list
                const unsigned long long n3 = W.cnt[3];
                W.pos[3] = (uint32_t)(n3 * p3 / np3);
                W.cnt[3] = (uint32_t)(n3 * (p3 + 1) / np3);
            }
        }
        __syncwarp();
    }
    if (P.pin_mask || W.hpin) unpin_root(P, W, c);
    return ok ? acc : 0ull;
}

// Per-warp shared-memory carve-up: WarpState | LeafState | PairState |
// ntd tail descriptors | 32 × cs leaf counters | 3 pinned-list tables.  The
// plans themselves stay in global memory (read through L1): the fewer bytes a
// warp holds, the more warps are resident, and the DFS is latency-bound.
__host__ __device__ constexpr size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }
__host__ __device__ inline size_t warp_smem_bytes(uint32_t tw, uint32_t ntd, uint32_t cs, uint32_t nvs,
                                                  uint32_t ntr = 0) {
    return align128(sizeof(WarpState)) + align128(leaf_bytes(ntr)) + align128(sizeof(PairState)) +
           align128(ntd * sizeof(TailDesc)) + align128(32ull * cs * sizeof(uint32_t)) +
           align128(nvs * sizeof(uint32_t)) + align128(3ull * tw * sizeof(uint32_t));
}

template <bool STATS>
__device__ __forceinline__ WarpState &setup_warp(unsigned char *smem, uint32_t wib, uint32_t tw, uint32_t tmode,
                                                 uint32_t ntd, uint32_t cs, uint32_t nvs, Ctx<STATS> &c,
                                                 uint32_t ntr = 0) {
    unsigned char *base = smem + (size_t)wib * warp_smem_bytes(tw, ntd, cs, nvs, ntr);
    WarpState &W = *reinterpret_cast<WarpState *>(base);
    base += align128(sizeof(WarpState));
    c.L = reinterpret_cast<LeafState *>(base);
    base += align128(leaf_bytes(ntr));
    c.PS = reinterpret_cast<PairState *>(base);
    base += align128(sizeof(PairState));
    c.td = reinterpret_cast<TailDesc *>(base);
    base += align128(ntd * sizeof(TailDesc));
    c.cnt = reinterpret_cast<uint32_t *>(base);
    c.cs = cs;
    base += align128(32ull * cs * sizeof(uint32_t));
    c.vs = reinterpret_cast<uint32_t *>(base);
    base += align128(nvs * sizeof(uint32_t));
    c.tab = reinterpret_cast<uint32_t *>(base);
    c.tw = tw;
    c.tmode = tmode;
    const uint32_t fill = tmode == 2 ? PIN_EMPTY : 0u;
    for (uint32_t w = lane_id(); w < 3 * tw; w += 32) c.tab[w] = fill;
    if (lane_id() == 0) { W.pmode[0] = 0; W.pmode[1] = 0; W.pmode[2] = 0; W.hpin = 0; }
    __syncwarp();
    return W;
}

// Tail descriptors and counters one plan's leaf needs.
__host__ __device__ inline uint32_t plan_ntd(const DevPlan &d) { return d.tail_mode == SGE_TAIL_IEP ? d.T : 1u; }
__host__ __device__ inline uint32_t plan_nvs(const DevPlan &d) {
    return d.join_style == SGE_JOIN_EXPLORATION ? d.nbufs : 1u;
}
__host__ __device__ inline uint32_t plan_cs(const DevPlan &d) {
    return d.tail_mode == SGE_TAIL_IEP ? (1u << d.T) : (d.tail_mode == SGE_TAIL_CHOOSE ? 2u : 1u);
}

// Root task t of plan P -> directed root edge (u, v).  A sample (or a
// rank's share) is the undirected edges e ≡ root_offset (mod root_stride);
// a plan whose root is unordered (ANY) runs both orientations of each, so
// the sample does not depend on which end of the root a plan matches first.
__device__ __forceinline__ uint2 root_edge(const DevGraph &g, const DevPlan &P, unsigned long long t) {
    uint2 e;
    if (P.root_kind == SGE_ROOT_ANY) {
        e = g.edges[P.root_offset + (t >> 1) * P.root_stride];
        if (t & 1) { uint32_t tmp = e.x; e.x = e.y; e.y = tmp; }
    } else {
        e = g.edges[P.root_offset + t * P.root_stride];
        if (P.root_kind == SGE_ROOT_DESC) { uint32_t tmp = e.x; e.x = e.y; e.y = tmp; }
    }
    return e;
}

// A root kept by the degree cap: both endpoints of degree <= root_maxdeg.
__device__ __forceinline__ bool root_kept(const DevGraph &g, const DevPlan &P, uint2 e) {
    if (P.vlab && (__ldg(P.vlab + e.x) != P.lab[0] || __ldg(P.vlab + e.y) != P.lab[1])) return false;
    if (!P.root_maxdeg) return true;
    return __ldg(g.off + e.x + 1) - __ldg(g.off + e.x) <= P.root_maxdeg &&
           __ldg(g.off + e.y + 1) - __ldg(g.off + e.y) <= P.root_maxdeg;
}

// Upper bound on a root's level-2 list: the smaller degree among level 2's
// root parents.
__device__ __forceinline__ uint32_t level2_bound(const DevGraph &g, const DevPlan &P, uint2 e) {
    uint32_t ub = 0xFFFFFFFFu;
    if (P.split_par & 1u) ub = min(ub, __ldg(g.off + e.x + 1) - __ldg(g.off + e.x));
    if (P.split_par & 2u) ub = min(ub, __ldg(g.off + e.y + 1) - __ldg(g.off + e.y));
    return ub;
}

// Heavy roots deferred by phase 0: their ids, per-plan counts, and the
// exclusive prefix of their task counts (phase 1 numbers tasks densely).
struct HeavyBuf {
    uint32_t *cnt;             // per plan
    uint32_t *ids;             // plan p's list at p * cap
    unsigned long long *pre;   // task-count prefix, parallel to ids
    unsigned long long *tot;   // per plan: phase-1 tasks
    unsigned long long *ptime; // per plan: warp-nanoseconds spent on its roots (both phases)
    uint32_t cap;
};

// A heavy root with level-2 bound b runs ceil(b / split_S) × split_P3 tasks.
// One warp per plan scans the heavy list between the two phases.
__global__ void heavy_prefix_kernel(DevGraph g, const DevPlan *__restrict__ plans, uint32_t nplans, HeavyBuf H) {
    const uint32_t p = blockIdx.x, lane = threadIdx.x & 31u;
    if (p >= nplans || threadIdx.x >= 32) return;
    const DevPlan &P = plans[p];
    const uint32_t n = min(H.cnt[p], H.cap);
    unsigned long long run = 0;
    for (uint32_t b = 0; b < n; b += 32) {
        const uint32_t h = b + lane;
        unsigned long long tasks = 0;
        if (h < n && P.split_S) {
            const uint2 e = root_edge(g, P, H.ids[(size_t)p * H.cap + h]);
            const uint32_t b2 = level2_bound(g, P, e);
            tasks = (unsigned long long)((b2 + P.split_S - 1) / P.split_S) * P.split_P3;
        }
        unsigned long long incl = tasks;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const unsigned long long v = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl += v;
        }
        if (h < n) H.pre[(size_t)p * H.cap + h] = run + incl - tasks;
        run += __shfl_sync(FULL_MASK, incl, 31);
    }
    if (lane == 0) H.tot[p] = run;
}

// Phase 0 counts every root, except that a root whose level-2 bound exceeds
// split_H is appended to its plan's heavy list (while there is room) instead.
// Phase 1 runs each heavy root as ceil(bound / S) × P3 tasks: task (c, q)
// covers level-2 candidates [c·S, (c+1)·S) and, below them, part q of P3 of
// each level-3 list, so one root's work spreads over the whole GPU.
// 4-warp blocks, 7 per SM: 72 registers per thread and ~8 KB of shared
// memory per warp fit 28 resident warps (the DFS is latency-bound, so
// resident warps set the speed)
constexpr uint32_t COUNT_MAX_WARPS = 4;
template <bool STATS>
__global__ void __launch_bounds__(COUNT_MAX_WARPS * 32, 7) count_kernel(DevGraph g, const DevPlan *__restrict__ plans, uint32_t nplans,
                                                    unsigned long long *queues, unsigned long long *counts,
                                                    uint32_t *scratch, uint32_t cap, uint32_t bufs_per_warp,
                                                    uint32_t tw, uint32_t tmode, unsigned long long deadline_ns,
                                                    uint32_t *flags, DevStats *stats, uint32_t phase, HeavyBuf H,
                                                    uint32_t ntd, uint32_t cs, uint32_t nvs, uint32_t ntr) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t lane = lane_id();
    const uint32_t wib = threadIdx.x >> 5;
    const size_t gwarp = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    Ctx<STATS> c;
    c.g = g;
    c.buf = scratch + gwarp * (size_t)bufs_per_warp * cap;
    c.cap = cap;
    c.flags = flags;
    c.set_ops = c.alg_bytes = c.partial = 0;
    WarpState &W = setup_warp(smem_raw, wib, tw, tmode, ntd, cs, nvs, c, ntr);
    unsigned long long roots = 0;
    // The time budget covers both launch phases: phase 0's first block
    // records its start next to the flags, and phase 1 measures from there.
    unsigned long long tstart = 0;
    unsigned long long *t0_slot = reinterpret_cast<unsigned long long *>(flags + 2);
    if (lane == 0) {
        tstart = globaltimer_ns();
        if (phase == 0 && blockIdx.x == 0 && wib == 0) *t0_slot = tstart;
        else if (phase == 1 && *(volatile unsigned long long *)t0_slot) tstart = *(volatile unsigned long long *)t0_slot;
    }
    c.tstart = __shfl_sync(FULL_MASK, tstart, 0);
    c.deadline = deadline_ns;
    // Plans are taken in order; each has its own task queue and chunk size, so
    // warps spread over the current plan and move on when it is exhausted.
    uint32_t cur = 0;
    unsigned long long acc = 0, ntasks = 0;
    auto load_plan = [&](uint32_t pi) {
        const DevPlan &Q = plans[pi];
        ntasks = phase == 0 ? Q.ntasks : H.tot[pi];
        c.g.hub_min = Q.no_hubs ? 0xFFFFFFFFu : g.hub_min;
    };
    if (nplans) load_plan(0);
    while (cur < nplans) {
        const DevPlan &P = plans[cur];
        if (out_of_time(c)) break;
        if (*(volatile uint32_t *)flags & FLAG_OVERFLOW) break;
        const uint32_t chunk = phase == 0 ? P.chunk : 1u;
        unsigned long long t0 = 0;
        if (lane == 0) t0 = atomicAdd(queues + cur, (unsigned long long)chunk);
        t0 = __shfl_sync(FULL_MASK, t0, 0);
        if (t0 >= ntasks) {
            if (lane == 0 && acc) atomicAdd(counts + cur, acc);
            acc = 0;
            if (++cur < nplans) load_plan(cur);
            continue;
        }
        const unsigned long long t1 = min(t0 + chunk, ntasks);
        if (phase == 1) {
            // the heavy root holding task t0: the last with pre[h] <= t0
            const uint32_t hn = min(H.cnt[cur], H.cap);
            const unsigned long long *pre = H.pre + (size_t)cur * H.cap;
            uint32_t lo = 0, len = hn;
            while (len > 0) {
                const uint32_t half = len >> 1;
                if (pre[lo + half] <= t0) { lo += half + 1; len -= half + 1; }
                else len = half;
            }
            const uint32_t h = lo - 1;
            const unsigned long long local = t0 - pre[h];
            const uint2 e = root_edge(g, P, H.ids[(size_t)cur * H.cap + h]);
            const uint32_t c2 = (uint32_t)(local / P.split_P3), q3 = (uint32_t)(local % P.split_P3);
            if (lane == 0) W.t_root = globaltimer_ns();
            acc += run_root<STATS>(P, W, c, e.x, e.y, c2 * P.split_S, (c2 + 1) * P.split_S, q3, P.split_P3);
            if (lane == 0) atomicAdd(H.ptime + cur, globaltimer_ns() - W.t_root);
            continue;
        }
        if (P.ne == 2) {
            // lane l takes task t0 + l; roots the degree cap drops are compacted out
            const uint32_t n = (uint32_t)(t1 - t0);
            uint32_t u = 0, v = 0;
            bool keep = false;
            if (lane < n) {
                const uint2 e = root_edge(g, P, t0 + lane);
                u = e.x;
                v = e.y;
                keep = root_kept(g, P, e);
            }
            const uint32_t kb = __ballot_sync(FULL_MASK, keep);
            const uint32_t nk = __popc(kb);
            // lane r takes the r-th kept root
            uint32_t src = 0;
            {
                uint32_t msk = kb;
                for (uint32_t r = 0; r < lane && msk; ++r) msk &= msk - 1;
                src = msk ? (uint32_t)(__ffs(msk) - 1) : 0u;
            }
            const uint32_t ku = __shfl_sync(FULL_MASK, u, src), kv = __shfl_sync(FULL_MASK, v, src);
            if (nk) {
                if (lane == 0) W.t_root = globaltimer_ns();
                acc += leaf_roots(P, W, c, nk, ku, kv);
                if (lane == 0) atomicAdd(H.ptime + cur, globaltimer_ns() - W.t_root);
            }
            roots += nk;
            continue;
        }
        for (unsigned long long t = t0; t < t1; ++t) {
            const uint2 e = root_edge(g, P, t);
            if (!root_kept(g, P, e)) continue;
            ++roots;
            if (P.split_S && level2_bound(g, P, e) > P.split_H) {
                uint32_t slot = 0;
                if (lane == 0) slot = atomicAdd(H.cnt + cur, 1u);
                slot = __shfl_sync(FULL_MASK, slot, 0);
                if (slot < H.cap) {
                    if (lane == 0) H.ids[(size_t)cur * H.cap + slot] = (uint32_t)t;
                    continue;
                }
            }
            if (lane == 0) W.t_root = globaltimer_ns();
            acc += run_root<STATS>(P, W, c, e.x, e.y);
            if (lane == 0) atomicAdd(H.ptime + cur, globaltimer_ns() - W.t_root);
        }
    }
    if (cur < nplans && lane == 0 && acc) atomicAdd(counts + cur, acc);
    if (STATS && lane == 0) {
        atomicAdd(&stats->set_ops, c.set_ops);
        atomicAdd(&stats->alg_bytes, c.alg_bytes);
        atomicAdd(&stats->partial, c.partial);
        atomicAdd(&stats->roots, roots);
    }
}


// ------------------------------------------------------------ enumeration --
// Writes every match of a plan (all k levels enumerated, no counting tail)
// as k vertex ids in pattern-vertex order: the tuples of nodeJoin /
// globalJoin before buildTrie (matching/join.cpp:309-421,1202-1420) and, for
// the whole pattern, the embedding set -r writes.  A warp owns one root edge;
// the last level's candidates are emitted 32 at a time with one atomicAdd of
// the output cursor per chunk.
__global__ void __launch_bounds__(256) enum_kernel(DevGraph g, const DevPlan *__restrict__ plan,
                                                   unsigned long long *queue, uint32_t *scratch, uint32_t cap,
                                                   uint32_t bufs_per_warp, uint32_t *flags, uint32_t *out,
                                                   unsigned long long out_cap, unsigned long long *out_n) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t lane = lane_id();
    const uint32_t wib = threadIdx.x >> 5;
    const DevPlan &P = *plan;
    const size_t gwarp = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    Ctx<false> c;
    c.g = g;
    c.buf = scratch + gwarp * (size_t)bufs_per_warp * cap;
    c.cap = cap;
    c.flags = flags;
    c.set_ops = c.alg_bytes = c.partial = 0;
    c.tstart = 0;
    c.deadline = 0;
    WarpState &W = setup_warp(smem_raw, wib, 0u, 0u, 1u, 1u, SGE_MAX_VSLOTS, c);
    const uint32_t k = P.k, last = k - 1;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(queue, 1ull);
        t = __shfl_sync(FULL_MASK, t, 0);
        if (t >= P.ntasks) break;
        if (*(volatile uint32_t *)flags & FLAG_OVERFLOW) break;
        const uint2 e = root_edge(g, P, t);
        set_match(g, W, 0, e.x);
        set_match(g, W, 1, e.y);
        uint32_t lv = 2;
        bool ok = build_level_wcoj(P, W, c, lv);
        if (ok) { __syncwarp(); if (lane == 0) W.pos[lv] = 0; __syncwarp(); }
        while (ok) {
            if (lv == last) {
                const uint32_t n = W.cnt[lv];
                const uint32_t *lst = W.list[lv];
                for (uint32_t b0 = 0; b0 < n; b0 += 32) {
                    const uint32_t idx = b0 + lane;
                    bool valid = idx < n;
                    const uint32_t x = valid ? lst[idx] : 0u;
                    if (valid) valid = !excluded(P, W, lv, x);
                    const uint32_t bal = __ballot_sync(FULL_MASK, valid);
                    unsigned long long base = 0;
                    if (lane == 0 && bal) base = atomicAdd(out_n, (unsigned long long)__popc(bal));
                    base = __shfl_sync(FULL_MASK, base, 0);
                    if (valid) {
                        const unsigned long long row = base + __popc(bal & ((1u << lane) - 1u));
                        if (row < out_cap) {
                            uint32_t *o = out + row * k;
                            for (uint32_t l = 0; l < last; ++l) o[P.order_[l]] = W.m[l];
                            o[P.order_[last]] = x;
                        }
                    }
                }
                if (lv == 2) break;
                --lv;
                continue;
            }
            const uint32_t pos = W.pos[lv];
            if (pos >= W.cnt[lv]) {
                if (lv == 2) break;
                --lv;
                continue;
            }
            const uint32_t x = W.list[lv][pos];
            __syncwarp();
            if (lane == 0) W.pos[lv] = pos + 1;
            __syncwarp();
            if (excluded(P, W, lv, x)) continue;
            set_match(g, W, lv, x);
            ++lv;
            if (!build_level_wcoj(P, W, c, lv)) { ok = false; break; }
            __syncwarp();
            if (lane == 0) W.pos[lv] = 0;
            __syncwarp();
        }
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct sge_graph {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t n = 0;
    uint64_t nnz = 0, m = 0;
    uint32_t max_deg = 0;
    uint32_t *d_off = nullptr, *d_adj = nullptr;
    uint2 *d_edges = nullptr;
    sge_graph_stats stats{};   // planner inputs (degree moments, clustering)
    uint32_t *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    unsigned char *d_batch = nullptr;
    size_t batch_bytes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int num_sms = 0;
    bool launched = false;     // a counting launch has run on this graph
    // hub index (neighbour bitmaps of the highest-degree vertices)
    uint32_t *d_hub_bits = nullptr;
    int32_t *d_hub_slot = nullptr;
    uint32_t hub_words = 0, hub_min = 0xFFFFFFFFu, hub_count = 0;
    uint64_t hub_bytes = 0;
    uint32_t *d_labels = nullptr;  // vertex labels (sge_graph_set_labels)
};

namespace {
DevGraph dev_graph(const sge_graph *g, bool hubs) {
    DevGraph d{g->d_off, g->d_adj, g->d_edges, g->n, g->m, g->d_hub_bits, g->d_hub_slot, g->hub_words, g->hub_min};
    if (!hubs || !g->d_hub_bits) d.hub_min = 0xFFFFFFFFu;
    return d;
}
}  // namespace

// Bag relations of a decomposition on one graph (sge_bags_create): for each
// bag with exactly one attribute of its own, the bag's tuples (the
// reference's nodeJoin, matching/join.cpp:309-421) as a trie
// (buildTrie, join.cpp:1713-1717) whose key columns are the bag's other
// attributes in ascending vertex order and whose last column is its own one.
struct BagRel {
    uint32_t priv = 0;                    // the bag's own pattern vertex
    uint32_t nkeys = 0;
    uint32_t keys[3] = {};                // its other attributes, ascending
    uint64_t rows = 0;
    sge_trie trie{};
    unsigned long long *first = nullptr;  // dense first key level (n + 1 offsets)
};
struct sge_bags {
    const sge_graph *g = nullptr;
    int device = 0;
    uint32_t k = 0;
    std::vector<BagRel> rels;
    DevTrie *d_tries = nullptr;
    uint64_t bytes = 0;
    uint32_t skipped = 0;  // bags whose relation exceeded max_rows
};

struct sge_plan {
    sge_plan_blob blob;
    DevPlan dp;
    sge_plan_tuning tune{};
    const sge_bags *bags = nullptr;  // bag relations its tail levels read (sge_plan_use_bags)
    bool has_labels = false;         // pattern labels attached (sge_plan_set_labels)
    uint32_t labels[SGE_MAX_K] = {};
};

namespace sge {
bool graph_stats(const sge_graph *g, sge_graph_stats *out) {
    if (!g) return false;
    *out = g->stats;
    return true;
}
}  // namespace sge

namespace {

#define CUDA_TRY(expr)                                                                               \
    do {                                                                                             \
        cudaError_t _e = (expr);                                                                     \
        if (_e != cudaSuccess) {                                                                     \
            return fail(_e == cudaErrorMemoryAllocation ? SGE_OOM : SGE_CUDA_ERROR, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(_e), __FILE__, __LINE__);                          \
        }                                                                                            \
    } while (0)

void to_devplan(const sge_plan_blob &b, DevPlan &d) {
    memset(&d, 0, sizeof d);
    for (uint32_t i = 0; i < SGE_MAX_K; ++i) {
        d.parents[i] = (uint16_t)b.parents[i];
        d.lower[i] = (uint16_t)b.lower[i];
        d.upper[i] = (uint16_t)b.upper[i];
        d.check[i] = (uint16_t)b.check[i];
        d.rest[i] = (uint16_t)b.rest[i];
        d.base[i] = (int8_t)b.base[i];
        for (uint32_t j = 0; j < SGE_MAX_K; ++j) d.slot[i][j] = -1;
    }
    d.k = b.k;
    d.ne = b.num_enum;
    d.T = b.tail_len;
    d.tail_mode = b.tail_mode;
    d.join_style = b.join_style;
    d.root_kind = b.root_kind;
    d.nparts = b.num_partitions;
    for (uint32_t p = 0; p < SGE_MAX_PARTITIONS; ++p) {
        d.part_coef[p] = (int8_t)b.part_coef[p];
        d.part_nblocks[p] = (uint8_t)b.part_nblocks[p];
        for (uint32_t x = 0; x < SGE_MAX_TAIL; ++x) d.part_block[p][x] = (uint8_t)b.part_block[p][x];
    }
    uint32_t nb = 0;
    if (b.join_style == SGE_JOIN_EXPLORATION) {
        for (uint32_t i = 2; i < b.k; ++i) {
            uint32_t par = b.parents[i];
            bool first = true;
            for (uint32_t msk = par; msk; msk &= msk - 1) {
                uint32_t j = (uint32_t)__builtin_ctz(msk);
                d.after[j] = (uint16_t)(d.after[j] | (1u << i));
                if (first) { d.slot[j][i] = -1; first = false; }
                else d.slot[j][i] = (int8_t)nb++;
            }
        }
    } else {
        nb = b.k;  // stored levels and hoisted tail lists use buffer index = level
    }
    d.nbufs = std::max<uint32_t>(nb, 1);
    // pin N(m[0]) / N(m[1]) when a level past 2 probes it (probed once per
    // candidate rather than once per root)
    d.pin_mask = 0;
    if (b.num_enum >= 3)
        for (uint32_t i = 3; i < b.k; ++i) {
            d.pin_mask |= b.parents[i] & 3u;
            if (b.join_style == SGE_JOIN_WCOJ && b.base[i] == 2) d.pin_mask |= 4u;
        }
    d.keep_full = 0;
    for (uint32_t i = 0; i < b.k; ++i)
        if (b.base[i] >= 0) d.keep_full |= 1u << b.base[i];
    // hoisted tail lists, the pair step and its inline tail (shared with the cost model)
    const ExecShape xs = exec_shape(b);
    d.hoist_mask = xs.hoist_mask;
    for (uint32_t i = 0; i < SGE_MAX_K; ++i) d.hoist_at[i] = xs.hoist_at[i];
    d.tail_par = 0;
    for (uint32_t i = b.num_enum; i < b.k; ++i) d.tail_par |= b.parents[i];
    // (labeled plans check every candidate's label where it is taken, so
    // they keep the level-by-level DFS: no pair step)
    d.pair = xs.pair && !b.labeled ? 1u : 0u;
    d.pair_direct = xs.pair_direct && !b.labeled ? 1u : 0u;
    // exploration: the running list of a tail level whose parents below the
    // leaf are exactly levels 0 and 1 is final once the root is matched;
    // it is pinned in the third table
    d.epin = 0;
    if (b.join_style == SGE_JOIN_EXPLORATION && b.num_enum >= 3) {
        const uint32_t lt = d.pair ? b.num_enum - 2 : b.num_enum - 1;
        for (uint32_t i = b.num_enum; i < b.k && !d.epin; ++i)
            if ((b.parents[i] & ((1u << lt) - 1u)) == 3u) d.epin = i;
    }
    d.mult = b.count_multiplier;
    d.choose_wrap = b.choose_wrap ? 1u : 0u;
    d.chunk = 1;
    d.split_par = b.num_enum >= 3 ? (b.parents[2] & 3u) : 0u;
    for (uint32_t i = 0; i < SGE_MAX_K; ++i) d.order_[i] = (uint8_t)b.order[i];
    d.split_S = 0;  // set per graph in sge_count
}

// Hub index: one neighbour bitmap per vertex of degree >= hub_min, with
// hub_min the smallest threshold (at least 16: shorter lists are searched in
// a few steps) whose bitmaps fit in min(4 GB, 1/16 of free HBM, and
// SGE_HUB_INDEX_MB when that environment variable is set).  HBM is
// plentiful next to the CSR, and a membership test in a hub's list, the
// costliest binary search of the join, becomes one load.
__global__ void hub_bits_kernel(const uint32_t *off, const uint32_t *adj, const uint32_t *hubs, uint32_t nh,
                                uint32_t words, uint32_t *bits) {
    for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint32_t v = hubs[h];
        uint32_t *b = bits + (size_t)h * words;
        for (uint32_t e = off[v] + threadIdx.x; e < off[v + 1]; e += blockDim.x) {
            const uint32_t y = adj[e];
            atomicOr(&b[y >> 5], 1u << (y & 31u));
        }
    }
}

sge_status build_hub_index(sge_graph *g, const uint32_t *off) {
    const uint32_t n = g->n;
    if (n == 0 || g->max_deg < 16) return SGE_OK;
    const uint64_t words = ((uint64_t)n + 31) / 32;
    std::vector<uint32_t> hist((size_t)g->max_deg + 1, 0);
    for (uint32_t v = 0; v < n; ++v) hist[off[v + 1] - off[v]]++;
    size_t free_b = 0, tot_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &tot_b));
    uint64_t budget = std::min<uint64_t>(4ull << 30, free_b / 16);
    if (const char *env = getenv("SGE_HUB_INDEX_MB")) budget = std::min<uint64_t>(budget, strtoull(env, nullptr, 10) << 20);
    const uint64_t max_hubs = std::min<uint64_t>(budget / (4 * words), 1u << 20);
    uint64_t above = 0;
    uint32_t thr = g->max_deg + 1;
    for (uint32_t d = g->max_deg; d >= 16; --d) {
        if (above + hist[d] > max_hubs) break;
        above += hist[d];
        thr = d;
    }
    if (above == 0) return SGE_OK;
    std::vector<int32_t> slot(n, -1);
    std::vector<uint32_t> hubs;
    hubs.reserve(above);
    for (uint32_t v = 0; v < n; ++v)
        if (off[v + 1] - off[v] >= thr) { slot[v] = (int32_t)hubs.size(); hubs.push_back(v); }
    uint32_t *d_hubs = nullptr;
    if (cudaMalloc(&g->d_hub_slot, 4ull * n) != cudaSuccess ||
        cudaMalloc(&g->d_hub_bits, 4ull * words * hubs.size()) != cudaSuccess ||
        cudaMalloc(&d_hubs, 4ull * hubs.size()) != cudaSuccess) {
        cudaFree(g->d_hub_slot);
        cudaFree(g->d_hub_bits);
        g->d_hub_slot = nullptr;
        g->d_hub_bits = nullptr;
        cudaGetLastError();
        return SGE_OK;  // no index: every probe is a binary search
    }
    CUDA_TRY(cudaMemcpyAsync(g->d_hub_slot, slot.data(), 4ull * n, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemcpyAsync(d_hubs, hubs.data(), 4ull * hubs.size(), cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemsetAsync(g->d_hub_bits, 0, 4ull * words * hubs.size(), g->stream));
    hub_bits_kernel<<<(unsigned)std::min<size_t>(hubs.size(), 65535), 256, 0, g->stream>>>(
        g->d_off, g->d_adj, d_hubs, (uint32_t)hubs.size(), (uint32_t)words, g->d_hub_bits);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    cudaFree(d_hubs);
    g->hub_words = (uint32_t)words;
    g->hub_min = thr;
    g->hub_count = (uint32_t)hubs.size();
    g->hub_bytes = 4ull * words * hubs.size() + 4ull * n;
    return SGE_OK;
}

sge_status ensure_scratch(sge_graph *g, size_t bytes) {
    if (g->scratch_bytes >= bytes) return SGE_OK;
    if (g->d_scratch) { cudaFree(g->d_scratch); g->d_scratch = nullptr; g->scratch_bytes = 0; }
    CUDA_TRY(cudaMalloc(&g->d_scratch, bytes));
    g->scratch_bytes = bytes;
    return SGE_OK;
}

sge_status ensure_batch(sge_graph *g, size_t bytes) {
    if (g->batch_bytes >= bytes) return SGE_OK;
    if (g->d_batch) { cudaFree(g->d_batch); g->d_batch = nullptr; g->batch_bytes = 0; }
    CUDA_TRY(cudaMalloc(&g->d_batch, bytes));
    g->batch_bytes = bytes;
    return SGE_OK;
}

// Host validation, before any device is touched: offsets monotone, lists
// sorted strictly increasing, in range, no self-loops; symmetric.  Symmetry
// costs one search per pair: every entry w > v of N(v) must find v among
// the entries of N(w) below w, which maps the upper entries one-to-one onto
// lower ones, so with equally many upper and lower entries every lower entry
// is some upper entry's mirror too.
// Offsets: off[0] = 0, off[n] = nnz, monotone (every list inside the array).
sge_status validate_offsets(const uint32_t *off, uint32_t n, uint64_t nnz) {
    if (off[0] != 0 || off[n] != nnz) return fail(SGE_BAD_INPUT, "offsets[0] must be 0 and offsets[n] = %llu", (unsigned long long)nnz);
    for (uint32_t v = 0; v < n; ++v)
        if (off[v + 1] < off[v]) return fail(SGE_BAD_INPUT, "offsets not monotone at vertex %u", v);
    return SGE_OK;
}

// The lists on the host: strictly increasing, in range, no self-loop, and
// symmetric (one search per entry above the diagonal, and as many entries
// above the diagonal as below).
sge_status validate_csr(const uint32_t *off, const uint32_t *nbrs, uint32_t n, uint64_t nnz) {
    sge_status ost = validate_offsets(off, n, nnz);
    if (ost != SGE_OK) return ost;
    unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::atomic<int> bad{0};
    std::atomic<uint32_t> bad_v{0};
    std::atomic<uint64_t> upper{0}, lower{0};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            uint64_t up = 0, lo = 0;
            for (uint64_t v = t; v < n && !bad.load(std::memory_order_relaxed); v += nt) {
                const uint32_t a = off[v], b = off[v + 1];
                for (uint32_t e = a; e < b; ++e) {
                    const uint32_t w = nbrs[e];
                    if (w >= n || w == v || (e > a && nbrs[e - 1] >= w)) { bad = 2; bad_v = (uint32_t)v; return; }
                    if (w < v) { ++lo; continue; }
                    ++up;
                    // v must be one of N(w)'s entries below w
                    if (!std::binary_search(nbrs + off[w], nbrs + off[w + 1], (uint32_t)v)) {
                        bad = 3;
                        bad_v = (uint32_t)v;
                        return;
                    }
                }
            }
            upper += up;
            lower += lo;
        });
    for (auto &x : th) x.join();
    if (!bad && upper.load() != lower.load()) { bad = 3; bad_v = 0; }
    if (bad == 1) return fail(SGE_BAD_INPUT, "offsets not monotone at vertex %u", (uint32_t)bad_v);
    if (bad == 2) return fail(SGE_BAD_INPUT, "neighbour list of vertex %u is not strictly increasing, out of range, or has a self-loop", (uint32_t)bad_v);
    if (bad == 3) return fail(SGE_BAD_INPUT, "CSR is not symmetric at vertex %u", (uint32_t)bad_v);
    return SGE_OK;
}

}  // namespace

namespace sge {
// Global clustering coefficient (closed wedges / wedges) from 2^16 wedges
// sampled with probability ∝ C(deg, 2) under a fixed seed.
double sample_clustering(const uint32_t *off, const uint32_t *nb, uint32_t n) {
    std::vector<double> cum(n + 1, 0.0);
    for (uint32_t v = 0; v < n; ++v) {
        double d = (double)(off[v + 1] - off[v]);
        cum[v + 1] = cum[v] + d * (d - 1) / 2;
    }
    if (cum[n] <= 0) return 0.0;
    Rng rng(0xC1A5u);
    const int S = 1 << 16;
    int closed = 0;
    for (int s = 0; s < S; ++s) {
        double r = (double)(rng.next() >> 11) * (1.0 / 9007199254740992.0) * cum[n];
        uint32_t v = (uint32_t)(std::upper_bound(cum.begin(), cum.end(), r) - cum.begin() - 1);
        if (v >= n) v = n - 1;
        uint32_t d = off[v + 1] - off[v];
        if (d < 2) { --s; continue; }
        uint32_t a = (uint32_t)rng.below(d), b = (uint32_t)rng.below(d - 1);
        if (b >= a) ++b;
        uint32_t x = nb[off[v] + a], y = nb[off[v] + b];
        if (std::binary_search(nb + off[x], nb + off[x + 1], y)) ++closed;
    }
    return (double)closed / S;
}
}  // namespace sge

namespace {
// Everything one counting launch needs, computed on the host.
struct LaunchCfg {
    std::vector<DevPlan> dps;
    uint32_t nplans = 0, wpb = 8, threads = 256, tmode = 0, tw = 0, cap = 0, nbufs = 1, heavy_cap = 1;
    uint32_t ntd = 1, cs = 1, nvs = 1;  // per-warp tail descriptors, leaf counters, version slots (largest plan)
    uint32_t ntr = 0;                   // per-warp trie ranges (bag relations of the plans)
    size_t smem = 0, blocks = 1, scratch_bytes = 0;
    bool want_stats = false, any_split = false, use_hubs = true;
    unsigned long long deadline = 0;
    size_t off_plans = 0, off_counts = 0, off_queue = 0, off_flags = 0, off_stats = 0, off_hcnt = 0, off_htot = 0,
           off_hids = 0, off_hpre = 0, off_ptime = 0, bytes_zeroed = 0, bytes = 0;
};

sge_status prepare_launch(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts &o,
                          size_t scratch_held, LaunchCfg &L) {
    L.nplans = nplans;
    L.dps.resize(nplans);
    unsigned long long total = 0;
    for (uint32_t i = 0; i < nplans; ++i) {
        if (!plans[i]) return fail(SGE_BAD_INPUT, "plan %u is null", i);
        DevPlan &d = L.dps[i];
        d = plans[i]->dp;
        d.task_begin = total;
        const unsigned long long stride = o.root_stride > 1 ? o.root_stride : 1ull;
        const unsigned long long offs = o.root_offset;
        if (stride > 1 && offs >= stride) return fail(SGE_BAD_INPUT, "root_offset %llu >= root_stride %llu", offs, stride);
        d.root_stride = stride;
        d.root_offset = stride > 1 ? offs : 0;
        const unsigned long long nedges = g->m > d.root_offset ? (g->m - d.root_offset + stride - 1) / stride : 0;
        d.ntasks = (d.root_kind == SGE_ROOT_ANY) ? 2ull * nedges : nedges;
        total += d.ntasks;
        L.nbufs = std::max(L.nbufs, d.nbufs);
        L.ntd = std::max(L.ntd, plan_ntd(d));
        L.cs = std::max(L.cs, plan_cs(d));
        L.nvs = std::max(L.nvs, plan_nvs(d));
        L.ntr = std::max<uint32_t>(L.ntr, d.ntrie);
        if (plans[i]->bags && plans[i]->bags->g != g)
            return fail(SGE_BAD_INPUT, "plan %u uses bag relations built on another graph", i);
        if (plans[i]->blob.labeled) {
            if (!plans[i]->has_labels) return fail(SGE_BAD_INPUT, "plan %u is labeled but has no labels (sge_plan_set_labels)", i);
            if (!g->d_labels) return fail(SGE_BAD_INPUT, "plan %u is labeled but the graph has no labels (sge_graph_set_labels)", i);
            d.vlab = g->d_labels;
            for (uint32_t l = 0; l < d.k; ++l) d.lab[l] = plans[i]->labels[plans[i]->blob.order[l]];
        }
        if (d.k > SGE_MAX_K) return fail(SGE_UNSUPPORTED, "plan %u has k=%u", i, d.k);
    }
    // pinned-list tables: a bitmap over all vertices when it fits in 4 KB.
    // Larger graphs pin nothing by default: 512-slot hashes (lists of at most
    // 256) cost 6 KB of shared memory per warp, and with the hub index the
    // long lists need no table; the freed shared memory keeps more warps
    // resident (pin_tables = 2 asks for the hashes anyway).
    if (o.pin_tables == 1) { L.tmode = 0; L.tw = 0; }
    else if (g->n <= 32768u) { L.tmode = 1; L.tw = std::max<uint32_t>(32u, ((g->n + 31u) / 32u + 31u) & ~31u); }
    else if (o.pin_tables == 2 || !g->d_hub_bits || o.no_hub_bitmaps) { L.tmode = 2; L.tw = 512; }
    else { L.tmode = 0; L.tw = 0; }
    L.want_stats = o.collect_counters != 0;
    for (auto &d : L.dps) d.root_maxdeg = o.root_max_degree;
    L.use_hubs = o.no_hub_bitmaps == 0;
    // warps per block: 4 or 2, whichever keeps more warps resident per SM
    // (shared memory per warp is several KB, so smaller blocks pack better)
    int bps = 0;
    {
        int best_warps = -1;
        const uint32_t choices[2] = {COUNT_MAX_WARPS, 2};
        for (uint32_t wpb : choices) {
            if (o.warps_per_block && wpb != std::min<uint32_t>(o.warps_per_block, COUNT_MAX_WARPS)) continue;
            const size_t smem = warp_smem_bytes(L.tw, L.ntd, L.cs, L.nvs, L.ntr) * wpb;
            int b = 0;
            // static (plan copies) + dynamic shared memory exceed the 48 KB default: opt in
            CUDA_TRY(cudaFuncSetAttribute(count_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            CUDA_TRY(cudaFuncSetAttribute(count_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            if (L.want_stats) CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, count_kernel<true>, wpb * 32, smem));
            else CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, count_kernel<false>, wpb * 32, smem));
            if (b * (int)wpb > best_warps) { best_warps = b * (int)wpb; bps = b; L.wpb = wpb; L.smem = smem; }
        }
        if (o.warps_per_block && best_warps < 0) {
            L.wpb = std::min<uint32_t>(std::max<uint32_t>(o.warps_per_block, 1), COUNT_MAX_WARPS);
            L.smem = warp_smem_bytes(L.tw, L.ntd, L.cs, L.nvs, L.ntr) * L.wpb;
        }
        L.threads = L.wpb * 32;
        CUDA_TRY(cudaFuncSetAttribute(count_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
        CUDA_TRY(cudaFuncSetAttribute(count_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
    }
    if (o.blocks_per_sm) bps = std::min<int>(bps, (int)o.blocks_per_sm);
    bps = std::max(bps, 1);
    L.cap = o.max_level_capacity ? o.max_level_capacity : std::max<uint32_t>(g->max_deg, 1);
    L.cap = (L.cap + 31) & ~31u;
    // fit the scratch into a quarter of free memory by trimming resident blocks
    size_t free_b = 0, tot_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &tot_b));
    const size_t per_block = (size_t)L.wpb * L.nbufs * L.cap * sizeof(uint32_t);
    size_t blocks = (size_t)g->num_sms * bps;
    const size_t budget = free_b / 4 + scratch_held;
    while (blocks > (size_t)g->num_sms && blocks * per_block > budget) blocks -= g->num_sms;
    if (blocks * per_block > budget) blocks = std::max<size_t>(1, budget / std::max<size_t>(per_block, 1));
    L.blocks = blocks;
    L.scratch_bytes = blocks * per_block;
    // heavy-root splitting (plans with >= 3 enumerated levels): a root whose
    // level-2 list may exceed split_H candidates runs as tasks of S
    // candidates.  A root's work grows with its level-2 list, and a warp's
    // share of the launch is about ntasks × (mean endpoint degree M2/M1) /
    // warps candidates; roots are split only when one could exceed a quarter
    // of that share (splitting repeats the root's setup in every task)
    unsigned long long max_tasks = 1;
    const unsigned long long warps = blocks * L.wpb;
    // mean level-2 bound of a root: the size-biased degree, but never more
    // than the degree cap of a capped sample
    double mean_deg = g->stats.moments[1] > 0 ? g->stats.moments[2] / g->stats.moments[1] : 1.0;
    if (o.root_max_degree) mean_deg = std::min(mean_deg, (double)o.root_max_degree);
    for (uint32_t pi = 0; pi < nplans; ++pi) {
        DevPlan &d = L.dps[pi];
        const sge_plan_tuning &tu = plans[pi]->tune;
        d.no_hubs = tu.no_hub_bitmaps ? 1u : 0u;
        // deeper plans do more work per level-2 candidate (and far more under
        // a hub), so their tasks hold fewer candidates: 128 at four
        // enumerated levels, a quarter as many per extra level
        const uint32_t deep = d.ne > 4 ? std::min<uint32_t>(d.ne - 4, 3u) : 0u;
        // where level 3 is enumerated by the DFS (or is the pair step's
        // level), a task takes one level-2 candidate and a part of its
        // level-3 list: 8 parts at five enumerated levels, 16 deeper
        const bool split3 = d.ne >= 5 || (d.ne == 4 && !d.pair);
        const uint32_t split_P3 = split3 ? (tu.level3_parts ? std::min(tu.level3_parts, 1024u)
                                                            : (d.ne >= 6 ? 16u : 8u))
                                         : 1u;
        const uint32_t split_S = split3 ? 1u : std::max<uint32_t>(128u >> (2 * deep), 2u);
        const double share = (double)d.ntasks * mean_deg / (double)std::max<unsigned long long>(warps, 1);
        const uint32_t thr = tu.heavy_threshold ? tu.heavy_threshold : o.heavy_threshold;
        const uint32_t split_H = thr ? std::max(thr, 4u * split_S)
                                     : (uint32_t)std::min(1e9, std::max(32.0, share / 4.0));
        if (d.ne >= 3 && g->max_deg > split_H) {
            d.split_S = split_S;
            d.split_H = split_H;
            d.split_P3 = split_P3;
            L.any_split = true;
        }
        max_tasks = std::max(max_tasks, d.ntasks);
        if (d.ne == 2) d.chunk = 32;  // one leaf over 32 root edges
        else if (o.chunk) d.chunk = o.chunk;
        else d.chunk = (uint32_t)std::max<unsigned long long>(1, std::min<unsigned long long>(8, d.ntasks / (warps * 64 + 1)));
    }
    L.heavy_cap = L.any_split ? (uint32_t)std::min<unsigned long long>(max_tasks, 1ull << 18) : 1u;
    // buffer: plans | counts | per-plan queues | flags | stats | heavy counts | heavy task totals |
    //         heavy lists | heavy task prefixes
    L.off_plans = 0;
    L.off_counts = (sizeof(DevPlan) * nplans + 255) & ~(size_t)255;
    L.off_queue = L.off_counts + ((8 * (size_t)nplans + 255) & ~(size_t)255);
    L.off_flags = L.off_queue + ((8 * (size_t)nplans + 255) & ~(size_t)255);
    L.off_stats = L.off_flags + 256;
    L.off_hcnt = L.off_stats + 256;
    L.off_htot = L.off_hcnt + ((4 * (size_t)nplans + 255) & ~(size_t)255);
    L.off_ptime = L.off_htot + ((8 * (size_t)nplans + 255) & ~(size_t)255);
    L.off_hids = L.off_ptime + ((8 * (size_t)nplans + 255) & ~(size_t)255);
    L.bytes_zeroed = L.off_hids;
    L.off_hpre = L.off_hids + (((size_t)L.heavy_cap * nplans * 4 + 255) & ~(size_t)255);
    L.bytes = L.off_hpre + (((size_t)L.heavy_cap * nplans * 8 + 255) & ~(size_t)255);
    if (o.time_budget_s > 0) L.deadline = std::max<unsigned long long>(1, (unsigned long long)(o.time_budget_s * 1e9));
    return SGE_OK;
}

// Stream-ordered: clear the counters, run phase 0 and (when roots may be
// split) phase 1.  Capturable (no host synchronisation).
sge_status enqueue_launch(sge_graph *g, const LaunchCfg &L, unsigned char *B, uint32_t *scratch, cudaStream_t s,
                          uint32_t &launches) {
    CUDA_TRY(cudaMemsetAsync(B + L.off_counts, 0, L.bytes_zeroed - L.off_counts, s));
    DevGraph dg = dev_graph(g, L.use_hubs);
    const DevPlan *dplans = reinterpret_cast<const DevPlan *>(B + L.off_plans);
    unsigned long long *dcounts = reinterpret_cast<unsigned long long *>(B + L.off_counts);
    unsigned long long *dqueue = reinterpret_cast<unsigned long long *>(B + L.off_queue);
    uint32_t *dflags = reinterpret_cast<uint32_t *>(B + L.off_flags);
    DevStats *dstats = reinterpret_cast<DevStats *>(B + L.off_stats);
    HeavyBuf H{reinterpret_cast<uint32_t *>(B + L.off_hcnt), reinterpret_cast<uint32_t *>(B + L.off_hids),
               reinterpret_cast<unsigned long long *>(B + L.off_hpre),
               reinterpret_cast<unsigned long long *>(B + L.off_htot),
               reinterpret_cast<unsigned long long *>(B + L.off_ptime), L.heavy_cap};
    launches = 0;
    for (uint32_t phase = 0; phase < (L.any_split ? 2u : 1u); ++phase) {
        if (phase == 1) {
            CUDA_TRY(cudaMemsetAsync(dqueue, 0, 8 * (size_t)L.nplans, s));
            heavy_prefix_kernel<<<L.nplans, 32, 0, s>>>(dg, dplans, L.nplans, H);
            CUDA_TRY(cudaGetLastError());
            ++launches;
        }
        if (L.want_stats)
            count_kernel<true><<<(unsigned)L.blocks, L.threads, L.smem, s>>>(
                dg, dplans, L.nplans, dqueue, dcounts, scratch, L.cap, L.nbufs, L.tw, L.tmode, L.deadline, dflags,
                dstats, phase, H, L.ntd, L.cs, L.nvs, L.ntr);
        else
            count_kernel<false><<<(unsigned)L.blocks, L.threads, L.smem, s>>>(
                dg, dplans, L.nplans, dqueue, dcounts, scratch, L.cap, L.nbufs, L.tw, L.tmode, L.deadline, dflags,
                dstats, phase, H, L.ntd, L.cs, L.nvs, L.ntr);
        CUDA_TRY(cudaGetLastError());
        ++launches;
    }
    return SGE_OK;
}

sge_status finish_counts(const LaunchCfg &L, const unsigned long long *hc, uint32_t hflags, const DevStats &hs,
                         float ms, uint32_t launches, std::chrono::steady_clock::time_point t_start,
                         const sge_plan *const *plans, uint64_t *counts, uint64_t *instances, sge_stats *stats,
                         const sge_count_opts &o) {
    for (uint32_t i = 0; i < L.nplans; ++i) {
        const uint64_t inst = hc[i];
        counts[i] = inst * plans[i]->blob.count_multiplier;
        if (instances) instances[i] = inst;
    }
    if (stats) {
        stats->kernel_ms = ms;
        stats->root_tasks = hs.roots;
        stats->set_ops = hs.set_ops;
        stats->alg_bytes = hs.alg_bytes;
        stats->partial_matches = hs.partial;
        stats->gpu_launches = launches;
        stats->status_flags = hflags;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    if (hflags & FLAG_OVERFLOW) return fail(SGE_STACK_OVERFLOW, "a candidate list exceeded the per-level capacity %u", L.cap);
    if (hflags & FLAG_TIMEOUT) return fail(SGE_TIMEOUT, "time budget of %.3f s exceeded; counts are partial", o.time_budget_s);
    return SGE_OK;
}

}  // namespace

// Directed-entry count above which sge_graph_create checks the lists on the
// device (the host check of 128M entries takes seconds; the device's, ms).
constexpr uint64_t SGE_HOST_VALIDATE_MAX = 1ull << 22;

namespace {
__global__ void csr_check_kernel(const uint32_t *off, const uint32_t *adj, uint32_t n, uint32_t *res,
                                 unsigned long long *cnt);
}  // namespace

namespace sge_csr_check {
// validate_csr's list checks for a CSR already on the device (same messages).
sge_status validate_csr_device(const uint32_t *d_off, const uint32_t *d_adj, uint32_t n, int device) {
    uint32_t *res = nullptr;
    unsigned long long *cnt = nullptr;
    CUDA_TRY(cudaMalloc(&res, 16));
    cudaError_t e = cudaMalloc(&cnt, 16);
    if (e != cudaSuccess) { cudaFree(res); return fail(SGE_OOM, "CSR check: %s", cudaGetErrorString(e)); }
    const uint32_t init[4] = {0u, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u};
    uint32_t h[4] = {0, 0, 0, 0};
    unsigned long long hc[2] = {0, 0};
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    e = cudaMemcpy(res, init, 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(cnt, 0, 16);
    if (e == cudaSuccess) {
        csr_check_kernel<<<(unsigned)std::max(sms, 1) * 8u, 256>>>(d_off, d_adj, n, res, cnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, res, 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hc, cnt, 16, cudaMemcpyDeviceToHost);
    cudaFree(res);
    cudaFree(cnt);
    if (e != cudaSuccess) return fail(SGE_CUDA_ERROR, "CSR check: %s", cudaGetErrorString(e));
    if (h[0] & 2u)
        return fail(SGE_BAD_INPUT, "neighbour list of vertex %u is not strictly increasing, out of range, or has a self-loop", h[1]);
    if (h[0] & 4u) return fail(SGE_BAD_INPUT, "CSR is not symmetric at vertex %u", h[2]);
    if (hc[0] != hc[1]) return fail(SGE_BAD_INPUT, "CSR is not symmetric at vertex %u", 0u);
    return SGE_OK;
}
}  // namespace sge_csr_check

extern "C" {

const char *sge_version(void) { return "sge 0.1 (sm_103a, ABI 1)"; }

int sge_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

sge_status sge_graph_create(const uint32_t *offsets, const uint32_t *nbrs, uint32_t n, uint64_t nnz, int device,
                            sge_graph **out) {
    using sge_csr_check::validate_csr_device;
    if (!offsets || (!nbrs && nnz) || !out) return fail(SGE_BAD_INPUT, "sge_graph_create: null argument");
    if (nnz % 2) return fail(SGE_BAD_INPUT, "odd number of directed edges (%llu)", (unsigned long long)nnz);
    if (nnz >= (1ull << 32)) return fail(SGE_BAD_INPUT, "%llu directed edges exceed the uint32 EdgeID range", (unsigned long long)nnz);
    // small graphs are checked on the host before any device is touched;
    // large ones have their offsets checked here and their lists on the device
    const bool on_device = nnz > SGE_HOST_VALIDATE_MAX;
    sge_status st = on_device ? validate_offsets(offsets, n, nnz) : validate_csr(offsets, nbrs, n, nnz);
    if (st != SGE_OK) return st;
    int ndev = sge_device_count();
    if (ndev == 0) return fail(SGE_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(SGE_BAD_INPUT, "device %d out of range (%d visible)", device, ndev);
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(device));
    // upload the CSR; the root edge list is built on the device and the
    // planner statistics from the host arrays (graph_adopt)
    uint32_t *d_off = nullptr, *d_adj = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&d_off, sizeof(uint32_t) * ((size_t)n + 1))) != cudaSuccess ||
        (e = cudaMalloc(&d_adj, sizeof(uint32_t) * std::max<uint64_t>(nnz, 1))) != cudaSuccess) {
        cudaFree(d_off);
        return fail(SGE_OOM, "device allocation of the graph failed: %s", cudaGetErrorString(e));
    }
    if ((e = cudaMemcpy(d_off, offsets, sizeof(uint32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (nnz && (e = cudaMemcpy(d_adj, nbrs, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice)) != cudaSuccess)) {
        cudaFree(d_off);
        cudaFree(d_adj);
        return fail(SGE_CUDA_ERROR, "graph upload failed: %s", cudaGetErrorString(e));
    }
    if (on_device) {
        st = validate_csr_device(d_off, d_adj, n, device);
        if (st != SGE_OK) {
            cudaFree(d_off);
            cudaFree(d_adj);
            return st;
        }
    }
    return graph_adopt(d_off, d_adj, n, nnz, device, out, offsets, nbrs);
}

}  // extern "C"

namespace {
// The checks of validate_csr on the device, one warp per vertex: res[0] |= 2
// (a list not strictly increasing, out of range or with a self-loop; res[1] =
// the smallest such vertex) or 4 (an entry above the diagonal without its
// reverse; res[2] = the smallest such vertex); cnt[0/1] = entries above/below
// the diagonal.  Offsets were checked on the host, so every list is in bounds.
__global__ void csr_check_kernel(const uint32_t *off, const uint32_t *adj, uint32_t n, uint32_t *res,
                                 unsigned long long *cnt) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long up = 0, lo = 0;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
        const uint32_t a = off[v], b = off[v + 1];
        for (uint32_t e = a + lane; e < b; e += 32) {
            const uint32_t w = adj[e];
            if (w >= n || w == v || (e > a && adj[e - 1] >= w)) {
                atomicOr(res, 2u);
                atomicMin(res + 1, v);
                continue;
            }
            if (w < v) { ++lo; continue; }
            ++up;
            const uint32_t wa = off[w];
            if (!contains(adj + wa, off[w + 1] - wa, v)) {
                atomicOr(res, 4u);
                atomicMin(res + 2, v);
            }
        }
    }
    up = warp_sum_u64(up);
    lo = warp_sum_u64(lo);
    if (lane == 0) {
        atomicAdd(cnt, up);
        atomicAdd(cnt + 1, lo);
    }
}

// Root edges of a device CSR: directed edge e = (src(e), adj[e]) is a root
// when adj[e] > src(e); pos[e] is its rank among the roots (CSR order).
__global__ void root_flags_kernel(const uint32_t *off, const uint32_t *adj, uint32_t n, unsigned long long nnz,
                                  uint32_t *flags) {
    const unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    const uint32_t src = ub(off, n + 1, (uint32_t)e) - 1;
    flags[e] = adj[e] > src ? 1u : 0u;
}
__global__ void root_scatter_kernel(const uint32_t *off, const uint32_t *adj, uint32_t n, unsigned long long nnz,
                                    const uint32_t *flags, const uint32_t *pos, uint2 *edges) {
    const unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz || !flags[e]) return;
    const uint32_t src = ub(off, n + 1, (uint32_t)e) - 1;
    edges[pos[e]] = make_uint2(src, adj[e]);
}
}  // namespace

sge_status sge::graph_adopt(uint32_t *d_off, uint32_t *d_adj, uint32_t n, uint64_t nnz, int device,
                            sge_graph **out, const uint32_t *h_off, const uint32_t *h_adj) {
    sge_graph *g = new sge_graph();
    g->device = device;
    g->d_off = d_off;
    g->d_adj = d_adj;
    g->n = n;
    g->nnz = nnz;
    g->m = nnz / 2;
    auto cleanup = [&](sge_status s) { sge_graph_destroy(g); return s; };
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return cleanup(fail(SGE_CUDA_ERROR, "%s", cudaGetErrorString(e)));
    cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&g->ev0)) != cudaSuccess || (e = cudaEventCreate(&g->ev1)) != cudaSuccess)
        return cleanup(fail(SGE_CUDA_ERROR, "stream/event creation: %s", cudaGetErrorString(e)));
    if ((e = cudaMalloc(&g->d_edges, sizeof(uint2) * std::max<uint64_t>(g->m, 1))) != cudaSuccess)
        return cleanup(fail(SGE_OOM, "device allocation of the root edges failed: %s", cudaGetErrorString(e)));
    if (nnz) {
        uint32_t *flags = nullptr, *pos = nullptr;
        if ((e = cudaMalloc(&flags, 4 * nnz)) != cudaSuccess || (e = cudaMalloc(&pos, 4 * nnz)) != cudaSuccess) {
            cudaFree(flags);
            return cleanup(fail(SGE_OOM, "root edge scratch: %s", cudaGetErrorString(e)));
        }
        const unsigned grid = (unsigned)((nnz + 255) / 256);
        root_flags_kernel<<<grid, 256, 0, g->stream>>>(d_off, d_adj, n, nnz, flags);
        sge_status st = device_exclusive_scan(flags, pos, nnz, g->stream);
        if (st == SGE_OK) {
            root_scatter_kernel<<<grid, 256, 0, g->stream>>>(d_off, d_adj, n, nnz, flags, pos, g->d_edges);
            e = cudaStreamSynchronize(g->stream);
            if (e != cudaSuccess) st = fail(SGE_CUDA_ERROR, "root edges: %s", cudaGetErrorString(e));
        }
        cudaFree(flags);
        cudaFree(pos);
        if (st != SGE_OK) return cleanup(st);
    }
    // planner statistics from the host arrays (a copy of the device CSR when
    // it was built on the device: the same numbers as a host-built graph)
    std::vector<uint32_t> off, adj;
    if (!h_off) {
        off.resize((size_t)n + 1);
        adj.resize(std::max<uint64_t>(nnz, 1));
        if ((e = cudaMemcpy(off.data(), d_off, 4 * ((size_t)n + 1), cudaMemcpyDeviceToHost)) != cudaSuccess ||
            (nnz && (e = cudaMemcpy(adj.data(), d_adj, 4 * nnz, cudaMemcpyDeviceToHost)) != cudaSuccess))
            return cleanup(fail(SGE_CUDA_ERROR, "graph read-back: %s", cudaGetErrorString(e)));
        h_off = off.data();
        h_adj = adj.data();
    }
    for (uint32_t v = 0; v < n; ++v) g->max_deg = std::max(g->max_deg, h_off[v + 1] - h_off[v]);
    sge_graph_stats_compute(h_off, h_adj, n, &g->stats);
    sge_status hst = build_hub_index(g, h_off);
    if (hst != SGE_OK) return cleanup(hst);
    *out = g;
    return SGE_OK;
}

extern "C" {

sge_status sge_graph_copy_csr(const sge_graph *g, uint32_t *offsets, uint32_t *nbrs) {
    if (!g || !offsets || (!nbrs && g->nnz)) return fail(SGE_BAD_INPUT, "sge_graph_copy_csr: null argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    CUDA_TRY(cudaMemcpy(offsets, g->d_off, 4 * ((size_t)g->n + 1), cudaMemcpyDeviceToHost));
    if (g->nnz) CUDA_TRY(cudaMemcpy(nbrs, g->d_adj, 4 * g->nnz, cudaMemcpyDeviceToHost));
    return SGE_OK;
}

sge_status sge_graph_destroy(sge_graph *g) {
    if (!g) return SGE_OK;
    DeviceGuard restore_device;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    cudaFree(g->d_off);
    cudaFree(g->d_adj);
    cudaFree(g->d_edges);
    cudaFree(g->d_scratch);
    cudaFree(g->d_batch);
    cudaFree(g->d_hub_bits);
    cudaFree(g->d_hub_slot);
    cudaFree(g->d_labels);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return SGE_OK;
}

sge_status sge_graph_get_info(const sge_graph *g, sge_graph_info *info) {
    if (!g || !info) return fail(SGE_BAD_INPUT, "sge_graph_get_info: null argument");
    info->num_vertices = g->n;
    info->num_directed_edges = g->nnz;
    info->max_degree = g->max_deg;
    info->device_bytes = 4ull * (g->n + 1) + 4ull * g->nnz + 8ull * g->m + g->hub_bytes;
    info->hub_count = g->hub_count;
    info->hub_min_degree = g->hub_min;
    return SGE_OK;
}

sge_status sge_plan_create(const sge_plan_blob *blob, sge_plan **out) {
    if (!out) return fail(SGE_BAD_INPUT, "sge_plan_create: null output");
    sge_status st = sge_plan_validate(blob);
    if (st != SGE_OK) return st;
    sge_plan *p = new sge_plan();
    p->blob = *blob;
    to_devplan(*blob, p->dp);
    *out = p;
    return SGE_OK;
}

sge_status sge_plan_destroy(sge_plan *p) {
    delete p;
    return SGE_OK;
}

sge_status sge_plan_set_tuning(sge_plan *p, const sge_plan_tuning *t) {
    if (!p) return fail(SGE_BAD_INPUT, "sge_plan_set_tuning: null plan");
    if (t) p->tune = *t;
    else p->tune = sge_plan_tuning{};
    return SGE_OK;
}

sge_status sge_plan_set_labels(sge_plan *p, const uint32_t *labels) {
    if (!p) return fail(SGE_BAD_INPUT, "sge_plan_set_labels: null plan");
    if (!labels) {
        p->has_labels = false;
        return SGE_OK;
    }
    if (!p->blob.labeled) return fail(SGE_BAD_INPUT, "the plan was planned without labels (sge_plan_opts.vertex_labels)");
    for (uint32_t u = 0; u < p->blob.k; ++u) p->labels[u] = labels[u];
    p->has_labels = true;
    return SGE_OK;
}

sge_status sge_graph_set_labels(sge_graph *g, const uint32_t *labels) {
    if (!g) return fail(SGE_BAD_INPUT, "sge_graph_set_labels: null graph");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    if (!labels) {
        cudaFree(g->d_labels);
        g->d_labels = nullptr;
        return SGE_OK;
    }
    if (!g->d_labels) CUDA_TRY(cudaMalloc(&g->d_labels, 4ull * std::max<uint32_t>(g->n, 1)));
    CUDA_TRY(cudaMemcpy(g->d_labels, labels, 4ull * g->n, cudaMemcpyHostToDevice));
    return SGE_OK;
}

static sge_status count_impl(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                             uint64_t *counts, uint64_t *instances, sge_stats *stats, double *busy_ms);

sge_status sge_count(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                     uint64_t *counts, uint64_t *instances, sge_stats *stats) {
    return count_impl(g, plans, nplans, opts, counts, instances, stats, nullptr);
}

sge_status sge_count_plan_times(sge_graph *g, const sge_plan *const *plans, uint32_t nplans,
                                const sge_count_opts *opts, uint64_t *counts, double *busy_ms, sge_stats *stats) {
    if (!busy_ms && nplans) return fail(SGE_BAD_INPUT, "sge_count_plan_times: null busy_ms");
    return count_impl(g, plans, nplans, opts, counts, nullptr, stats, busy_ms);
}

static sge_status count_impl(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                             uint64_t *counts, uint64_t *instances, sge_stats *stats, double *busy_ms) {
    auto t_start = std::chrono::steady_clock::now();
    if (!g || (!plans && nplans) || (!counts && nplans)) return fail(SGE_BAD_INPUT, "sge_count: null argument");
    if (nplans == 0) return SGE_OK;
    sge_count_opts o{};
    if (opts) o = *opts;
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    LaunchCfg L;
    sge_status st = prepare_launch(g, plans, nplans, o, g->scratch_bytes, L);
    if (st != SGE_OK) return st;
    if ((st = ensure_scratch(g, L.scratch_bytes)) != SGE_OK) return st;
    if ((st = ensure_batch(g, L.bytes)) != SGE_OK) return st;
    unsigned char *B = g->d_batch;
    CUDA_TRY(cudaMemcpyAsync(B + L.off_plans, L.dps.data(), sizeof(DevPlan) * nplans, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaEventRecord(g->ev0, g->stream));
    uint32_t launches = 0;
    if ((st = enqueue_launch(g, L, B, g->d_scratch, g->stream, launches)) != SGE_OK) return st;
    g->launched = true;
    CUDA_TRY(cudaEventRecord(g->ev1, g->stream));
    std::vector<unsigned long long> hc(nplans);
    uint32_t hflags = 0;
    DevStats hs{};
    CUDA_TRY(cudaMemcpyAsync(hc.data(), B + L.off_counts, 8 * nplans, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaMemcpyAsync(&hflags, B + L.off_flags, 4, cudaMemcpyDeviceToHost, g->stream));
    if (L.want_stats) CUDA_TRY(cudaMemcpyAsync(&hs, B + L.off_stats, sizeof hs, cudaMemcpyDeviceToHost, g->stream));
    std::vector<unsigned long long> hp(busy_ms ? nplans : 0);
    if (busy_ms) CUDA_TRY(cudaMemcpyAsync(hp.data(), B + L.off_ptime, 8 * (size_t)nplans, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    for (uint32_t i = 0; busy_ms && i < nplans; ++i) busy_ms[i] = (double)hp[i] / 1e6;
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    return finish_counts(L, hc.data(), hflags, hs, ms, launches, t_start, plans, counts, instances, stats, o);
}

// GPU root sampling as the planner's cost: each shortlisted candidate counts
// one residue class of the root tasks with the instrumented kernel, and the
// candidate with the least sampled work (algorithmic bytes + 64 B per set
// operation) wins.  Work, not time: a sample's time is set by its slowest
// root, its work by all of them.  A candidate is cut off past 0.5 s, or past
// four times the fastest sample so far; when every candidate is cut off the
// cost model's choice stands.
sge_status sge_plan_pattern_sampled(uint32_t k, uint32_t m, const uint32_t *edges, sge_graph *g,
                                    const sge_plan_opts *opts, uint32_t shortlist, uint64_t sample_stride,
                                    sge_plan_blob *out, double *sampled_ms) {
    if (!g || !out || !edges) return fail(SGE_BAD_INPUT, "sge_plan_pattern_sampled: null argument");
    if (opts && opts->vertex_labels) return fail(SGE_UNSUPPORTED, "sampled planning takes unlabeled patterns");
    if (shortlist == 0) shortlist = 8;
    std::vector<sge_plan_blob> cands(shortlist);
    uint32_t n = 0;
    sge_status st = sge_plan_candidates(k, m, edges, &g->stats, opts, cands.data(), shortlist, &n);
    if (st != SGE_OK) return st;
    if (n == 0) return fail(SGE_BAD_INPUT, "sge_plan_pattern_sampled: no candidate plan");
    sge_count_opts o{};
    o.root_stride = std::max<uint64_t>(sample_stride, 1);
    o.root_offset = 0;
    o.collect_counters = 1;
    uint32_t best = 0;
    double best_ms = -1, best_work = -1;
    for (uint32_t i = 0; i < n; ++i) {
        sge_plan *p = nullptr;
        if ((st = sge_plan_create(&cands[i], &p)) != SGE_OK) return st;
        uint64_t cnt = 0;
        sge_stats ss{};
        o.time_budget_s = best_ms < 0 ? 0.5 : std::min(0.5, std::max(2e-3, 4.0 * best_ms / 1e3));
        st = sge_count(g, &p, 1, &o, &cnt, nullptr, &ss);
        sge_plan_destroy(p);
        double ms = -1;
        if (st == SGE_OK) ms = ss.kernel_ms;
        else if (st != SGE_TIMEOUT) return st;
        if (sampled_ms) sampled_ms[i] = ms;
        if (ms < 0) continue;
        const double work = (double)ss.alg_bytes + 64.0 * (double)ss.set_ops;
        if (best_work < 0 || work < best_work) { best_work = work; best = i; }
        if (best_ms < 0 || ms < best_ms) best_ms = ms;
    }
    if (sampled_ms)
        for (uint32_t i = n; i < shortlist; ++i) sampled_ms[i] = -1;
    *out = cands[best];
    return SGE_OK;
}

// ---- batches replayed from a captured CUDA graph ----
struct sge_batch {
    sge_graph *g = nullptr;
    LaunchCfg L;
    std::vector<const sge_plan *> plans;
    sge_count_opts o{};
    unsigned char *d_buf = nullptr;
    uint32_t *d_scratch = nullptr;
    unsigned char *h_res = nullptr;  // pinned: counts | flags | stats
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t launches = 0;
};

sge_status sge_batch_destroy(sge_batch *b) {
    if (!b) return SGE_OK;
    DeviceGuard restore_device;
    cudaSetDevice(b->g->device);
    cudaStreamSynchronize(b->g->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    cudaFree(b->d_buf);
    cudaFree(b->d_scratch);
    if (b->h_res) cudaFreeHost(b->h_res);
    delete b;
    return SGE_OK;
}

sge_status sge_batch_create(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                            sge_batch **out) {
    if (!g || !plans || nplans == 0 || !out) return fail(SGE_BAD_INPUT, "sge_batch_create: bad argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    sge_batch *b = new sge_batch();
    b->g = g;
    if (opts) b->o = *opts;
    b->plans.assign(plans, plans + nplans);
    auto bail = [&](sge_status st) { sge_batch_destroy(b); return st; };
    sge_status st = prepare_launch(g, plans, nplans, b->o, 0, b->L);
    if (st != SGE_OK) return bail(st);
    cudaError_t e;
    const size_t res_bytes = 8 * (size_t)nplans + 16 + sizeof(DevStats);
    if ((e = cudaMalloc(&b->d_buf, b->L.bytes)) != cudaSuccess || (e = cudaMalloc(&b->d_scratch, std::max<size_t>(b->L.scratch_bytes, 4))) != cudaSuccess ||
        (e = cudaMallocHost(&b->h_res, res_bytes)) != cudaSuccess || (e = cudaEventCreate(&b->ev0)) != cudaSuccess ||
        (e = cudaEventCreate(&b->ev1)) != cudaSuccess)
        return bail(fail(SGE_OOM, "sge_batch_create: %s", cudaGetErrorString(e)));
    if ((e = cudaMemcpy(b->d_buf + b->L.off_plans, b->L.dps.data(), sizeof(DevPlan) * nplans, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail(SGE_CUDA_ERROR, "sge_batch_create: plan upload: %s", cudaGetErrorString(e)));
    // capture: clear counters, both launch phases, read back counts/flags/stats
    if ((e = cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return bail(fail(SGE_CUDA_ERROR, "stream capture: %s", cudaGetErrorString(e)));
    st = enqueue_launch(g, b->L, b->d_buf, b->d_scratch, g->stream, b->launches);
    if (st == SGE_OK) {
        cudaMemcpyAsync(b->h_res, b->d_buf + b->L.off_counts, 8 * (size_t)nplans, cudaMemcpyDeviceToHost, g->stream);
        cudaMemcpyAsync(b->h_res + 8 * (size_t)nplans, b->d_buf + b->L.off_flags, 4, cudaMemcpyDeviceToHost, g->stream);
        cudaMemcpyAsync(b->h_res + 8 * (size_t)nplans + 16, b->d_buf + b->L.off_stats, sizeof(DevStats),
                        cudaMemcpyDeviceToHost, g->stream);
    }
    e = cudaStreamEndCapture(g->stream, &b->graph);
    if (st != SGE_OK) return bail(st);
    if (e != cudaSuccess) return bail(fail(SGE_CUDA_ERROR, "stream capture: %s", cudaGetErrorString(e)));
    if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess)
        return bail(fail(SGE_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(e)));
    *out = b;
    return SGE_OK;
}

sge_status sge_batch_run(sge_batch *b, uint64_t *counts, uint64_t *instances, sge_stats *stats) {
    auto t_start = std::chrono::steady_clock::now();
    if (!b || !counts) return fail(SGE_BAD_INPUT, "sge_batch_run: null argument");
    sge_graph *g = b->g;
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    CUDA_TRY(cudaEventRecord(b->ev0, g->stream));
    CUDA_TRY(cudaGraphLaunch(b->exec, g->stream));
    CUDA_TRY(cudaEventRecord(b->ev1, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    const uint32_t n = b->L.nplans;
    uint32_t hflags = 0;
    DevStats hs{};
    memcpy(&hflags, b->h_res + 8 * (size_t)n, 4);
    memcpy(&hs, b->h_res + 8 * (size_t)n + 16, sizeof hs);
    return finish_counts(b->L, reinterpret_cast<const unsigned long long *>(b->h_res), hflags, hs, ms, b->launches,
                         t_start, b->plans.data(), counts, instances, stats, b->o);
}

sge_status sge_enumerate(sge_graph *g, const sge_plan *p, uint32_t *d_out, uint64_t capacity, uint64_t *n_matches) {
    if (!g || !p || !n_matches || (!d_out && capacity)) return fail(SGE_BAD_INPUT, "sge_enumerate: null argument");
    if (p->blob.tail_len != 1)
        return fail(SGE_BAD_INPUT, "sge_enumerate needs a plan with a one-level tail (plan it without IEP)");
    if (p->blob.labeled) return fail(SGE_UNSUPPORTED, "sge_enumerate takes unlabeled plans");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    DevPlan d = p->dp;
    d.ne = d.k;  // every level is enumerated
    d.ntrie = 0;
    d.hoist_mask = 0;
    d.root_stride = 1;
    d.root_offset = 0;
    d.ntasks = (d.root_kind == SGE_ROOT_ANY) ? 2ull * g->m : g->m;
    d.nbufs = d.k;
    const uint32_t wpb = 8, threads = 256;
    const size_t smem = warp_smem_bytes(0, 1, 1, SGE_MAX_VSLOTS) * wpb;
    CUDA_TRY(cudaFuncSetAttribute(enum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int bps = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, enum_kernel, threads, smem));
    bps = std::max(bps, 1);
    const uint32_t cap = (std::max<uint32_t>(g->max_deg, 1) + 31) & ~31u;
    size_t free_b = 0, tot_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &tot_b));
    const size_t per_block = (size_t)wpb * d.nbufs * cap * sizeof(uint32_t);
    size_t blocks = (size_t)g->num_sms * bps;
    const size_t budget = free_b / 4 + g->scratch_bytes;
    while (blocks > 1 && blocks * per_block > budget) --blocks;
    sge_status st = ensure_scratch(g, blocks * per_block);
    if (st != SGE_OK) return st;
    st = ensure_batch(g, sizeof(DevPlan) + 256);
    if (st != SGE_OK) return st;
    unsigned char *B = g->d_batch;
    unsigned long long *dq = reinterpret_cast<unsigned long long *>(B + sizeof(DevPlan));
    unsigned long long *dn = dq + 1;
    uint32_t *dflags = reinterpret_cast<uint32_t *>(dq + 2);
    CUDA_TRY(cudaMemsetAsync(dq, 0, 24, g->stream));
    CUDA_TRY(cudaMemcpyAsync(B, &d, sizeof(DevPlan), cudaMemcpyHostToDevice, g->stream));
    DevGraph dg = dev_graph(g, true);
    enum_kernel<<<(unsigned)blocks, threads, smem, g->stream>>>(dg, reinterpret_cast<const DevPlan *>(B), dq,
                                                                g->d_scratch, cap, d.nbufs, dflags, d_out, capacity, dn);
    CUDA_TRY(cudaGetLastError());
    unsigned long long n = 0;
    uint32_t flags = 0;
    CUDA_TRY(cudaMemcpyAsync(&n, dn, 8, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaMemcpyAsync(&flags, dflags, 4, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    *n_matches = n;
    if (flags & FLAG_OVERFLOW) return fail(SGE_STACK_OVERFLOW, "a candidate list exceeded the per-level capacity");
    if (n > capacity) return fail(SGE_OOM, "%llu matches exceed the output capacity %llu", n, (unsigned long long)capacity);
    return SGE_OK;
}

sge_status sge_count_host(const uint32_t *offsets, const uint32_t *nbrs, uint32_t n, uint64_t nnz,
                          const sge_plan_blob *blobs, uint32_t nplans, const sge_count_opts *opts, uint64_t *counts,
                          sge_stats *stats) {
    if (!blobs && nplans) return fail(SGE_BAD_INPUT, "sge_count_host: null plans");
    for (uint32_t i = 0; i < nplans; ++i)
        if (blobs[i].labeled) return fail(SGE_UNSUPPORTED, "sge_count_host takes unlabeled plans");
    sge_graph *g = nullptr;
    sge_status st = sge_graph_create(offsets, nbrs, n, nnz, 0, &g);
    if (st != SGE_OK) return st;
    std::vector<sge_plan *> ps(nplans, nullptr);
    for (uint32_t i = 0; i < nplans && st == SGE_OK; ++i) st = sge_plan_create(&blobs[i], &ps[i]);
    if (st == SGE_OK) st = sge_count(g, ps.data(), nplans, opts, counts, nullptr, stats);
    for (auto *p : ps) sge_plan_destroy(p);
    sge_graph_destroy(g);
    return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Counting without device allocation (sge_count_noalloc)
// ---------------------------------------------------------------------------
// The launch's working memory lives in one file-scope device array: a header
// (queue counter, flags), the plan table, then the per-warp candidate lists.
// Host code must not use the array's name as an address (it is a host-side
// stand-in); the device address is looked up once per device with that device
// current (cudaGetSymbolAddress) and passed to the kernel.
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SGE_NOALLOC_SCRATCH_BYTES];

constexpr size_t NOALLOC_HDR = 256;  // queue (u64) + flags (u32)
constexpr size_t NOALLOC_PLANS = (sizeof(DevPlan) * SGE_NOALLOC_MAX_PLANS + 255) & ~(size_t)255;
constexpr size_t NOALLOC_LISTS = NOALLOC_HDR + NOALLOC_PLANS;
constexpr int NOALLOC_MAX_DEVICES = 64;

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Root tasks are the directed edges e of the CSR (source found by binary
// search on the offsets); ASC/DESC plans skip the half with the wrong orientation.
__global__ void __launch_bounds__(256) count_kernel_noalloc(DevGraph g, const DevPlan *__restrict__ plans,
                                                            uint32_t nplans, unsigned long long nnz,
                                                            unsigned long long *queue,
                                                            unsigned long long *counts, uint32_t *lists,
                                                            uint32_t cap, uint32_t bufs_per_warp, uint32_t chunk,
                                                            uint32_t *flags) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t lane = lane_id();
    const uint32_t wib = threadIdx.x >> 5;
    const size_t gwarp = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    Ctx<false> c;
    c.g = g;
    c.buf = lists + gwarp * (size_t)bufs_per_warp * cap;
    c.cap = cap;
    c.flags = flags;
    c.set_ops = c.alg_bytes = c.partial = 0;
    WarpState &W = setup_warp(smem_raw, wib, 0u, 0u, SGE_MAX_TAIL, 16u, SGE_MAX_VSLOTS, c);  // no pinned tables here
    c.tstart = 0;
    c.deadline = 0;
    const unsigned long long total = nnz * nplans;
    int cur = -1;
    unsigned long long acc = 0;
    while (true) {
        unsigned long long t0 = 0;
        if (lane == 0) t0 = atomicAdd(queue, (unsigned long long)chunk);
        t0 = __shfl_sync(FULL_MASK, t0, 0);
        if (t0 >= total) break;
        if (*(volatile uint32_t *)flags & FLAG_OVERFLOW) break;
        const unsigned long long t1 = min(t0 + chunk, total);
        for (unsigned long long t = t0; t < t1; ++t) {
            const int pi = (int)(t / nnz);
            if (pi != cur) {
                if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc * plans[cur].mult);
                acc = 0;
                cur = pi;
            }
            const DevPlan &P = plans[cur];
            const uint32_t e = (uint32_t)(t - (unsigned long long)pi * nnz);
            const uint32_t u = ub(g.off, g.n + 1, e) - 1;  // source of directed edge e
            const uint32_t v = g.adj[e];
            if (P.root_kind == SGE_ROOT_ASC && !(u < v)) continue;
            if (P.root_kind == SGE_ROOT_DESC && !(u > v)) continue;
            acc += run_root<false>(P, W, c, u, v);
        }
    }
    if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc * plans[cur].mult);
}

}  // namespace

extern "C" sge_status sge_count_noalloc(const uint32_t *d_offsets, const uint32_t *d_nbrs, uint32_t n, uint64_t nnz,
                                        uint32_t max_degree, const sge_plan_blob *plans, uint32_t nplans,
                                        uint64_t *d_counts, void *stream_) {
    if (!d_offsets || (!d_nbrs && nnz) || (!plans && nplans) || (!d_counts && nplans))
        return fail(SGE_BAD_INPUT, "sge_count_noalloc: null argument");
    if (nplans == 0) return SGE_OK;
    if (nplans > SGE_NOALLOC_MAX_PLANS)
        return fail(SGE_UNSUPPORTED, "sge_count_noalloc: %u plans (limit %u)", nplans, SGE_NOALLOC_MAX_PLANS);
    if (nnz >= (1ull << 32)) return fail(SGE_BAD_INPUT, "%llu directed edges exceed the uint32 EdgeID range", (unsigned long long)nnz);
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(SGE_UNSUPPORTED, "device %d beyond the set-up table", dev);
    // The array's device address: looked up again on every call made outside
    // stream capture (a context torn down and rebuilt, e.g. after
    // cudaDeviceReset, reloads the module and may move the array); a call
    // made while `stream` is capturing uses the address of this device's last
    // uncaptured call, so one such call must come first.
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    CUDA_TRY(cudaStreamIsCapturing(stream, &cap_status));
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (cap_status == cudaStreamCaptureStatusNone) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return fail(SGE_CUDA_ERROR, "cudaGetSymbolAddress(static scratch) on device %d: %s", dev,
                            cudaGetErrorString(e));
            g_noalloc_ptr[dev] = p;
        } else if (!g_noalloc_ptr[dev]) {
            return fail(SGE_BAD_INPUT,
                        "sge_count_noalloc: first call on device %d made during stream capture; make one call "
                        "outside capture first", dev);
        }
        base = g_noalloc_ptr[dev];
    }
    // plans: validate, convert, copy into the array's plan table in one copy
    uint32_t nbufs = 1;
    std::vector<DevPlan> dps(nplans);
    for (uint32_t i = 0; i < nplans; ++i) {
        sge_status st = sge_plan_validate(&plans[i]);
        if (st != SGE_OK) return st;
        if (plans[i].labeled) return fail(SGE_UNSUPPORTED, "sge_count_noalloc takes unlabeled plans");
        DevPlan &dp = dps[i];
        to_devplan(plans[i], dp);
        dp.task_begin = 0;
        dp.ntasks = nnz;
        dp.root_stride = 1;
        dp.root_offset = 0;
        nbufs = std::max(nbufs, dp.nbufs);
    }
    CUDA_TRY(cudaMemcpyAsync(static_cast<unsigned char *>(base) + NOALLOC_HDR, dps.data(), sizeof(DevPlan) * nplans,
                             cudaMemcpyHostToDevice, stream));
    const uint32_t cap = (std::max<uint32_t>(max_degree, 1) + 31) & ~31u;
    const size_t per_warp = (size_t)nbufs * cap * sizeof(uint32_t);
    const size_t avail = SGE_NOALLOC_SCRATCH_BYTES - NOALLOC_LISTS;
    const uint32_t wpb = 8, threads = wpb * 32;
    const size_t smem = warp_smem_bytes(0, SGE_MAX_TAIL, 16, SGE_MAX_VSLOTS) * wpb;
    size_t max_blocks = avail / (per_warp * wpb);
    if (max_blocks == 0)
        return fail(SGE_UNSUPPORTED,
                    "sge_count_noalloc: %u levels x max degree %u need %zu bytes per 8-warp block; the static "
                    "scratch holds %zu", nbufs, max_degree, per_warp * wpb, avail);
    int bps = 0, sms = 0;
    CUDA_TRY(cudaFuncSetAttribute(count_kernel_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, count_kernel_noalloc, threads, smem));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t blocks = std::max<size_t>(1, std::min<size_t>(max_blocks, (size_t)std::max(bps, 1) * sms));
    // clear what must start at zero: queue, flags, and the caller's counts
    CUDA_TRY(cudaMemsetAsync(base, 0, NOALLOC_HDR, stream));
    CUDA_TRY(cudaMemsetAsync(d_counts, 0, sizeof(uint64_t) * nplans, stream));
    DevGraph dg{d_offsets, d_nbrs, nullptr, n, nnz / 2, nullptr, nullptr, 0u, 0xFFFFFFFFu};
    unsigned char *B = static_cast<unsigned char *>(base);
    count_kernel_noalloc<<<(unsigned)blocks, threads, smem, stream>>>(
        dg, reinterpret_cast<const DevPlan *>(B + NOALLOC_HDR), nplans, nnz,
        reinterpret_cast<unsigned long long *>(B), reinterpret_cast<unsigned long long *>(d_counts),
        reinterpret_cast<uint32_t *>(B + NOALLOC_LISTS), cap, nbufs, 4, reinterpret_cast<uint32_t *>(B + 8));
    CUDA_TRY(cudaGetLastError());
    uint32_t flags = 0;
    CUDA_TRY(cudaMemcpyAsync(&flags, B + 8, sizeof flags, cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (flags & FLAG_OVERFLOW)
        return fail(SGE_STACK_OVERFLOW, "a candidate list exceeded max_degree %u (pass a true upper bound)", max_degree);
    return SGE_OK;
}

// ---- bag relations ----
namespace {

// first[v] = first level-1 node under key v: the child offset of the first
// level-0 node with value >= v (all level-1 nodes when there is none).
__global__ void trie_first_kernel(const uint32_t *val0, const unsigned long long *child0, unsigned long long len0,
                                  unsigned long long len1, uint32_t n, unsigned long long *first) {
    const unsigned long long v = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (v > n) return;
    unsigned long long lo = 0, w = len0;
    while (w > 0) {
        const unsigned long long half = w >> 1;
        if (val0[lo + half] < v) { lo += half + 1; w -= half + 1; }
        else w = half;
    }
    first[v] = lo < len0 ? child0[lo] : len1;
}

void free_rel(BagRel &r) {
    sge_trie_free(&r.trie);
    cudaFree(r.first);
    r.first = nullptr;
}

// The bag's sub-pattern planned for all of its embeddings: no symmetry
// restrictions, both orientations of every root edge, every earlier level
// that is not a parent excluded (injectivity).
void strip_restrictions(sge_plan_blob &b) {
    for (uint32_t i = 0; i < SGE_MAX_K; ++i) b.lower[i] = b.upper[i] = 0;
    b.root_kind = SGE_ROOT_ANY;
    for (uint32_t i = 1; i < b.k; ++i) {
        const uint32_t below = i < b.num_enum ? (1u << i) - 1u : (1u << b.num_enum) - 1u;
        b.check[i] = below & ~b.parents[i];
    }
    b.num_restrictions = 0;
    b.count_multiplier = 1;
    b.single_bag = 0;
}

// One relation: count its tuples, enumerate them, sort, build the trie and
// its dense first level.  *skipped is set (and nothing built) when the
// relation holds more than max_rows tuples.
sge_status build_rel(sge_graph *g, const sge_plan_blob &blob, uint32_t arity, uint64_t max_rows, size_t bag,
                     BagRel &r, bool *skipped) {
    *skipped = false;
    sge_plan *sp = nullptr;
    sge_status st = sge_plan_create(&blob, &sp);
    if (st != SGE_OK) return st;
    uint64_t cnt = 0, rows = 0;
    const sge_plan *cp = sp;
    st = sge_count(g, &cp, 1, nullptr, &cnt, &rows, nullptr);
    if (st == SGE_OK && rows > max_rows) {
        sge_plan_destroy(sp);
        *skipped = true;
        return SGE_OK;
    }
    uint32_t *d = nullptr;
    if (st == SGE_OK && rows) {
        cudaError_t e = cudaMalloc(&d, rows * arity * 4ull);
        if (e != cudaSuccess) st = fail(SGE_OOM, "bag %zu: %llu tuples: %s", bag, (unsigned long long)rows, cudaGetErrorString(e));
    }
    uint64_t n2 = 0;
    if (st == SGE_OK && rows) st = sge_enumerate(g, sp, d, rows, &n2);
    if (st == SGE_OK && rows && n2 != rows)
        st = fail(SGE_CUDA_ERROR, "bag %zu: enumerated %llu tuples, counted %llu", bag, (unsigned long long)n2,
                  (unsigned long long)rows);
    if (st == SGE_OK && rows) st = sge_sort_tuples(d, rows, arity);
    if (st == SGE_OK) st = sge_trie_build(d, rows, arity, &r.trie);
    cudaFree(d);
    sge_plan_destroy(sp);
    if (st != SGE_OK) return st;
    r.rows = rows;
    CUDA_TRY(cudaMalloc(&r.first, 8ull * (g->n + 1)));
    if (rows == 0) {
        CUDA_TRY(cudaMemset(r.first, 0, 8ull * (g->n + 1)));
    } else {
        trie_first_kernel<<<(unsigned)((g->n + 256) / 256), 256>>>(r.trie.values[0], r.trie.child[0],
                                                                  r.trie.level_len[0], r.trie.level_len[1], g->n,
                                                                  r.first);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaDeviceSynchronize());
    }
    return SGE_OK;
}

}  // namespace

extern "C" {

sge_status sge_bags_create(sge_graph *g, uint32_t k, uint32_t m, const uint32_t *edges, const char *plan_text,
                           uint64_t max_rows, sge_bags **out) {
    if (!g || !edges || !plan_text || !out) return fail(SGE_BAD_INPUT, "sge_bags_create: null argument");
    *out = nullptr;
    if (k < 3 || k > SGE_MAX_K) return fail(SGE_BAD_INPUT, "pattern k=%u outside 3..%u", k, SGE_MAX_K);
    uint32_t adj[SGE_MAX_K] = {};
    for (uint32_t e = 0; e < m; ++e) {
        const uint32_t a = edges[2 * e], b = edges[2 * e + 1];
        if (a >= k || b >= k || a == b) return fail(SGE_BAD_INPUT, "pattern edge %u (%u,%u) is invalid", e, a, b);
        adj[a] |= 1u << b;
        adj[b] |= 1u << a;
    }
    std::vector<std::vector<uint32_t>> bags;
    sge_status st = parse_bag_text(k, plan_text, bags);
    if (st != SGE_OK) return st;
    std::vector<uint32_t> mask(bags.size(), 0);
    for (size_t b = 0; b < bags.size(); ++b)
        for (uint32_t u : bags[b]) mask[b] |= 1u << u;
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(g->device));
    sge_bags *B = new sge_bags();
    B->g = g;
    B->device = g->device;
    B->k = k;
    auto bail = [&](sge_status s) {
        sge_bags_destroy(B);
        return s;
    };
    // every bag but the global one (printed last)
    for (size_t b = 0; b + 1 < bags.size(); ++b) {
        uint32_t others = 0;
        for (size_t c = 0; c < bags.size(); ++c)
            if (c != b) others |= mask[c];
        const uint32_t own = mask[b] & ~others;
        const uint32_t size = (uint32_t)__builtin_popcount(mask[b]);
        if (__builtin_popcount(own) != 1 || size < 3 || size > 4) continue;
        BagRel r;
        r.priv = (uint32_t)__builtin_ctz(own);
        if (adj[r.priv] & ~mask[b]) continue;  // (a decomposition keeps a vertex's edges in its only bag)
        uint32_t col[SGE_MAX_K];
        for (uint32_t msk = mask[b] & ~own; msk; msk &= msk - 1) {
            const uint32_t u = (uint32_t)__builtin_ctz(msk);
            col[u] = r.nkeys;
            r.keys[r.nkeys++] = u;
        }
        col[r.priv] = r.nkeys;
        std::vector<uint32_t> sub;
        for (uint32_t e = 0; e < m; ++e) {
            const uint32_t a = edges[2 * e], c = edges[2 * e + 1];
            if (((mask[b] >> a) & 1u) && ((mask[b] >> c) & 1u)) { sub.push_back(col[a]); sub.push_back(col[c]); }
        }
        sge_plan_opts o{};
        o.join_style = SGE_JOIN_WCOJ;
        o.use_iep = 0;
        o.max_tail = 1;
        sge_plan_blob blob;
        // a bag whose sub-pattern is not connected is not planned (its tail
        // level keeps intersecting adjacency lists)
        if (sge_plan_pattern_stats(size, (uint32_t)sub.size() / 2, sub.data(), &g->stats, &o, &blob) != SGE_OK) continue;
        strip_restrictions(blob);
        // (the sort and the trie index rows with 32 bits)
        const uint64_t cap = std::min<uint64_t>(max_rows ? max_rows : ~0ull, 0xFFFFFFFFull);
        bool skipped = false;
        st = build_rel(g, blob, size, cap, b, r, &skipped);
        if (st != SGE_OK) {
            free_rel(r);
            return bail(st);
        }
        if (skipped) {
            ++B->skipped;
            continue;
        }
        B->bytes += 8ull * (g->n + 1);
        for (uint32_t l = 0; l < size; ++l)
            B->bytes += 4ull * r.trie.level_len[l] + (l + 1 < size ? 8ull * (r.trie.level_len[l] + 1) : 0ull);
        B->rels.push_back(r);
    }
    if (!B->rels.empty()) {
        std::vector<DevTrie> dt(B->rels.size());
        for (size_t i = 0; i < B->rels.size(); ++i) {
            const BagRel &r = B->rels[i];
            DevTrie &t = dt[i];
            memset(&t, 0, sizeof t);
            t.first = r.first;
            t.nkeys = r.nkeys;
            for (uint32_t l = 1; l <= r.nkeys; ++l) t.val[l] = r.trie.values[l];
            for (uint32_t l = 1; l < r.nkeys; ++l) t.child[l] = r.trie.child[l];
        }
        cudaError_t e = cudaMalloc(&B->d_tries, sizeof(DevTrie) * dt.size());
        if (e == cudaSuccess) e = cudaMemcpy(B->d_tries, dt.data(), sizeof(DevTrie) * dt.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(fail(SGE_CUDA_ERROR, "sge_bags_create: %s", cudaGetErrorString(e)));
    }
    *out = B;
    return SGE_OK;
}

sge_status sge_bags_info(const sge_bags *b, uint32_t *num_relations, uint64_t *rows, uint64_t *device_bytes,
                         uint32_t *own_vertices, uint32_t *num_skipped) {
    if (!b) return fail(SGE_BAD_INPUT, "sge_bags_info: null bags");
    uint64_t total = 0;
    for (size_t i = 0; i < b->rels.size(); ++i) {
        total += b->rels[i].rows;
        if (own_vertices) own_vertices[i] = b->rels[i].priv;
    }
    if (num_relations) *num_relations = (uint32_t)b->rels.size();
    if (rows) *rows = total;
    if (device_bytes) *device_bytes = b->bytes;
    if (num_skipped) *num_skipped = b->skipped;
    return SGE_OK;
}

sge_status sge_bags_destroy(sge_bags *b) {
    if (!b) return SGE_OK;
    DeviceGuard restore_device;
    cudaSetDevice(b->device);
    for (auto &r : b->rels) free_rel(r);
    cudaFree(b->d_tries);
    delete b;
    return SGE_OK;
}

sge_status sge_plan_use_bags(sge_plan *p, const sge_bags *b, uint32_t *levels) {
    if (!p) return fail(SGE_BAD_INPUT, "sge_plan_use_bags: null plan");
    if (levels) *levels = 0;
    // back to the plan's own device form (its tuning is kept)
    to_devplan(p->blob, p->dp);
    p->bags = nullptr;
    if (!b) return SGE_OK;
    const sge_plan_blob &bl = p->blob;
    if (b->k != bl.k) return fail(SGE_BAD_INPUT, "bags of a %u-vertex pattern, plan of %u vertices", b->k, bl.k);
    if (bl.join_style != SGE_JOIN_WCOJ) return fail(SGE_UNSUPPORTED, "bag relations need a WCOJ plan");
    if (bl.labeled) return fail(SGE_UNSUPPORTED, "bag relations take unlabeled plans");
    uint32_t level_of[SGE_MAX_K];
    for (uint32_t i = 0; i < bl.k; ++i) level_of[bl.order[i]] = i;
    DevPlan &d = p->dp;
    for (uint32_t i = 0; i < SGE_MAX_K; ++i) d.tri[i] = -1;
    uint32_t j = 0;
    for (size_t ri = 0; ri < b->rels.size() && j < 2; ++ri) {
        const BagRel &r = b->rels[ri];
        const uint32_t li = level_of[r.priv];
        if (li < bl.num_enum) continue;  // its own vertex is enumerated, not a tail level
        bool keyed = true;
        for (uint32_t c = 0; c < r.nkeys; ++c) keyed &= level_of[r.keys[c]] < bl.num_enum;
        if (!keyed) continue;
        d.tri[li] = (int8_t)j;
        d.trel[j] = (uint8_t)ri;
        for (uint32_t c = 0; c < r.nkeys; ++c) d.tkey[j][c] = (uint8_t)level_of[r.keys[c]];
        d.hoist_mask &= ~(1u << li);  // the trie replaces the hoisted intersection
        ++j;
    }
    if (j == 0) return SGE_OK;
    d.ntrie = j;
    d.tries = b->d_tries;
    d.pair_direct = 0;
    // N(m[0]) / N(m[1]) / level 2's list stay pinned only for levels that still probe them
    d.pin_mask = 0;
    if (bl.num_enum >= 3)
        for (uint32_t i = 3; i < bl.k; ++i) {
            if (i >= bl.num_enum && d.tri[i] >= 0) continue;
            d.pin_mask |= bl.parents[i] & 3u;
            if (bl.base[i] == 2) d.pin_mask |= 4u;
        }
    p->bags = b;
    if (levels) *levels = j;
    return SGE_OK;
}

}  // extern "C"
