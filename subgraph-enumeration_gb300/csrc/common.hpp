// Internal helpers shared by the host translation units of libsge.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <string>
#include <vector>
#include "sge.h"

namespace sge {

// Thread-local last-error message (sge_last_error).
void set_error(const char *fmt, ...);
const char *last_error();

// Returns `st` after recording a formatted message.
sge_status fail(sge_status st, const char *fmt, ...);

// Bags of a decomposition printed by the reference (HyperTree::writeToStream:
// "num bags: N", then one comma-separated attribute order per bag, the global
// bag last; or an order file): each bag's attributes in its order.  Checks
// that every attribute is a vertex of the k-vertex pattern, named once per
// bag, and that the bags cover every vertex.
sge_status parse_bag_text(uint32_t k, const char *text, std::vector<std::vector<uint32_t>> &bags);

// splitmix64: the deterministic counter-based generator behind every seeded
// generator and sampler in the library (same stream on every host).
static inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(splitmix64(seed ^ 0x5347454E5347454Eull)) {}
    uint64_t next() { s += 0x9E3779B97F4A7C15ull; uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull; z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31); }
    // uniform in [0, n) without modulo bias worth caring about for n << 2^64
    uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
};

// How the executor runs a plan's last levels.  The engine builds its device
// plan from this, and the planner's cost model prices the same shape.
//  - hoist: a WCOJ tail level whose parents (two or more) are all matched
//    before the last enumerated level has its list computed once, right
//    after level hoist_at (its last parent, at least level 1);
//  - pair: the last two enumerated levels run as one step flattened over
//    (candidate, element) pairs, which needs every tail list to be
//    independent of level ne-2's per-candidate state (no tail reuses level
//    ne-1's stored list or is hoisted right after level ne-2; with
//    exploration, no tail's running list intersects N(m[ne-2]) into earlier
//    parents, which the DFS would build once per candidate of level ne-2);
//  - pair_direct: a single tail level that neither has level ne-1 as a
//    parent nor is bounded by it is counted per pair inline, when its lists
//    reduce to one.
struct ExecShape {
    uint32_t hoist_mask = 0;
    uint8_t hoist_at[SGE_MAX_K] = {};
    bool pair = false, pair_direct = false;
};

inline ExecShape exec_shape(const sge_plan_blob &b) {
    ExecShape x;
    const uint32_t ne = b.num_enum, k = b.k;
    if (b.join_style == SGE_JOIN_WCOJ && ne >= 3)
        for (uint32_t i = ne; i < k; ++i) {
            const uint32_t par = b.parents[i];
            const uint32_t last = 31u - (uint32_t)__builtin_clz(par);
            if (__builtin_popcount(par) >= 2 && last + 1 < ne) {
                x.hoist_mask |= 1u << i;
                x.hoist_at[i] = (uint8_t)(last < 1 ? 1u : last);
            }
        }
    if (ne >= 4) {
        const uint32_t a = ne - 2;
        bool ok = true;
        for (uint32_t i = ne; i < k; ++i) {
            if (b.join_style == SGE_JOIN_WCOJ && b.base[i] == (int)(ne - 1)) ok = false;
            if (((x.hoist_mask >> i) & 1u) && x.hoist_at[i] == a) ok = false;
            if (b.join_style == SGE_JOIN_EXPLORATION && ((b.parents[i] >> a) & 1u) &&
                (b.parents[i] & ((1u << a) - 1u)))
                ok = false;
        }
        x.pair = ok;
    }
    x.pair_direct = x.pair && b.tail_mode == SGE_TAIL_SINGLE && b.tail_len == 1 && ne < k &&
                    !(((b.parents[ne] | b.lower[ne] | b.upper[ne]) >> (ne - 1)) & 1u);
    return x;
}

}  // namespace sge
