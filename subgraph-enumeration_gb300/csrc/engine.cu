// GB300 (sm_103a) execution engine: device graph, compiled plans, and the
// persistent counting kernel behind sge_count.
//
// Replaces the reference's join drivers: sharedJoin / globalJoin / traverse
// (matching/join.cpp:812-1691) and their OpenMP split parSharedJoin /
// subtreeSharedJoin (matching/parallel.cpp:167-1844).  The reference gives one
// OpenMP task per root (a candidate of the first shared attribute, or a data
// edge, parallel.cpp:1272,1414); here one warp owns one root edge at a time,
// taken from a global atomic queue, and runs the plan's depth-first search
// with all 32 lanes cooperating on every set operation:
//   - candidate generation = bound trimming (setBeginPos/setEndPos,
//     utility/utils.cpp:581-612) + k-way intersection (ComputeCandidates /
//     MultiIntersection, utility/compute_set_intersection.cpp:10-87,308-342)
//     done as a warp-parallel membership test of the shortest list against
//     the others (binary search per lane), compacted with ballot/popc;
//   - the last tail_len levels are counted, not enumerated: numResults
//     (relation/relation.cpp:290-338), choosec (utils.cpp:80-94) and the
//     inclusion–exclusion of numUniqueCombine (utils.cpp:290-350);
//   - exploration style (-i) keeps running candidate lists per later level,
//     updated as soon as a parent is matched (join.cpp:266-307).
// Counts are exact uint64 (wrapping like the reference's size_t).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "common.hpp"

using namespace sge;

#define FULL_MASK 0xFFFFFFFFu
#define SGE_MAX_BUFS 32

namespace {

struct DevGraph {
    const uint32_t *off;    // n+1
    const uint32_t *adj;    // nnz
    const uint2 *edges;     // m undirected edges (u<v)
    uint32_t n;
    uint64_t m;
};

// Compact device form of sge_plan_blob (+ batch bookkeeping).
struct DevPlan {
    uint32_t parents[SGE_MAX_K], lower[SGE_MAX_K], upper[SGE_MAX_K], check[SGE_MAX_K], rest[SGE_MAX_K];
    int32_t base[SGE_MAX_K];
    uint32_t after[SGE_MAX_K];       // exploration: later levels having this level as a parent
    int8_t slot[SGE_MAX_K][SGE_MAX_K];  // exploration: buffer slot of version (j, i), -1 = direct N(m[j])
    uint32_t k, ne, T, tail_mode, join_style, root_kind, nparts, nbufs;
    int32_t part_coef[SGE_MAX_PARTITIONS];
    uint32_t part_nblocks[SGE_MAX_PARTITIONS];
    uint32_t part_block[SGE_MAX_PARTITIONS][SGE_MAX_TAIL];
    unsigned long long task_begin, ntasks;        // this batch's task range for the plan
    unsigned long long root_stride, root_offset;  // task j of the plan = root root_offset + j*root_stride
};

struct DevStats {
    unsigned long long set_ops, alg_bytes, partial, roots;
};

// Flags written by kernels (never trapped on): bit0 overflow, bit1 timeout.
enum { FLAG_OVERFLOW = 1u, FLAG_TIMEOUT = 2u };

struct WarpState {
    uint32_t m[SGE_MAX_K];
    uint32_t pos[SGE_MAX_K];
    uint32_t cnt[SGE_MAX_K];
    const uint32_t *list[SGE_MAX_K];
    uint32_t vlen[SGE_MAX_K][SGE_MAX_K];  // exploration version lengths (j, i)
    unsigned long long S[16];
};

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

__device__ __forceinline__ unsigned long long binom_exact(unsigned long long n, uint32_t r) {
    if (n < r) return 0ull;
    unsigned __int128 acc = 1;
    for (uint32_t i = 0; i < r; ++i) acc = acc * (unsigned __int128)(n - i) / (unsigned __int128)(i + 1);
    return (unsigned long long)acc;
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

__device__ __forceinline__ void nbr(const DevGraph &g, uint32_t v, const uint32_t *&p, uint32_t &len) {
    uint32_t a = __ldg(g.off + v), b = __ldg(g.off + v + 1);
    p = g.adj + a;
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
    unsigned long long set_ops, alg_bytes, partial;
};

// Base list of level i for WCOJ: a reused stored list or the smallest parent
// list; `rest` returns the parents still to test.
template <bool STATS>
__device__ __forceinline__ void wcoj_base(const DevPlan &P, const WarpState &W, Ctx<STATS> &c, uint32_t i,
                                          const uint32_t *&bp, uint32_t &blen, uint32_t &rest) {
    if (P.base[i] >= 0) {
        uint32_t l = (uint32_t)P.base[i];
        bp = W.list[l];
        blen = W.cnt[l];
        rest = P.rest[i];
    } else {
        uint32_t best = 0, bestlen = 0xFFFFFFFFu;
        const uint32_t *bestp = nullptr;
        for (uint32_t msk = P.parents[i]; msk; msk &= msk - 1) {
            uint32_t j = __ffs(msk) - 1;
            const uint32_t *p;
            uint32_t len;
            nbr(c.g, W.m[j], p, len);
            if (STATS) c.alg_bytes += 8;
            if (len < bestlen) { bestlen = len; bestp = p; best = j; }
        }
        bp = bestp;
        blen = bestlen;
        rest = P.parents[i] & ~(1u << best);
    }
}

// Warp-cooperative filter of [bp, bp+blen) by membership in all parent lists
// of `rest` and by the exclusion set of level i; stores the survivors (in
// order) to out when STORE.  Returns the survivor count (warp-uniform).
template <bool STATS, bool STORE>
__device__ __forceinline__ uint32_t setop(const DevPlan &P, const WarpState &W, Ctx<STATS> &c, uint32_t i,
                                          const uint32_t *bp, uint32_t blen, uint32_t rest, uint32_t *out) {
    const uint32_t lane = lane_id();
    const uint32_t *lp[SGE_MAX_K];
    uint32_t ll[SGE_MAX_K];
    uint32_t nl = 0;
    for (uint32_t msk = rest; msk; msk &= msk - 1) {
        uint32_t j = __ffs(msk) - 1;
        nbr(c.g, W.m[j], lp[nl], ll[nl]);
        if (STATS) c.alg_bytes += 8ull + 4ull * ll[nl];
        ++nl;
    }
    if (STATS) { c.set_ops += 1; c.alg_bytes += 4ull * blen; }
    uint32_t total = 0;
    for (uint32_t off = 0; off < blen; off += 32) {
        uint32_t idx = off + lane;
        bool ok = idx < blen;
        uint32_t x = ok ? bp[idx] : 0u;
        for (uint32_t l = 0; l < nl && ok; ++l) ok = contains(lp[l], ll[l], x);
        if (ok) ok = !excluded(P, W, i, x);
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
template <bool STATS>
__device__ __forceinline__ bool build_level_wcoj(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t i) {
    const uint32_t *bp;
    uint32_t blen, rest;
    wcoj_base(P, W, c, i, bp, blen, rest);
    Bounds b = level_bounds(P, W, i);
    trim(bp, blen, b);
    if (rest == 0) {
        // the base list itself (exclusions are applied while iterating)
        __syncwarp();
        if (lane_id() == 0) { W.list[i] = bp; W.cnt[i] = blen; }
        __syncwarp();
        return true;
    }
    uint32_t *out = c.buf + (size_t)i * c.cap;
    uint32_t n = setop<STATS, true>(P, W, c, i, bp, blen, rest, out);
    __syncwarp();
    if (lane_id() == 0) { W.list[i] = out; W.cnt[i] = n; }
    __syncwarp();
    if (n > c.cap) {
        if (lane_id() == 0) atomicOr(c.flags, FLAG_OVERFLOW);
        return false;
    }
    return true;
}

// Exploration: version (j, i) list pointer.
template <bool STATS>
__device__ __forceinline__ const uint32_t *version_ptr(const DevPlan &P, const WarpState &W, const Ctx<STATS> &c,
                                                       uint32_t j, uint32_t i) {
    int s = P.slot[j][i];
    if (s < 0) return c.g.adj + __ldg(c.g.off + W.m[j]);
    return c.buf + (size_t)s * c.cap;
}

// Exploration: after level j is matched, intersect N(m[j]) into the running
// list of every later level that has j as a parent.  false = prune (empty) or
// overflow.
template <bool STATS>
__device__ __forceinline__ bool explore_update(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t j) {
    const uint32_t lane = lane_id();
    for (uint32_t msk = P.after[j]; msk; msk &= msk - 1) {
        uint32_t i = __ffs(msk) - 1;
        uint32_t below = P.parents[i] & ((1u << j) - 1u);
        if (below == 0) {
            uint32_t a = __ldg(c.g.off + W.m[j]), bnd = __ldg(c.g.off + W.m[j] + 1);
            if (STATS) c.alg_bytes += 8;
            __syncwarp();
            if (lane == 0) W.vlen[j][i] = bnd - a;
            __syncwarp();
            if (bnd == a) return false;
            continue;
        }
        uint32_t pj = 31 - __clz(below);  // previous parent of i
        const uint32_t *prev = version_ptr(P, W, c, pj, i);
        uint32_t plen = W.vlen[pj][i];
        const uint32_t *np;
        uint32_t nl;
        nbr(c.g, W.m[j], np, nl);
        uint32_t *out = c.buf + (size_t)P.slot[j][i] * c.cap;
        if (STATS) { c.set_ops += 1; c.alg_bytes += 8ull + 4ull * (plen + nl); }
        uint32_t total = 0;
        // probe the longer list with the shorter one
        const bool swap = nl < plen;
        const uint32_t *sp = swap ? np : prev;
        uint32_t sl = swap ? nl : plen;
        const uint32_t *lp = swap ? prev : np;
        uint32_t ll = swap ? plen : nl;
        for (uint32_t off = 0; off < sl; off += 32) {
            uint32_t idx = off + lane;
            bool ok = idx < sl;
            uint32_t x = ok ? sp[idx] : 0u;
            if (ok) ok = contains(lp, ll, x);
            uint32_t bal = __ballot_sync(FULL_MASK, ok);
            uint32_t p = total + __popc(bal & ((1u << lane) - 1u));
            if (ok && p < c.cap) out[p] = x;
            total += __popc(bal);
        }
        __syncwarp();
        if (lane == 0) W.vlen[j][i] = total;
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
    uint32_t blen = W.vlen[lastp][i];
    Bounds b = level_bounds(P, W, i);
    trim(bp, blen, b);
    __syncwarp();
    if (lane_id() == 0) { W.list[i] = bp; W.cnt[i] = blen; }
    __syncwarp();
}

// Leaf count of the tail levels [ne, k) for the current partial match.
template <bool STATS>
__device__ unsigned long long tail_count(const DevPlan &P, WarpState &W, Ctx<STATS> &c) {
    const uint32_t lane = lane_id();
    const uint32_t ne = P.ne, T = P.T;
    const bool explore = P.join_style == SGE_JOIN_EXPLORATION;
    const uint32_t passes = (P.tail_mode == SGE_TAIL_IEP) ? T : 1u;
    for (uint32_t t = 0; t < passes; ++t) {
        const uint32_t i = ne + t;
        const uint32_t *bp;
        uint32_t blen, rest;
        if (explore) {
            uint32_t lastp = 31 - __clz(P.parents[i]);
            bp = version_ptr(P, W, c, lastp, i);
            blen = W.vlen[lastp][i];
            rest = 0;
        } else {
            wcoj_base(P, W, c, i, bp, blen, rest);
        }
        Bounds b = level_bounds(P, W, i);
        trim(bp, blen, b);
        // rest lists of t
        const uint32_t *lp[SGE_MAX_K];
        uint32_t ll[SGE_MAX_K];
        uint32_t nl = 0;
        for (uint32_t msk = rest; msk; msk &= msk - 1) {
            uint32_t j = __ffs(msk) - 1;
            nbr(c.g, W.m[j], lp[nl], ll[nl]);
            if (STATS) c.alg_bytes += 8ull + 4ull * ll[nl];
            ++nl;
        }
        // other tail positions u > t (IEP only)
        const uint32_t nu = (P.tail_mode == SGE_TAIL_IEP) ? (T - 1 - t) : 0u;
        Bounds ub_[SGE_MAX_TAIL];
        const uint32_t *up_[SGE_MAX_TAIL][SGE_MAX_K];
        uint32_t ul_[SGE_MAX_TAIL][SGE_MAX_K];
        uint32_t un_[SGE_MAX_TAIL];
        for (uint32_t q = 0; q < nu; ++q) {
            const uint32_t u = i + 1 + q;
            ub_[q] = level_bounds(P, W, u);
            un_[q] = 0;
            if (explore) {
                uint32_t lastp = 31 - __clz(P.parents[u]);
                up_[q][0] = version_ptr(P, W, c, lastp, u);
                ul_[q][0] = W.vlen[lastp][u];
                un_[q] = 1;
                if (STATS) c.alg_bytes += 4ull * ul_[q][0];
            } else {
                for (uint32_t msk = P.parents[u]; msk; msk &= msk - 1) {
                    uint32_t j = __ffs(msk) - 1;
                    nbr(c.g, W.m[j], up_[q][un_[q]], ul_[q][un_[q]]);
                    if (STATS) c.alg_bytes += 8ull + 4ull * ul_[q][un_[q]];
                    un_[q]++;
                }
            }
        }
        if (STATS) { c.set_ops += 1; c.alg_bytes += 4ull * blen; }
        uint32_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (uint32_t off = 0; off < blen; off += 32) {
            uint32_t idx = off + lane;
            bool ok = idx < blen;
            uint32_t x = ok ? bp[idx] : 0u;
            for (uint32_t l = 0; l < nl && ok; ++l) ok = contains(lp[l], ll[l], x);
            if (ok) ok = !excluded(P, W, i, x);
            if (ok) {
                uint32_t fm = 0;
                for (uint32_t q = 0; q < nu; ++q) {
                    const uint32_t u = i + 1 + q;
                    bool f = (!ub_[q].has_lo || x > ub_[q].lo) && (!ub_[q].has_hi || x < ub_[q].hi);
                    for (uint32_t l = 0; l < un_[q] && f; ++l) f = contains(up_[q][l], ul_[q][l], x);
                    if (f) f = !excluded(P, W, u, x);
                    fm |= (uint32_t)f << q;
                }
#pragma unroll
                for (uint32_t s = 0; s < 8; ++s) cnt[s] += ((fm & s) == s) ? 1u : 0u;
            }
        }
        const uint32_t nsub = 1u << nu;
#pragma unroll
        for (uint32_t s = 0; s < 8; ++s) {
            uint32_t tot = __reduce_add_sync(FULL_MASK, cnt[s]);
            if (s < nsub && lane == 0) W.S[(1u << t) | (s << (t + 1))] = tot;
        }
    }
    __syncwarp();
    unsigned long long r;
    if (P.tail_mode == SGE_TAIL_SINGLE) {
        r = W.S[1];
    } else if (P.tail_mode == SGE_TAIL_CHOOSE) {
        r = binom_exact(W.S[1], T);
    } else {
        r = 0;
        for (uint32_t p = 0; p < P.nparts; ++p) {
            unsigned long long term = (unsigned long long)(long long)P.part_coef[p];
            for (uint32_t bk = 0; bk < P.part_nblocks[p]; ++bk) term *= W.S[P.part_block[p][bk]];
            r += term;
        }
    }
    __syncwarp();
    return r;
}

// One root edge: DFS over levels 2..ne-1, tail count at the leaves.
template <bool STATS>
__device__ unsigned long long run_root(const DevPlan &P, WarpState &W, Ctx<STATS> &c, uint32_t u, uint32_t v) {
    const uint32_t lane = lane_id();
    const bool explore = P.join_style == SGE_JOIN_EXPLORATION;
    __syncwarp();
    if (lane == 0) { W.m[0] = u; W.m[1] = v; }
    __syncwarp();
    if (explore) {
        if (!explore_update(P, W, c, 0)) return 0;
        if (!explore_update(P, W, c, 1)) return 0;
    }
    const uint32_t ne = P.ne;
    if (ne == 2) return tail_count(P, W, c);
    unsigned long long acc = 0;
    uint32_t lv = 2;
    if (explore) explore_level(P, W, c, lv);
    else if (!build_level_wcoj(P, W, c, lv)) return 0;
    __syncwarp();
    if (lane == 0) W.pos[lv] = 0;
    __syncwarp();
    while (true) {
        uint32_t pos = W.pos[lv];
        if (pos >= W.cnt[lv]) {
            if (lv == 2) break;
            --lv;
            continue;
        }
        uint32_t x = W.list[lv][pos];
        __syncwarp();
        if (lane == 0) W.pos[lv] = pos + 1;
        __syncwarp();
        if (excluded(P, W, lv, x)) continue;
        __syncwarp();
        if (lane == 0) W.m[lv] = x;
        __syncwarp();
        if (STATS) c.partial += 1;
        if (explore && !explore_update(P, W, c, lv)) continue;
        if (lv + 1 == ne) {
            acc += tail_count(P, W, c);
            continue;
        }
        ++lv;
        if (explore) explore_level(P, W, c, lv);
        else if (!build_level_wcoj(P, W, c, lv)) return 0;
        __syncwarp();
        if (lane == 0) W.pos[lv] = 0;
        __syncwarp();
    }
    return acc;
}

template <bool STATS>
__global__ void __launch_bounds__(256) count_kernel(DevGraph g, const DevPlan *__restrict__ plans, uint32_t nplans,
                                                    unsigned long long total_tasks, unsigned long long *queue,
                                                    unsigned long long *counts, uint32_t *scratch, uint32_t cap,
                                                    uint32_t bufs_per_warp, uint32_t chunk,
                                                    unsigned long long deadline_ns, uint32_t *flags,
                                                    DevStats *stats) {
    extern __shared__ unsigned char smem_raw[];
    const uint32_t lane = lane_id();
    const uint32_t wib = threadIdx.x >> 5;
    WarpState &W = reinterpret_cast<WarpState *>(smem_raw)[wib];
    __shared__ DevPlan Psh[8];
    DevPlan &P = Psh[wib];
    const size_t gwarp = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    Ctx<STATS> c;
    c.g = g;
    c.buf = scratch + gwarp * (size_t)bufs_per_warp * cap;
    c.cap = cap;
    c.flags = flags;
    c.set_ops = c.alg_bytes = c.partial = 0;
    unsigned long long roots = 0;
    unsigned long long tstart = 0;
    if (lane == 0) tstart = globaltimer_ns();
    tstart = __shfl_sync(FULL_MASK, tstart, 0);
    int cur = -1;
    unsigned long long acc = 0;
    while (true) {
        unsigned long long t0 = 0;
        if (lane == 0) t0 = atomicAdd(queue, (unsigned long long)chunk);
        t0 = __shfl_sync(FULL_MASK, t0, 0);
        if (t0 >= total_tasks) break;
        if (deadline_ns) {
            unsigned long long now = 0;
            if (lane == 0) now = globaltimer_ns();
            now = __shfl_sync(FULL_MASK, now, 0);
            if (now - tstart > deadline_ns) {
                if (lane == 0) atomicOr(flags, FLAG_TIMEOUT);
                break;
            }
        }
        if (*(volatile uint32_t *)flags & FLAG_OVERFLOW) break;
        unsigned long long t1 = min(t0 + chunk, total_tasks);
        for (unsigned long long t = t0; t < t1; ++t) {
            // locate the plan owning task t (plans are sorted by task_begin)
            if (cur < 0 || t < P.task_begin || t >= P.task_begin + P.ntasks) {
                if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc);
                acc = 0;
                int lo = 0, hi = (int)nplans - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (plans[mid].task_begin <= t) lo = mid; else hi = mid - 1;
                }
                cur = lo;
                __syncwarp();
                const uint32_t *src = reinterpret_cast<const uint32_t *>(plans + cur);
                uint32_t *dst = reinterpret_cast<uint32_t *>(&P);
                for (uint32_t w = lane; w < sizeof(DevPlan) / 4; w += 32) dst[w] = src[w];
                __syncwarp();
            }
            unsigned long long lt = P.root_offset + (t - P.task_begin) * P.root_stride;
            uint2 e;
            if (P.root_kind == SGE_ROOT_ANY) {
                e = g.edges[lt >> 1];
                if (lt & 1) { uint32_t tmp = e.x; e.x = e.y; e.y = tmp; }
            } else {
                e = g.edges[lt];
                if (P.root_kind == SGE_ROOT_DESC) { uint32_t tmp = e.x; e.x = e.y; e.y = tmp; }
            }
            acc += run_root<STATS>(P, W, c, e.x, e.y);
            ++roots;
        }
    }
    if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc);
    if (STATS && lane == 0) {
        atomicAdd(&stats->set_ops, c.set_ops);
        atomicAdd(&stats->alg_bytes, c.alg_bytes);
        atomicAdd(&stats->partial, c.partial);
        atomicAdd(&stats->roots, roots);
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
};

struct sge_plan {
    sge_plan_blob blob;
    DevPlan dp;
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
        d.parents[i] = b.parents[i];
        d.lower[i] = b.lower[i];
        d.upper[i] = b.upper[i];
        d.check[i] = b.check[i];
        d.rest[i] = b.rest[i];
        d.base[i] = b.base[i];
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
        d.part_coef[p] = b.part_coef[p];
        d.part_nblocks[p] = b.part_nblocks[p];
        for (uint32_t x = 0; x < SGE_MAX_TAIL; ++x) d.part_block[p][x] = b.part_block[p][x];
    }
    uint32_t nb = 0;
    if (b.join_style == SGE_JOIN_EXPLORATION) {
        for (uint32_t i = 2; i < b.k; ++i) {
            uint32_t par = b.parents[i];
            bool first = true;
            for (uint32_t msk = par; msk; msk &= msk - 1) {
                uint32_t j = (uint32_t)__builtin_ctz(msk);
                d.after[j] |= 1u << i;
                if (first) { d.slot[j][i] = -1; first = false; }
                else d.slot[j][i] = (int8_t)nb++;
            }
        }
    } else {
        nb = b.num_enum;  // stored levels use buffer index = level
    }
    d.nbufs = std::max<uint32_t>(nb, 1);
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

// Host validation: sorted, in range, no self-loops, no duplicates; symmetric
// (full check with threads).
sge_status validate_csr(const uint32_t *off, const uint32_t *nbrs, uint32_t n, uint64_t nnz) {
    if (off[0] != 0 || off[n] != nnz) return fail(SGE_BAD_INPUT, "offsets[0] must be 0 and offsets[n] = %llu", (unsigned long long)nnz);
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::atomic<int> bad{0};
    std::atomic<uint32_t> bad_v{0};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            for (uint64_t v = t; v < n && !bad.load(std::memory_order_relaxed); v += nt) {
                uint32_t a = off[v], b = off[v + 1];
                if (b < a || b > nnz) { bad = 1; bad_v = (uint32_t)v; return; }
                for (uint32_t e = a; e < b; ++e) {
                    uint32_t w = nbrs[e];
                    if (w >= n || w == v || (e > a && nbrs[e - 1] >= w)) { bad = 2; bad_v = (uint32_t)v; return; }
                    // symmetry: v must appear in N(w)
                    const uint32_t *p = nbrs + off[w];
                    const uint32_t *q = nbrs + off[w + 1];
                    if (off[w + 1] < off[w] || off[w + 1] > nnz) { bad = 1; bad_v = w; return; }
                    if (!std::binary_search(p, q, (uint32_t)v)) { bad = 3; bad_v = (uint32_t)v; return; }
                }
            }
        });
    for (auto &x : th) x.join();
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

extern "C" {

const char *sge_version(void) { return "sge 0.1 (sm_103a, ABI 1)"; }

int sge_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

sge_status sge_graph_create(const uint32_t *offsets, const uint32_t *nbrs, uint32_t n, uint64_t nnz, int device,
                            sge_graph **out) {
    if (!offsets || (!nbrs && nnz) || !out) return fail(SGE_BAD_INPUT, "sge_graph_create: null argument");
    if (nnz % 2) return fail(SGE_BAD_INPUT, "odd number of directed edges (%llu)", (unsigned long long)nnz);
    if (nnz >= (1ull << 32)) return fail(SGE_BAD_INPUT, "%llu directed edges exceed the uint32 EdgeID range", (unsigned long long)nnz);
    sge_status st = validate_csr(offsets, nbrs, n, nnz);
    if (st != SGE_OK) return st;
    int ndev = sge_device_count();
    if (ndev == 0) return fail(SGE_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(SGE_BAD_INPUT, "device %d out of range (%d visible)", device, ndev);
    CUDA_TRY(cudaSetDevice(device));
    sge_graph *g = new sge_graph();
    g->device = device;
    g->n = n;
    g->nnz = nnz;
    g->m = nnz / 2;
    cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
    // root edge list (u<v) and degree moments
    std::vector<uint2> edges;
    edges.reserve(g->m);
    for (uint32_t v = 0; v < n; ++v) {
        uint32_t d = offsets[v + 1] - offsets[v];
        g->max_deg = std::max(g->max_deg, d);
        for (uint32_t e = offsets[v]; e < offsets[v + 1]; ++e)
            if (nbrs[e] > v) edges.push_back(make_uint2(v, nbrs[e]));
    }
    sge_graph_stats_compute(offsets, nbrs, n, &g->stats);
    auto cleanup = [&](sge_status s) { sge_graph_destroy(g); return s; };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&g->ev0)) != cudaSuccess || (e = cudaEventCreate(&g->ev1)) != cudaSuccess)
        return cleanup(fail(SGE_CUDA_ERROR, "stream/event creation: %s", cudaGetErrorString(e)));
    if ((e = cudaMalloc(&g->d_off, sizeof(uint32_t) * ((size_t)n + 1))) != cudaSuccess ||
        (e = cudaMalloc(&g->d_adj, sizeof(uint32_t) * std::max<uint64_t>(nnz, 1))) != cudaSuccess ||
        (e = cudaMalloc(&g->d_edges, sizeof(uint2) * std::max<uint64_t>(g->m, 1))) != cudaSuccess)
        return cleanup(fail(SGE_OOM, "device allocation of the graph failed: %s", cudaGetErrorString(e)));
    if ((e = cudaMemcpyAsync(g->d_off, offsets, sizeof(uint32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, g->stream)) != cudaSuccess ||
        (nnz && (e = cudaMemcpyAsync(g->d_adj, nbrs, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, g->stream)) != cudaSuccess) ||
        (g->m && (e = cudaMemcpyAsync(g->d_edges, edges.data(), sizeof(uint2) * g->m, cudaMemcpyHostToDevice, g->stream)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(g->stream)) != cudaSuccess)
        return cleanup(fail(SGE_CUDA_ERROR, "graph upload failed: %s", cudaGetErrorString(e)));
    *out = g;
    return SGE_OK;
}

sge_status sge_graph_destroy(sge_graph *g) {
    if (!g) return SGE_OK;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    cudaFree(g->d_off);
    cudaFree(g->d_adj);
    cudaFree(g->d_edges);
    cudaFree(g->d_scratch);
    cudaFree(g->d_batch);
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
    info->device_bytes = 4ull * (g->n + 1) + 4ull * g->nnz + 8ull * g->m;
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

sge_status sge_count(sge_graph *g, const sge_plan *const *plans, uint32_t nplans, const sge_count_opts *opts,
                     uint64_t *counts, uint64_t *instances, sge_stats *stats) {
    auto t_start = std::chrono::steady_clock::now();
    if (!g || (!plans && nplans) || (!counts && nplans)) return fail(SGE_BAD_INPUT, "sge_count: null argument");
    if (nplans == 0) return SGE_OK;
    sge_count_opts o{};
    if (opts) o = *opts;
    CUDA_TRY(cudaSetDevice(g->device));
    std::vector<DevPlan> dps(nplans);
    unsigned long long total = 0;
    uint32_t nbufs = 1;
    for (uint32_t i = 0; i < nplans; ++i) {
        if (!plans[i]) return fail(SGE_BAD_INPUT, "plan %u is null", i);
        dps[i] = plans[i]->dp;
        dps[i].task_begin = total;
        const unsigned long long all = (dps[i].root_kind == SGE_ROOT_ANY) ? 2ull * g->m : g->m;
        const unsigned long long stride = o.root_stride > 1 ? o.root_stride : 1ull;
        const unsigned long long offs = o.root_offset;
        if (stride > 1 && offs >= stride) return fail(SGE_BAD_INPUT, "root_offset %llu >= root_stride %llu", offs, stride);
        dps[i].root_stride = stride;
        dps[i].root_offset = stride > 1 ? offs : 0;
        dps[i].ntasks = all > dps[i].root_offset ? (all - dps[i].root_offset + stride - 1) / stride : 0;
        total += dps[i].ntasks;
        nbufs = std::max(nbufs, dps[i].nbufs);
        if (dps[i].k > SGE_MAX_K) return fail(SGE_UNSUPPORTED, "plan %u has k=%u", i, dps[i].k);
    }
    const uint32_t wpb = o.warps_per_block ? std::min<uint32_t>(o.warps_per_block, 8) : 8;
    const uint32_t threads = wpb * 32;
    const size_t smem = sizeof(WarpState) * wpb;
    const bool want_stats = o.collect_counters != 0;
    int bps = 0;
    if (want_stats) CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, count_kernel<true>, threads, smem));
    else CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, count_kernel<false>, threads, smem));
    if (o.blocks_per_sm) bps = std::min<int>(bps, (int)o.blocks_per_sm);
    bps = std::max(bps, 1);
    uint32_t cap = o.max_level_capacity ? o.max_level_capacity : std::max<uint32_t>(g->max_deg, 1);
    cap = (cap + 31) & ~31u;
    // fit the scratch into a quarter of free memory by trimming resident blocks
    size_t free_b = 0, tot_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &tot_b));
    size_t per_block = (size_t)wpb * nbufs * cap * sizeof(uint32_t);
    size_t blocks = (size_t)g->num_sms * bps;
    size_t budget = free_b / 4 + g->scratch_bytes;
    while (blocks > (size_t)g->num_sms && blocks * per_block > budget) blocks -= g->num_sms;
    if (blocks * per_block > budget) blocks = std::max<size_t>(1, budget / std::max<size_t>(per_block, 1));
    sge_status st = ensure_scratch(g, blocks * per_block);
    if (st != SGE_OK) return st;
    // batch buffer: plans | counts | queue | flags | stats
    size_t off_plans = 0;
    size_t off_counts = (sizeof(DevPlan) * nplans + 255) & ~(size_t)255;
    size_t off_queue = off_counts + ((8 * (size_t)nplans + 255) & ~(size_t)255);
    size_t off_flags = off_queue + 256;
    size_t off_stats = off_flags + 256;
    size_t bytes = off_stats + 256;
    st = ensure_batch(g, bytes);
    if (st != SGE_OK) return st;
    unsigned char *B = g->d_batch;
    CUDA_TRY(cudaMemcpyAsync(B + off_plans, dps.data(), sizeof(DevPlan) * nplans, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemsetAsync(B + off_counts, 0, bytes - off_counts, g->stream));
    uint32_t chunk = o.chunk;
    if (!chunk) {
        unsigned long long warps = blocks * wpb;
        chunk = (uint32_t)std::max<unsigned long long>(1, std::min<unsigned long long>(8, total / (warps * 64 + 1)));
    }
    unsigned long long deadline = 0;  // ns after each warp's start; 0 = none
    DevGraph dg{g->d_off, g->d_adj, g->d_edges, g->n, g->m};
    CUDA_TRY(cudaEventRecord(g->ev0, g->stream));
    const DevPlan *dplans = reinterpret_cast<const DevPlan *>(B + off_plans);
    unsigned long long *dcounts = reinterpret_cast<unsigned long long *>(B + off_counts);
    unsigned long long *dqueue = reinterpret_cast<unsigned long long *>(B + off_queue);
    uint32_t *dflags = reinterpret_cast<uint32_t *>(B + off_flags);
    DevStats *dstats = reinterpret_cast<DevStats *>(B + off_stats);
    if (o.time_budget_s > 0) deadline = std::max<unsigned long long>(1, (unsigned long long)(o.time_budget_s * 1e9));
    if (want_stats)
        count_kernel<true><<<(unsigned)blocks, threads, smem, g->stream>>>(dg, dplans, nplans, total, dqueue, dcounts,
                                                                         g->d_scratch, cap, nbufs, chunk, deadline,
                                                                         dflags, dstats);
    else
        count_kernel<false><<<(unsigned)blocks, threads, smem, g->stream>>>(dg, dplans, nplans, total, dqueue, dcounts,
                                                                          g->d_scratch, cap, nbufs, chunk, deadline,
                                                                          dflags, dstats);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(g->ev1, g->stream));
    std::vector<unsigned long long> hc(nplans);
    uint32_t hflags = 0;
    DevStats hs{};
    CUDA_TRY(cudaMemcpyAsync(hc.data(), dcounts, 8 * nplans, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaMemcpyAsync(&hflags, dflags, 4, cudaMemcpyDeviceToHost, g->stream));
    if (want_stats) CUDA_TRY(cudaMemcpyAsync(&hs, dstats, sizeof hs, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    for (uint32_t i = 0; i < nplans; ++i) {
        uint64_t inst = hc[i];
        counts[i] = inst * plans[i]->blob.count_multiplier;
        if (instances) instances[i] = inst;
    }
    if (stats) {
        stats->kernel_ms = ms;
        stats->root_tasks = hs.roots;
        stats->set_ops = hs.set_ops;
        stats->alg_bytes = hs.alg_bytes;
        stats->partial_matches = hs.partial;
        stats->gpu_launches = 1;
        stats->status_flags = hflags;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    if (hflags & FLAG_OVERFLOW) return fail(SGE_STACK_OVERFLOW, "a candidate list exceeded the per-level capacity %u", cap);
    if (hflags & FLAG_TIMEOUT) return fail(SGE_TIMEOUT, "time budget of %.3f s exceeded; counts are partial", o.time_budget_s);
    return SGE_OK;
}

sge_status sge_count_host(const uint32_t *offsets, const uint32_t *nbrs, uint32_t n, uint64_t nnz,
                          const sge_plan_blob *blobs, uint32_t nplans, const sge_count_opts *opts, uint64_t *counts,
                          sge_stats *stats) {
    if (!blobs && nplans) return fail(SGE_BAD_INPUT, "sge_count_host: null plans");
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
    extern __shared__ unsigned char smem_raw[];
    const uint32_t lane = lane_id();
    const uint32_t wib = threadIdx.x >> 5;
    WarpState &W = reinterpret_cast<WarpState *>(smem_raw)[wib];
    __shared__ DevPlan Psh[8];
    DevPlan &P = Psh[wib];
    const size_t gwarp = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    Ctx<false> c;
    c.g = g;
    c.buf = lists + gwarp * (size_t)bufs_per_warp * cap;
    c.cap = cap;
    c.flags = flags;
    c.set_ops = c.alg_bytes = c.partial = 0;
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
                if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc * P.task_begin);
                acc = 0;
                cur = pi;
                __syncwarp();
                const uint32_t *src = reinterpret_cast<const uint32_t *>(plans + cur);
                uint32_t *dst = reinterpret_cast<uint32_t *>(&P);
                for (uint32_t w = lane; w < sizeof(DevPlan) / 4; w += 32) dst[w] = src[w];
                __syncwarp();
            }
            const uint32_t e = (uint32_t)(t - (unsigned long long)pi * nnz);
            const uint32_t u = ub(g.off, g.n + 1, e) - 1;  // source of directed edge e
            const uint32_t v = g.adj[e];
            if (P.root_kind == SGE_ROOT_ASC && !(u < v)) continue;
            if (P.root_kind == SGE_ROOT_DESC && !(u > v)) continue;
            acc += run_root<false>(P, W, c, u, v);
        }
    }
    // P.task_begin carries the plan's count multiplier in this variant
    if (cur >= 0 && lane == 0 && acc) atomicAdd(counts + cur, acc * P.task_begin);
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
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return fail(SGE_CUDA_ERROR, "cudaGetSymbolAddress(static scratch) on device %d: %s", dev,
                            cudaGetErrorString(e));
            g_noalloc_ptr[dev] = p;
        }
        base = g_noalloc_ptr[dev];
    }
    // plans: validate, convert, copy into the array's plan table
    uint32_t nbufs = 1;
    for (uint32_t i = 0; i < nplans; ++i) {
        sge_status st = sge_plan_validate(&plans[i]);
        if (st != SGE_OK) return st;
        DevPlan dp;
        to_devplan(plans[i], dp);
        dp.task_begin = plans[i].count_multiplier;  // multiplier, applied at the atomic flush
        dp.ntasks = nnz;
        dp.root_stride = 1;
        dp.root_offset = 0;
        nbufs = std::max(nbufs, dp.nbufs);
        CUDA_TRY(cudaMemcpyAsync(static_cast<unsigned char *>(base) + NOALLOC_HDR + i * sizeof(DevPlan), &dp,
                                 sizeof(DevPlan), cudaMemcpyHostToDevice, stream));
    }
    const uint32_t cap = (std::max<uint32_t>(max_degree, 1) + 31) & ~31u;
    const size_t per_warp = (size_t)nbufs * cap * sizeof(uint32_t);
    const size_t avail = SGE_NOALLOC_SCRATCH_BYTES - NOALLOC_LISTS;
    const uint32_t wpb = 8, threads = wpb * 32;
    const size_t smem = sizeof(WarpState) * wpb;
    size_t max_blocks = avail / (per_warp * wpb);
    if (max_blocks == 0)
        return fail(SGE_UNSUPPORTED,
                    "sge_count_noalloc: %u levels x max degree %u need %zu bytes per 8-warp block; the static "
                    "scratch holds %zu", nbufs, max_degree, per_warp * wpb, avail);
    int bps = 0, sms = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, count_kernel_noalloc, threads, smem));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t blocks = std::max<size_t>(1, std::min<size_t>(max_blocks, (size_t)std::max(bps, 1) * sms));
    // clear what must start at zero: queue, flags, and the caller's counts
    CUDA_TRY(cudaMemsetAsync(base, 0, NOALLOC_HDR, stream));
    CUDA_TRY(cudaMemsetAsync(d_counts, 0, sizeof(uint64_t) * nplans, stream));
    DevGraph dg{d_offsets, d_nbrs, nullptr, n, nnz / 2};
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
