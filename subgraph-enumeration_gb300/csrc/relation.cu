// Bag relations on the device: canonical instance tuples, a stable LSD radix
// sort of uint32 tuples, and trie levels built from the sorted tuples.
//
// The reference materialises a bag as vector<vector<VertexID>> tuples
// (nodeJoin, matching/join.cpp:309-421), std::sorts them and groups them
// column by column into nested TrieLevel{values, children}
// (buildTrie, join.cpp:1713-1717; TrieLevel::buildTrieFromSortedMatchesBatch,
// relation/relation.cpp:340-379).  Here tuples are rows of a device array;
// the sort is an LSD radix sort (8-bit digits, last column first, stable
// scatter by warp match + per-warp digit counts), and each trie level is a
// flat array of values plus child offsets into the next level (CSR form of
// the same tree), built with boundary flags and prefix sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "device_util.hpp"

using namespace sge;

namespace {

#define CUDA_TRY(expr)                                                                               \
    do {                                                                                             \
        cudaError_t _e = (expr);                                                                     \
        if (_e != cudaSuccess)                                                                       \
            return fail(_e == cudaErrorMemoryAllocation ? SGE_OOM : SGE_CUDA_ERROR, "%s: %s", #expr, \
                        cudaGetErrorString(_e));                                                     \
    } while (0)

constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 4;  // per thread per tile: a tile is 1024 elements
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;
constexpr int MAX_ARITY = 16;

// ---- canonical form: the lexicographically smallest image of a tuple under
// the pattern's automorphisms (one representative per automorphism class) ----
__global__ void canon_kernel(uint32_t *t, unsigned long long n, uint32_t k, const uint8_t *__restrict__ perms,
                             uint32_t naut) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t *row = t + i * k;
    uint32_t best[MAX_ARITY], cur[MAX_ARITY];
    for (uint32_t j = 0; j < k; ++j) best[j] = row[j];
    for (uint32_t a = 0; a < naut; ++a) {
        const uint8_t *s = perms + (size_t)a * k;
        int cmp = 0;
        for (uint32_t j = 0; j < k; ++j) {
            cur[j] = row[s[j]];
            if (cmp == 0) cmp = cur[j] < best[j] ? -1 : (cur[j] > best[j] ? 1 : 0);
        }
        if (cmp < 0)
            for (uint32_t j = 0; j < k; ++j) best[j] = cur[j];
    }
    for (uint32_t j = 0; j < k; ++j) row[j] = best[j];
}

// ---- radix sort of a permutation by one 8-bit digit of one column ----
__device__ __forceinline__ uint32_t digit_of(const uint32_t *t, uint32_t arity, uint32_t col, uint32_t shift,
                                             uint32_t idx) {
    return (t[(size_t)idx * arity + col] >> shift) & 0xFFu;
}

// per-tile digit histogram, stored digit-major: hist[d * ntiles + tile]
__global__ void hist_kernel(const uint32_t *t, const uint32_t *perm, unsigned long long n, uint32_t arity,
                            uint32_t col, uint32_t shift, uint32_t *hist, uint32_t ntiles) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const unsigned long long base = (unsigned long long)blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; ++r) {
        const unsigned long long i = base + r * SORT_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[digit_of(t, arity, col, shift, perm[i])], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// exclusive scan in place over m entries, single block (chunked sequentially)
__global__ void scan_single_block(uint32_t *a, unsigned long long m) {
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (unsigned long long base = 0; base < m; base += 1024) {
        const unsigned long long i = base + threadIdx.x;
        const uint32_t v = i < m ? a[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            uint32_t x = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0u;
            __syncthreads();
            s[threadIdx.x] += x;
            __syncthreads();
        }
        if (i < m) a[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
}

// stable scatter: rank = tile offset of the digit + earlier passes over this
// tile + earlier warps of this pass + earlier lanes with the same digit
__global__ void scatter_kernel(const uint32_t *t, const uint32_t *perm_in, uint32_t *perm_out, unsigned long long n,
                               uint32_t arity, uint32_t col, uint32_t shift, const uint32_t *offs, uint32_t ntiles) {
    __shared__ uint32_t base_off[256];
    __shared__ uint32_t warp_cnt[SORT_THREADS / 32][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = threadIdx.x; d < 256; d += blockDim.x) base_off[d] = offs[(size_t)d * ntiles + blockIdx.x];
    const unsigned long long tile = (unsigned long long)blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ITEMS; ++r) {
        for (int d = threadIdx.x; d < 256; d += blockDim.x)
            for (int w = 0; w < SORT_THREADS / 32; ++w) warp_cnt[w][d] = 0;
        __syncthreads();
        const unsigned long long i = tile + r * SORT_THREADS + threadIdx.x;
        const bool valid = i < n;
        const uint32_t idx = valid ? perm_in[i] : 0u;
        const uint32_t d = valid ? digit_of(t, arity, col, shift, idx) : 256u + lane;  // invalid lanes: unique keys
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        // exclusive prefix over warps per digit; add into base_off after use
        uint32_t my_prefix = 0;
        if (valid)
            for (int w = 0; w < warp; ++w) my_prefix += warp_cnt[w][d];
        if (valid) perm_out[base_off[d] + my_prefix + rank] = idx;
        __syncthreads();
        for (int dd = threadIdx.x; dd < 256; dd += blockDim.x) {
            uint32_t tot = 0;
            for (int w = 0; w < SORT_THREADS / 32; ++w) tot += warp_cnt[w][dd];
            base_off[dd] += tot;
        }
        __syncthreads();
    }
}

__global__ void iota_kernel(uint32_t *p, unsigned long long n) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}

__global__ void gather_rows(const uint32_t *in, const uint32_t *perm, uint32_t *out, unsigned long long n,
                            uint32_t arity) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t *src = in + (size_t)perm[i] * arity;
    uint32_t *dst = out + i * arity;
    for (uint32_t j = 0; j < arity; ++j) dst[j] = src[j];
}

// ---- trie levels from sorted tuples ----
// flags[i] = 1 when row i starts a new node of the level (its prefix of
// length lvl+1 differs from row i-1's)
__global__ void boundary_kernel(const uint32_t *t, unsigned long long n, uint32_t arity, uint32_t lvl,
                                uint32_t *flags) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t f = i == 0;
    if (!f)
        for (uint32_t j = 0; j <= lvl && !f; ++j) f = t[i * arity + j] != t[(i - 1) * arity + j];
    flags[i] = f;
}

__global__ void level_values(const uint32_t *t, unsigned long long n, uint32_t arity, uint32_t lvl,
                             const uint32_t *flags, const uint32_t *pos, uint32_t *values) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n && flags[i]) values[pos[i]] = t[i * arity + lvl];
}

// child offset of node p at level lvl = position of its first row's node at lvl+1
__global__ void level_children(unsigned long long n, const uint32_t *flags, const uint32_t *pos,
                               const uint32_t *pos_next, unsigned long long *child) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n && flags[i]) child[pos[i]] = pos_next[i];
}

inline unsigned grid_for(unsigned long long n, unsigned b = 256) { return (unsigned)((n + b - 1) / b); }

// exclusive scan of n uint32 (device), two levels: per-1024 block sums then a
// single-block scan of the sums, then a fix-up.
__global__ void block_scan(const uint32_t *in, uint32_t *out, unsigned long long n, uint32_t *sums) {
    __shared__ uint32_t s[1024];
    const unsigned long long i = blockIdx.x * 1024ull + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t x = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0u;
        __syncthreads();
        s[threadIdx.x] += x;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == 1023) sums[blockIdx.x] = s[1023];
}
__global__ void add_block_offsets(uint32_t *out, unsigned long long n, const uint32_t *sums) {
    const unsigned long long i = blockIdx.x * 1024ull + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}

sge_status exclusive_scan(const uint32_t *in, uint32_t *out, unsigned long long n, uint32_t *tmp_sums,
                          cudaStream_t s) {
    const unsigned nb = (unsigned)((n + 1023) / 1024);
    block_scan<<<nb, 1024, 0, s>>>(in, out, n, tmp_sums);
    scan_single_block<<<1, 1024, 0, s>>>(tmp_sums, nb);
    add_block_offsets<<<nb, 1024, 0, s>>>(out, n, tmp_sums);
    CUDA_TRY(cudaGetLastError());
    return SGE_OK;
}

}  // namespace

sge_status sge::device_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, cudaStream_t s) {
    if (n == 0) return SGE_OK;
    uint32_t *sums = nullptr;
    CUDA_TRY(cudaMalloc(&sums, sizeof(uint32_t) * ((n + 1023) / 1024)));
    sge_status st = exclusive_scan(in, out, n, sums, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFree(sums);
    if (st != SGE_OK) return st;
    if (e != cudaSuccess) return fail(SGE_CUDA_ERROR, "device_exclusive_scan: %s", cudaGetErrorString(e));
    return SGE_OK;
}

extern "C" {

sge_status sge_canonicalize(uint32_t *d_tuples, uint64_t n, uint32_t k, const uint8_t *perms, uint32_t naut) {
    if ((!d_tuples && n) || !perms || k == 0 || k > MAX_ARITY || naut == 0)
        return fail(SGE_BAD_INPUT, "sge_canonicalize: bad argument");
    if (n == 0) return SGE_OK;
    uint8_t *dp = nullptr;
    CUDA_TRY(cudaMalloc(&dp, (size_t)naut * k));
    CUDA_TRY(cudaMemcpy(dp, perms, (size_t)naut * k, cudaMemcpyHostToDevice));
    canon_kernel<<<grid_for(n), 256>>>(d_tuples, n, k, dp, naut);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(dp);
    if (e != cudaSuccess) return fail(SGE_CUDA_ERROR, "canonicalize: %s", cudaGetErrorString(e));
    return SGE_OK;
}

// Lexicographic sort of n rows of `arity` uint32 (device, in place).
sge_status sge_sort_tuples(uint32_t *d_tuples, uint64_t n, uint32_t arity) {
    if ((!d_tuples && n) || arity == 0 || arity > MAX_ARITY) return fail(SGE_BAD_INPUT, "sge_sort_tuples: bad argument");
    if (n <= 1) return SGE_OK;
    if (n >= (1ull << 32)) return fail(SGE_UNSUPPORTED, "sge_sort_tuples: more than 2^32 rows");
    const uint32_t ntiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
    uint32_t *pa = nullptr, *pb = nullptr, *hist = nullptr, *rows = nullptr, *sums = nullptr;
    auto cleanup = [&]() { cudaFree(pa); cudaFree(pb); cudaFree(hist); cudaFree(rows); cudaFree(sums); };
    cudaError_t e;
    const unsigned long long nh = 256ull * ntiles;  // digit-major histogram entries
    if ((e = cudaMalloc(&pa, n * 4)) != cudaSuccess || (e = cudaMalloc(&pb, n * 4)) != cudaSuccess ||
        (e = cudaMalloc(&hist, nh * 4)) != cudaSuccess ||
        (e = cudaMalloc(&sums, ((nh + 1023) / 1024) * 4)) != cudaSuccess ||
        (e = cudaMalloc(&rows, n * arity * 4ull)) != cudaSuccess) {
        cleanup();
        return fail(SGE_OOM, "sge_sort_tuples: %s", cudaGetErrorString(e));
    }
    iota_kernel<<<grid_for(n), 256>>>(pa, n);
    for (int col = (int)arity - 1; col >= 0; --col)
        for (uint32_t shift = 0; shift < 32; shift += 8) {
            hist_kernel<<<ntiles, SORT_THREADS>>>(d_tuples, pa, n, arity, (uint32_t)col, shift, hist, ntiles);
            // offsets: exclusive scan of the histogram, in place (per-1024 block scans, then
            // one block over the block sums)
            const sge_status sst = exclusive_scan(hist, hist, nh, sums, 0);
            if (sst != SGE_OK) {
                cleanup();
                return sst;
            }
            scatter_kernel<<<ntiles, SORT_THREADS>>>(d_tuples, pa, pb, n, arity, (uint32_t)col, shift, hist, ntiles);
            std::swap(pa, pb);
        }
    gather_rows<<<grid_for(n), 256>>>(d_tuples, pa, rows, n, arity);
    e = cudaMemcpy(d_tuples, rows, n * arity * 4ull, cudaMemcpyDeviceToDevice);
    cudaError_t e2 = cudaDeviceSynchronize();
    cleanup();
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(SGE_CUDA_ERROR, "sge_sort_tuples: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return SGE_OK;
}

// Trie levels of sorted tuples: level l has len[l] values (device array
// values[l]); node p of level l < arity-1 owns children
// [child[l][p], child[l][p+1]) of level l+1 (child[l] has len[l]+1 entries).
sge_status sge_trie_build(const uint32_t *d_sorted, uint64_t n, uint32_t arity, sge_trie *out) {
    if (!out || (!d_sorted && n) || arity == 0 || arity > SGE_TRIE_MAX_LEVELS)
        return fail(SGE_BAD_INPUT, "sge_trie_build: bad argument");
    memset(out, 0, sizeof *out);
    out->arity = arity;
    if (n == 0) return SGE_OK;
    if (n >= (1ull << 32)) return fail(SGE_UNSUPPORTED, "sge_trie_build: more than 2^32 rows");
    std::vector<uint32_t *> flags(arity, nullptr), pos(arity, nullptr);
    uint32_t *sums = nullptr;
    auto cleanup = [&]() {
        for (auto p : flags) cudaFree(p);
        for (auto p : pos) cudaFree(p);
        cudaFree(sums);
    };
    cudaError_t e = cudaMalloc(&sums, ((n + 1023) / 1024 + 1) * 4);
    for (uint32_t l = 0; l < arity && e == cudaSuccess; ++l) {
        if ((e = cudaMalloc(&flags[l], n * 4)) != cudaSuccess) break;
        e = cudaMalloc(&pos[l], n * 4);
    }
    if (e != cudaSuccess) { cleanup(); return fail(SGE_OOM, "sge_trie_build: %s", cudaGetErrorString(e)); }
    for (uint32_t l = 0; l < arity; ++l) {
        boundary_kernel<<<grid_for(n), 256>>>(d_sorted, n, arity, l, flags[l]);
        sge_status st = exclusive_scan(flags[l], pos[l], n, sums, 0);
        if (st != SGE_OK) { cleanup(); return st; }
        uint32_t last_pos = 0, last_flag = 0;
        cudaMemcpy(&last_pos, pos[l] + n - 1, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&last_flag, flags[l] + n - 1, 4, cudaMemcpyDeviceToHost);
        out->level_len[l] = (uint64_t)last_pos + last_flag;
        if ((e = cudaMalloc(&out->values[l], out->level_len[l] * 4)) != cudaSuccess) break;
        level_values<<<grid_for(n), 256>>>(d_sorted, n, arity, l, flags[l], pos[l], out->values[l]);
    }
    for (uint32_t l = 0; l + 1 < arity && e == cudaSuccess; ++l) {
        if ((e = cudaMalloc(&out->child[l], (out->level_len[l] + 1) * 8)) != cudaSuccess) break;
        level_children<<<grid_for(n), 256>>>(n, flags[l], pos[l], pos[l + 1], out->child[l]);
        const unsigned long long endv = out->level_len[l + 1];
        cudaMemcpy(out->child[l] + out->level_len[l], &endv, 8, cudaMemcpyHostToDevice);
    }
    cudaError_t e2 = cudaDeviceSynchronize();
    cleanup();
    if (e != cudaSuccess || e2 != cudaSuccess) {
        sge_trie_free(out);
        return fail(SGE_CUDA_ERROR, "sge_trie_build: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    return SGE_OK;
}

sge_status sge_trie_copy_level(const sge_trie *t, uint32_t level, uint32_t *values, unsigned long long *child) {
    if (!t || level >= t->arity || (!values && t->level_len[level])) return fail(SGE_BAD_INPUT, "sge_trie_copy_level: bad argument");
    const uint64_t n = t->level_len[level];
    if (n) CUDA_TRY(cudaMemcpy(values, t->values[level], n * 4, cudaMemcpyDeviceToHost));
    if (child && level + 1 < t->arity && t->child[level])
        CUDA_TRY(cudaMemcpy(child, t->child[level], (n + 1) * 8, cudaMemcpyDeviceToHost));
    return SGE_OK;
}

sge_status sge_trie_free(sge_trie *t) {
    if (!t) return SGE_OK;
    for (uint32_t l = 0; l < SGE_TRIE_MAX_LEVELS; ++l) {
        cudaFree(t->values[l]);
        cudaFree(t->child[l]);
        t->values[l] = nullptr;
        t->child[l] = nullptr;
    }
    return SGE_OK;
}

// The sorted instance set of a pattern (the embedding set -r writes; the
// reference never produces one): count, enumerate into an exactly sized
// device buffer, canonicalise under the automorphisms, sort, copy to host.
sge_status sge_match_set(sge_graph *g, const sge_plan *p, uint32_t k, uint32_t m, const uint32_t *edges,
                         uint32_t *host_out, uint64_t cap_rows, uint64_t *n_rows) {
    if (!g || !p || !n_rows || (!host_out && cap_rows)) return fail(SGE_BAD_INPUT, "sge_match_set: null argument");
    uint64_t counts = 0, inst = 0;
    const sge_plan *pp = p;
    sge_status st = sge_count(g, &pp, 1, nullptr, &counts, &inst, nullptr);
    if (st != SGE_OK) return st;
    *n_rows = inst;
    if (inst > cap_rows) return fail(SGE_OOM, "%llu instances exceed the %llu-row output", (unsigned long long)inst,
                                     (unsigned long long)cap_rows);
    if (inst == 0) return SGE_OK;
    uint32_t *d = nullptr;
    CUDA_TRY(cudaMalloc(&d, inst * k * 4ull));
    uint64_t n2 = 0;
    st = sge_enumerate(g, p, d, inst, &n2);
    if (st == SGE_OK && n2 != inst)
        st = fail(SGE_CUDA_ERROR, "enumeration produced %llu rows but the count is %llu", (unsigned long long)n2,
                  (unsigned long long)inst);
    std::vector<uint8_t> perms((size_t)4096 * k);
    uint32_t naut = 0;
    if (st == SGE_OK) st = sge_pattern_automorphisms(k, m, edges, perms.data(), 4096, &naut);
    if (st == SGE_OK) st = sge_canonicalize(d, inst, k, perms.data(), naut);
    if (st == SGE_OK) st = sge_sort_tuples(d, inst, k);
    if (st == SGE_OK && cudaMemcpy(host_out, d, inst * k * 4ull, cudaMemcpyDeviceToHost) != cudaSuccess)
        st = fail(SGE_CUDA_ERROR, "sge_match_set: copy-out failed");
    cudaFree(d);
    return st;
}

}  // extern "C"
