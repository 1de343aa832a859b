// Device graph ingest: the symmetric CSR the join reads, built on the GPU
// from an undirected edge list, and R-MAT data graphs generated on the GPU.
//
// The reference builds its CSR on the host: Graph::addDirectedEdges
// (relation/graph.cpp:143-173) inserts both directions of every edge and
// sorts each list; loadDataGraph (graph.cpp:255-419) reads text or BINGRPH.
// Here an edge list already in device memory becomes a CSR with one sort of
// (src, dst) rows, a duplicate/self-loop filter, an ordered compaction and
// one binary search per vertex for the offsets.  The R-MAT generator draws
// the same counter-based splitmix64 stream as the host generator
// (sge_gen_rmat), so a seed gives the same graph on either side.
#include <cuda_runtime.h>

#include <algorithm>
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

constexpr uint32_t NONE = 0xFFFFFFFFu;

inline unsigned grid_for(unsigned long long n, unsigned b = 256) { return (unsigned)((n + b - 1) / b); }

__device__ __forceinline__ uint64_t splitmix64_d(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Both directions of every edge as (src, dst) rows; self-loops become
// (NONE, NONE) rows, which sort last and are dropped.  An id >= n sets *bad.
__global__ void directed_rows(const uint32_t *edges, unsigned long long m, uint32_t n, uint32_t *rows,
                              uint32_t *bad) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t u = edges[2 * i], v = edges[2 * i + 1];
    uint32_t *r = rows + 4 * i;
    if (u >= n || v >= n) atomicOr(bad, 1u);
    if (u == v || u >= n || v >= n) {
        r[0] = r[1] = r[2] = r[3] = NONE;
        return;
    }
    r[0] = u;
    r[1] = v;
    r[2] = v;
    r[3] = u;
}

// keep[i] = row i is a real edge and differs from row i-1 (rows sorted)
__global__ void first_of_run(const uint32_t *rows, unsigned long long n, uint32_t *keep) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t a = rows[2 * i], b = rows[2 * i + 1];
    keep[i] = (a != NONE) && (i == 0 || a != rows[2 * i - 2] || b != rows[2 * i - 1]) ? 1u : 0u;
}

__global__ void compact_rows(const uint32_t *rows, unsigned long long n, const uint32_t *keep, const uint32_t *pos,
                             uint32_t *src, uint32_t *adj) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    src[pos[i]] = rows[2 * i];
    adj[pos[i]] = rows[2 * i + 1];
}

// off[v] = first position whose source is >= v (std::lower_bound)
__global__ void offsets_from_sources(const uint32_t *src, unsigned long long nnz, uint32_t n, uint32_t *off) {
    const unsigned long long v = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v > n) return;
    unsigned long long lo = 0, len = nnz;
    while (len > 0) {
        const unsigned long long half = len >> 1;
        if (src[lo + half] < (uint32_t)v) { lo += half + 1; len -= half + 1; }
        else len = half;
    }
    off[v] = (uint32_t)lo;
}

// One R-MAT draw per thread as a (u, v, draw index) row, u < v; a self-loop
// draw becomes (NONE, NONE, index).  Quadrant choices come two per 64-bit
// splitmix64 word, keyed by (seed, draw index, bit) exactly as on the host.
__global__ void rmat_rows(uint64_t seed, uint32_t scale, uint32_t ta, uint32_t tab, uint32_t tabc,
                          unsigned long long draws, uint32_t *rows) {
    const unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= draws) return;
    uint32_t u = 0, v = 0;
    uint64_t word = 0;
    for (uint32_t bit = 0; bit < scale; ++bit) {
        uint32_t r;
        if ((bit & 1u) == 0) {
            word = splitmix64_d(seed * 0x100000001B3ull + idx * 64 + bit);
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
    uint32_t *r = rows + 3 * idx;
    if (u == v) { r[0] = r[1] = NONE; }
    else { r[0] = min(u, v); r[1] = max(u, v); }
    r[2] = (uint32_t)idx;
}

// The first draw of every distinct edge (rows sorted by (u, v, index)) as an
// (index, u, v) row; *count receives the number of distinct edges.
__global__ void first_draws(const uint32_t *rows, unsigned long long n, uint32_t *out, unsigned long long *count) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t u = rows[3 * i], v = rows[3 * i + 1];
    if (u == NONE) return;
    if (i > 0 && rows[3 * i - 3] == u && rows[3 * i - 2] == v) return;
    const unsigned long long p = atomicAdd(count, 1ull);
    out[3 * p] = rows[3 * i + 2];
    out[3 * p + 1] = u;
    out[3 * p + 2] = v;
}

// (index, u, v) rows -> (u, v) edge pairs
__global__ void drop_index(const uint32_t *rows, unsigned long long n, uint32_t *edges) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    edges[2 * i] = rows[3 * i + 1];
    edges[2 * i + 1] = rows[3 * i + 2];
}

struct DevBuf {
    void *p = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    template <class T> T *as() { return static_cast<T *>(p); }
};

}  // namespace

extern "C" {

sge_status sge_graph_create_from_device_edges(const uint32_t *d_edges, uint64_t m, uint32_t num_vertices, int device,
                                              sge_graph **out) {
    if ((!d_edges && m) || !out) return fail(SGE_BAD_INPUT, "sge_graph_create_from_device_edges: null argument");
    if (2 * m >= (1ull << 32)) return fail(SGE_BAD_INPUT, "%llu edges exceed the uint32 EdgeID range", (unsigned long long)m);
    int ndev = sge_device_count();
    if (ndev == 0) return fail(SGE_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(SGE_BAD_INPUT, "device %d out of range (%d visible)", device, ndev);
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(device));
    const unsigned long long nd = 2 * m;  // directed rows
    DevBuf rows, keep, pos, src, bad;
    uint32_t *d_off = nullptr, *d_adj = nullptr;
    CUDA_TRY(cudaMalloc(&bad.p, 4));
    CUDA_TRY(cudaMemset(bad.p, 0, 4));
    uint64_t nnz = 0;
    if (m) {
        CUDA_TRY(cudaMalloc(&rows.p, 8 * nd));
        directed_rows<<<grid_for(m), 256>>>(d_edges, m, num_vertices, rows.as<uint32_t>(), bad.as<uint32_t>());
        CUDA_TRY(cudaGetLastError());
        uint32_t hbad = 0;
        CUDA_TRY(cudaMemcpy(&hbad, bad.p, 4, cudaMemcpyDeviceToHost));
        if (hbad) return fail(SGE_BAD_INPUT, "edge list has a vertex id >= num_vertices (%u)", num_vertices);
        sge_status st = sge_sort_tuples(rows.as<uint32_t>(), nd, 2);
        if (st != SGE_OK) return st;
        CUDA_TRY(cudaMalloc(&keep.p, 4 * nd));
        CUDA_TRY(cudaMalloc(&pos.p, 4 * nd));
        first_of_run<<<grid_for(nd), 256>>>(rows.as<uint32_t>(), nd, keep.as<uint32_t>());
        CUDA_TRY(cudaGetLastError());
        st = device_exclusive_scan(keep.as<uint32_t>(), pos.as<uint32_t>(), nd, 0);
        if (st != SGE_OK) return st;
        uint32_t last_pos = 0, last_keep = 0;
        CUDA_TRY(cudaMemcpy(&last_pos, pos.as<uint32_t>() + nd - 1, 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(&last_keep, keep.as<uint32_t>() + nd - 1, 4, cudaMemcpyDeviceToHost));
        nnz = (uint64_t)last_pos + last_keep;
    }
    CUDA_TRY(cudaMalloc(&src.p, 4 * std::max<uint64_t>(nnz, 1)));
    cudaError_t e;
    if ((e = cudaMalloc(&d_adj, 4 * std::max<uint64_t>(nnz, 1))) != cudaSuccess ||
        (e = cudaMalloc(&d_off, 4 * ((size_t)num_vertices + 1))) != cudaSuccess) {
        cudaFree(d_adj);
        return fail(SGE_OOM, "device CSR allocation: %s", cudaGetErrorString(e));
    }
    if (nnz)
        compact_rows<<<grid_for(nd), 256>>>(rows.as<uint32_t>(), nd, keep.as<uint32_t>(), pos.as<uint32_t>(),
                                             src.as<uint32_t>(), d_adj);
    offsets_from_sources<<<grid_for((unsigned long long)num_vertices + 1), 256>>>(src.as<uint32_t>(), nnz,
                                                                                 num_vertices, d_off);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
        cudaFree(d_adj);
        cudaFree(d_off);
        return fail(SGE_CUDA_ERROR, "device CSR build: %s", cudaGetErrorString(e));
    }
    return graph_adopt(d_off, d_adj, num_vertices, nnz, device, out);
}

sge_status sge_graph_create_rmat(uint32_t scale, uint64_t m, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm,
                                 uint64_t seed, int device, sge_graph **out) {
    if (scale < 1 || scale > 31 || !out) return fail(SGE_BAD_INPUT, "sge_graph_create_rmat: bad argument");
    if ((uint64_t)a_ppm + b_ppm + c_ppm > 1000000u) return fail(SGE_BAD_INPUT, "sge_graph_create_rmat: a+b+c > 1");
    const uint64_t max_edges = ((uint64_t)1 << scale) * (((uint64_t)1 << scale) - 1) / 2;
    if (m > max_edges / 2) return fail(SGE_BAD_INPUT, "sge_graph_create_rmat: %llu edges too dense for scale %u", (unsigned long long)m, scale);
    int ndev = sge_device_count();
    if (ndev == 0) return fail(SGE_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(SGE_BAD_INPUT, "device %d out of range (%d visible)", device, ndev);
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(device));
    auto thr = [](uint64_t ppm) { return (uint32_t)std::min<uint64_t>(0xFFFFFFFFull, (ppm << 32) / 1000000u); };
    const uint32_t ta = thr(a_ppm), tab = thr((uint64_t)a_ppm + b_ppm), tabc = thr((uint64_t)a_ppm + b_ppm + c_ppm);
    // the host generator's rounds: draw, count distinct edges, keep the m
    // whose first draw comes earliest (sge_gen_rmat in generators.cpp)
    uint64_t draws = m + m / 4 + 1024;
    for (int round = 0; round < 64; ++round) {
        if (draws >= (1ull << 32)) return fail(SGE_UNSUPPORTED, "sge_graph_create_rmat: %llu draws exceed 2^32", (unsigned long long)draws);
        DevBuf rows, firsts, count, edges;
        CUDA_TRY(cudaMalloc(&rows.p, 12 * draws));
        rmat_rows<<<grid_for(draws), 256>>>(seed, scale, ta, tab, tabc, draws, rows.as<uint32_t>());
        CUDA_TRY(cudaGetLastError());
        sge_status st = sge_sort_tuples(rows.as<uint32_t>(), draws, 3);
        if (st != SGE_OK) return st;
        CUDA_TRY(cudaMalloc(&firsts.p, 12 * draws));
        CUDA_TRY(cudaMalloc(&count.p, 8));
        CUDA_TRY(cudaMemset(count.p, 0, 8));
        first_draws<<<grid_for(draws), 256>>>(rows.as<uint32_t>(), draws, firsts.as<uint32_t>(),
                                              count.as<unsigned long long>());
        CUDA_TRY(cudaGetLastError());
        unsigned long long uniq = 0;
        CUDA_TRY(cudaMemcpy(&uniq, count.p, 8, cudaMemcpyDeviceToHost));
        if (uniq >= m) {
            st = sge_sort_tuples(firsts.as<uint32_t>(), uniq, 3);  // by first-draw index
            if (st != SGE_OK) return st;
            CUDA_TRY(cudaMalloc(&edges.p, 8 * std::max<uint64_t>(m, 1)));
            if (m) drop_index<<<grid_for(m), 256>>>(firsts.as<uint32_t>(), m, edges.as<uint32_t>());
            CUDA_TRY(cudaDeviceSynchronize());
            rows.release();  // the draws are not needed for the CSR build
            firsts.release();
            return sge_graph_create_from_device_edges(edges.as<uint32_t>(), m, 1u << scale, device, out);
        }
        draws += (m - uniq) * 2 + (m - uniq) / 2 + 1024;
    }
    return fail(SGE_BAD_INPUT, "sge_graph_create_rmat: could not reach %llu distinct edges", (unsigned long long)m);
}

}  // extern "C"
