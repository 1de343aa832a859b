// Seeded synthetic inputs: R-MAT and Chung-Lu data graphs, random connected
// patterns.  Every random draw comes from splitmix64 streams and all sampling
// decisions are integer comparisons, so a seed produces the same graph on
// every host (x86 here, Arm on the GPU hosts).
#include "common.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_set>
#include <vector>

using namespace sge;

namespace {

unsigned host_threads() { return std::max(1u, std::min(64u, std::thread::hardware_concurrency())); }

// Sorts 64-bit keys with a parallel MSD bucket pass followed by per-bucket sorts.
void parallel_sort_u64(std::vector<uint64_t> &a) {
    const size_t n = a.size();
    if (n < (1u << 20)) { std::sort(a.begin(), a.end()); return; }
    const unsigned nt = host_threads();
    const int B = 4096;
    uint64_t mx = 0;
    for (uint64_t x : a) mx = std::max(mx, x);
    int shift = 0;
    while (shift < 64 && (mx >> shift) >= (uint64_t)B) ++shift;
    std::vector<std::vector<size_t>> cnt(nt, std::vector<size_t>(B, 0));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            size_t lo = n * t / nt, hi = n * (t + 1) / nt;
            for (size_t i = lo; i < hi; ++i) cnt[t][a[i] >> shift]++;
        });
    for (auto &x : th) x.join();
    th.clear();
    std::vector<size_t> start(B + 1, 0);
    std::vector<std::vector<size_t>> pos(nt, std::vector<size_t>(B, 0));
    size_t acc = 0;
    for (int b = 0; b < B; ++b) {
        start[b] = acc;
        for (unsigned t = 0; t < nt; ++t) { pos[t][b] = acc; acc += cnt[t][b]; }
    }
    start[B] = acc;
    std::vector<uint64_t> out(n);
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            size_t lo = n * t / nt, hi = n * (t + 1) / nt;
            for (size_t i = lo; i < hi; ++i) out[pos[t][a[i] >> shift]++] = a[i];
        });
    for (auto &x : th) x.join();
    th.clear();
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            for (int b = (int)t; b < B; b += (int)nt) std::sort(out.begin() + start[b], out.begin() + start[b + 1]);
        });
    for (auto &x : th) x.join();
    a.swap(out);
}

// One R-MAT draw: `scale` quadrant choices, two per 64-bit random word.
inline uint64_t rmat_draw(uint64_t seed, uint64_t idx, uint32_t scale, uint32_t ta, uint32_t tab, uint32_t tabc) {
    uint32_t u = 0, v = 0;
    uint64_t word = 0;
    for (uint32_t bit = 0; bit < scale; ++bit) {
        uint32_t r;
        if ((bit & 1) == 0) {
            word = splitmix64(seed * 0x100000001B3ull + idx * 64 + bit);
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
    if (u > v) std::swap(u, v);
    return ((uint64_t)u << 32) | v;
}

}  // namespace

extern "C" {

sge_status sge_gen_rmat(uint32_t scale, uint64_t m, uint32_t a_ppm, uint32_t b_ppm, uint32_t c_ppm, uint64_t seed,
                        uint32_t **edges_out, uint64_t *m_out) {
    if (scale < 1 || scale > 31 || !edges_out || !m_out) return fail(SGE_BAD_INPUT, "sge_gen_rmat: bad argument");
    if ((uint64_t)a_ppm + b_ppm + c_ppm > 1000000u) return fail(SGE_BAD_INPUT, "sge_gen_rmat: a+b+c > 1");
    const uint64_t max_edges = ((uint64_t)1 << scale) * (((uint64_t)1 << scale) - 1) / 2;
    if (m > max_edges / 2) return fail(SGE_BAD_INPUT, "sge_gen_rmat: %llu edges too dense for scale %u", (unsigned long long)m, scale);
    auto thr = [](uint64_t ppm) { return (uint32_t)std::min<uint64_t>(0xFFFFFFFFull, (ppm << 32) / 1000000u); };
    const uint32_t ta = thr(a_ppm), tab = thr((uint64_t)a_ppm + b_ppm), tabc = thr((uint64_t)a_ppm + b_ppm + c_ppm);
    const unsigned nt = host_threads();
    // Draw in rounds until at least m distinct edges exist; then keep exactly
    // the m edges whose first draw index is smallest (deterministic cut).
    uint64_t draws = m + m / 4 + 1024;
    std::vector<uint64_t> keyed;  // (edge key) only, for counting
    for (int round = 0; round < 64; ++round) {
        std::vector<uint64_t> keys(draws);
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t]() {
                uint64_t lo = draws * t / nt, hi = draws * (t + 1) / nt;
                for (uint64_t i = lo; i < hi; ++i) keys[i] = rmat_draw(seed, i, scale, ta, tab, tabc);
            });
        for (auto &x : th) x.join();
        std::vector<uint64_t> s(keys);
        parallel_sort_u64(s);
        uint64_t uniq = 0;
        for (size_t i = 0; i < s.size(); ++i)
            if (s[i] != ~0ull && (i == 0 || s[i] != s[i - 1])) ++uniq;
        if (uniq >= m) {
            // first-draw index of each distinct edge: scan draws in order with a
            // sorted-membership pass: keep draw i iff it is the first occurrence.
            // Done by sorting (key, idx) pairs packed as key-major.
            std::vector<uint64_t> firsts;
            {
                // pair sort: stable partition by key using an index array
                std::vector<uint64_t> idx(draws);
                for (uint64_t i = 0; i < draws; ++i) idx[i] = i;
                std::stable_sort(idx.begin(), idx.end(), [&](uint64_t x, uint64_t y) { return keys[x] < keys[y]; });
                firsts.reserve(uniq);
                for (size_t i = 0; i < idx.size(); ++i) {
                    uint64_t kx = keys[idx[i]];
                    if (kx == ~0ull) continue;
                    if (i == 0 || kx != keys[idx[i - 1]]) firsts.push_back(idx[i]);
                }
            }
            if (firsts.size() > m) {
                std::nth_element(firsts.begin(), firsts.begin() + (ptrdiff_t)m, firsts.end());
                firsts.resize(m);
            }
            std::vector<uint64_t> chosen(firsts.size());
            for (size_t i = 0; i < firsts.size(); ++i) chosen[i] = keys[firsts[i]];
            parallel_sort_u64(chosen);
            uint32_t *e = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (chosen.size() ? chosen.size() : 1));
            if (!e) return fail(SGE_OOM, "sge_gen_rmat: host allocation failed");
            for (size_t i = 0; i < chosen.size(); ++i) {
                e[2 * i] = (uint32_t)(chosen[i] >> 32);
                e[2 * i + 1] = (uint32_t)chosen[i];
            }
            *edges_out = e;
            *m_out = chosen.size();
            return SGE_OK;
        }
        draws += (m - uniq) * 2 + (m - uniq) / 2 + 1024;
    }
    return fail(SGE_BAD_INPUT, "sge_gen_rmat: could not reach %llu distinct edges", (unsigned long long)m);
}

// Chung-Lu: expected degree of vertex i proportional to (i+1)^(-1/(gamma-1)),
// scaled to mean degree 2m/n and capped at max_deg; endpoints of each draw are
// sampled from the integer-rounded weights; self-loops and repeats are skipped
// until m distinct edges exist.
sge_status sge_gen_chung_lu(uint32_t n, uint64_t m, uint32_t gamma_milli, uint32_t max_deg, uint64_t seed,
                            uint32_t **edges_out, uint64_t *m_out) {
    if (n < 2 || gamma_milli <= 1000 || !edges_out || !m_out) return fail(SGE_BAD_INPUT, "sge_gen_chung_lu: bad argument");
    if (m > (uint64_t)n * (n - 1) / 4) return fail(SGE_BAD_INPUT, "sge_gen_chung_lu: too dense");
    const double alpha = 1000.0 / ((double)gamma_milli - 1000.0);
    std::vector<double> w(n);
    double sum = 0;
    for (uint32_t i = 0; i < n; ++i) { w[i] = std::pow((double)(i + 1), -alpha); sum += w[i]; }
    const double target = 2.0 * (double)m;
    double cap = max_deg ? (double)max_deg : (double)(n - 1);
    // scale, cap, rescale the uncapped part (a few fixed iterations)
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
    std::vector<uint64_t> cdf(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) {
        double x = std::min(cap, w[i] * scale);
        uint64_t iw = (uint64_t)std::llround(x * 256.0);
        if (iw == 0) iw = 1;
        cdf[i + 1] = cdf[i] + iw;
    }
    const uint64_t total = cdf[n];
    Rng rng(seed);
    auto pick = [&]() -> uint32_t {
        uint64_t r = rng.below(total);
        return (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r) - cdf.begin() - 1);
    };
    std::unordered_set<uint64_t> seen;
    seen.reserve(m * 2);
    std::vector<uint64_t> keys;
    keys.reserve(m);
    uint64_t guard = 0;
    while (keys.size() < m) {
        if (++guard > 200 * m + 100000) return fail(SGE_BAD_INPUT, "sge_gen_chung_lu: could not reach %llu distinct edges", (unsigned long long)m);
        uint32_t u = pick(), v = pick();
        if (u == v) continue;
        if (u > v) std::swap(u, v);
        uint64_t key = ((uint64_t)u << 32) | v;
        if (seen.insert(key).second) keys.push_back(key);
    }
    std::sort(keys.begin(), keys.end());
    uint32_t *e = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (keys.size() ? keys.size() : 1));
    if (!e) return fail(SGE_OOM, "sge_gen_chung_lu: host allocation failed");
    for (size_t i = 0; i < keys.size(); ++i) {
        e[2 * i] = (uint32_t)(keys[i] >> 32);
        e[2 * i + 1] = (uint32_t)keys[i];
    }
    *edges_out = e;
    *m_out = keys.size();
    return SGE_OK;
}

sge_status sge_gen_pattern(uint32_t k, uint32_t m, uint64_t seed, uint32_t *edges) {
    if (k < 2 || k > SGE_MAX_K || !edges) return fail(SGE_BAD_INPUT, "sge_gen_pattern: k=%u outside 2..%u", k, SGE_MAX_K);
    if (m < k - 1 || m > k * (k - 1) / 2) return fail(SGE_BAD_INPUT, "sge_gen_pattern: m=%u impossible for a connected %u-vertex pattern", m, k);
    Rng rng(seed ^ 0x50415454ull);
    bool adj[SGE_MAX_K][SGE_MAX_K] = {};
    // random labelled spanning tree (each vertex attaches to a random earlier one)
    uint32_t perm[SGE_MAX_K];
    for (uint32_t i = 0; i < k; ++i) perm[i] = i;
    for (uint32_t i = k - 1; i > 0; --i) { uint32_t j = (uint32_t)rng.below(i + 1); std::swap(perm[i], perm[j]); }
    uint32_t cnt = 0;
    for (uint32_t i = 1; i < k; ++i) {
        uint32_t j = (uint32_t)rng.below(i);
        uint32_t a = perm[i], b = perm[j];
        adj[a][b] = adj[b][a] = true;
        ++cnt;
    }
    while (cnt < m) {
        uint32_t a = (uint32_t)rng.below(k), b = (uint32_t)rng.below(k);
        if (a == b || adj[a][b]) continue;
        adj[a][b] = adj[b][a] = true;
        ++cnt;
    }
    uint32_t w = 0;
    for (uint32_t a = 0; a < k; ++a)
        for (uint32_t b = a + 1; b < k; ++b)
            if (adj[a][b]) { edges[2 * w] = a; edges[2 * w + 1] = b; ++w; }
    return SGE_OK;
}

}  // extern "C"
