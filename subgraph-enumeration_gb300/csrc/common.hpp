// Internal helpers shared by the host translation units of libsge.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <string>
#include "sge.h"

namespace sge {

// Thread-local last-error message (sge_last_error).
void set_error(const char *fmt, ...);
const char *last_error();

// Returns `st` after recording a formatted message.
sge_status fail(sge_status st, const char *fmt, ...);

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

}  // namespace sge
