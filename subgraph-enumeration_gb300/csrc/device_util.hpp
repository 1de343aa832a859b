// Internal device-side helpers shared by the CUDA translation units of libsge.
#pragma once
#include <cuda_runtime.h>

#include "common.hpp"

namespace sge {

// Restores the caller's current device when an entry point returns, so that
// a call which selects the graph's (or scorer's) device does not move a
// multi-GPU caller's later allocations and launches to that device.
struct DeviceGuard {
    int prev = -1;
    DeviceGuard() {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            prev = -1;
            cudaGetLastError();
        }
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;
};

// Exclusive prefix sum of n uint32 values in device memory (out may alias
// nothing in `in`), ordered on stream s; temporary space is allocated here.
sge_status device_exclusive_scan(const uint32_t *in, uint32_t *out, uint64_t n, cudaStream_t s);

// Wraps a CSR already in device memory on `device` (d_off: n+1 offsets,
// d_adj: nnz neighbours; symmetric, lists strictly increasing, no
// self-loops) as a graph, which takes ownership of both arrays (also on
// failure).  The root-edge list is built on the device; the planner's
// statistics are computed on the host, from h_off/h_adj when the caller has
// the CSR in host memory, else from a copy.
sge_status graph_adopt(uint32_t *d_off, uint32_t *d_adj, uint32_t n, uint64_t nnz, int device, sge_graph **out,
                       const uint32_t *h_off = nullptr, const uint32_t *h_adj = nullptr);

}  // namespace sge
