// Learned plan scorer: a 3-layer MLP (in → H → H → 1, ReLU) that predicts a
// plan's log runtime from its features.  It stands in for the cost the
// reference's optimizer minimises (computeOrderCost / optCostOrder,
// plan/optimizer.cpp:319-577, fed by cardEstimateUnlabeled,
// plan/estimator.cpp:562-661); the cost model stays as the fallback and as
// the baseline the scorer is compared with.
//
// Training runs on the GPU in FP32 with this file's kernels (tiled SGEMM,
// bias/ReLU epilogues, column-sum bias gradients, Adam).  Batched inference
// runs in BF16 on the tensor cores (mma.sync m16n8k16, FP32 accumulate): the
// scorer is a few microseconds per pattern, far from any roofline that would
// justify the tcgen05 machinery.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "device_util.hpp"

using namespace sge;

struct sge_mlp {
    int device = 0;
    uint32_t in = 0, hid = 0;
    cudaStream_t stream = nullptr;
    // parameters (FP32): W1 [hid×in], b1 [hid], W2 [hid×hid], b2 [hid], W3 [hid], b3 [1]
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    size_t np = 0;
    uint64_t adam_t = 0;
    // BF16 copies of the weight matrices for inference
    __nv_bfloat16 *d_w1h = nullptr, *d_w2h = nullptr;
    bool bf16_stale = true;
    // workspace
    float *d_ws = nullptr;
    size_t ws_floats = 0;
};

namespace {

#define CUDA_TRY(expr)                                                                               \
    do {                                                                                             \
        cudaError_t _e = (expr);                                                                     \
        if (_e != cudaSuccess)                                                                       \
            return fail(_e == cudaErrorMemoryAllocation ? SGE_OOM : SGE_CUDA_ERROR, "%s: %s", #expr, \
                        cudaGetErrorString(_e));                                                     \
    } while (0)

constexpr int TILE = 16;

// C[M×N] = op(A)·op(B) (+ bias[N]) (ReLU) ; A is M×K (TA: stored K×M), B is K×N
// (TB: stored N×K), all row-major.  beta accumulates into C.
template <bool TA, bool TB>
__global__ void sgemm(const float *__restrict__ A, const float *__restrict__ B, float *__restrict__ C, int M, int N,
                      int K, const float *__restrict__ bias, int relu, float beta) {
    __shared__ float As[TILE][TILE + 1];
    __shared__ float Bs[TILE][TILE + 1];
    const int r = blockIdx.y * TILE + threadIdx.y, col = blockIdx.x * TILE + threadIdx.x;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += TILE) {
        const int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
        As[threadIdx.y][threadIdx.x] = (r < M && ka < K) ? (TA ? A[(size_t)ka * M + r] : A[(size_t)r * K + ka]) : 0.f;
        Bs[threadIdx.y][threadIdx.x] = (kb < K && col < N) ? (TB ? B[(size_t)col * K + kb] : B[(size_t)kb * N + col]) : 0.f;
        __syncthreads();
#pragma unroll
        for (int t = 0; t < TILE; ++t) acc += As[threadIdx.y][t] * Bs[t][threadIdx.x];
        __syncthreads();
    }
    if (r < M && col < N) {
        float v = acc;
        if (bias) v += bias[col];
        if (relu) v = v > 0.f ? v : 0.f;
        C[(size_t)r * N + col] = beta != 0.f ? beta * C[(size_t)r * N + col] + v : v;
    }
}

// dZ = dA ⊙ (Z > 0)
__global__ void relu_grad(float *dA, const float *Z, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n && Z[i] <= 0.f) dA[i] = 0.f;
}

// out[j] = Σ_i X[i][j]  (bias gradient), X is rows×cols
__global__ void colsum(const float *X, float *out, int rows, int cols) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.f;
    for (int i = 0; i < rows; ++i) s += X[(size_t)i * cols + j];
    out[j] = s;
}

// dy = (y - t) / B ; loss partials
__global__ void mse_grad(const float *y, const float *t, float *dy, float *loss, int B) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    float d = y[i] - t[i];
    dy[i] = d / (float)B;
    atomicAdd(loss, 0.5f * d * d / (float)B);
}

__global__ void adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                     float eps, float c1, float c2) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

__global__ void to_bf16(const float *x, __nv_bfloat16 *y, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// ---- BF16 tensor-core layer: Z[B×N] = X[B×K]·Wᵀ (W is N×K) + bias, ReLU ----
// One warp computes a 16×8 tile with mma.sync.m16n8k16 (row.col, f32 accumulate).
// Fragment layout (PTX ISA, m16n8k16 .bf16): g = lane/4, t = lane%4;
//   A regs: (g, 2t..2t+1), (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..)
//   B regs: (k 2t..2t+1, n g), (k 2t+8..2t+9, n g)
//   C/D:    (g, 2t), (g, 2t+1), (g+8, 2t), (g+8, 2t+1)
__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16 *p, int stride_ok0, int stride_ok1) {
    __nv_bfloat162 v;
    v.x = stride_ok0 ? p[0] : __float2bfloat16_rn(0.f);
    v.y = stride_ok1 ? p[1] : __float2bfloat16_rn(0.f);
    return *reinterpret_cast<uint32_t *>(&v);
}

__global__ void bf16_linear(const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ W,
                            const float *__restrict__ bias, float *__restrict__ Z, __nv_bfloat16 *__restrict__ Zh,
                            int B, int N, int K, int relu) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int tiles_n = (N + 7) / 8;
    const int tm = warp / tiles_n, tn = warp % tiles_n;
    if (tm * 16 >= B) return;
    const int g = lane >> 2, t = lane & 3;
    const int r0 = tm * 16 + g, r1 = r0 + 8, n = tn * 8 + g;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int ka = k0 + 2 * t, kb = ka + 8;
        uint32_t a0 = pack2(X + (size_t)r0 * K + ka, r0 < B && ka < K, r0 < B && ka + 1 < K);
        uint32_t a1 = pack2(X + (size_t)r1 * K + ka, r1 < B && ka < K, r1 < B && ka + 1 < K);
        uint32_t a2 = pack2(X + (size_t)r0 * K + kb, r0 < B && kb < K, r0 < B && kb + 1 < K);
        uint32_t a3 = pack2(X + (size_t)r1 * K + kb, r1 < B && kb < K, r1 < B && kb + 1 < K);
        uint32_t b0 = pack2(W + (size_t)n * K + ka, n < N && ka < K, n < N && ka + 1 < K);
        uint32_t b1 = pack2(W + (size_t)n * K + kb, n < N && kb < K, n < N && kb + 1 < K);
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(c0), "+f"(c1), "+f"(c2), "+f"(c3)
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    const int col0 = tn * 8 + 2 * t;
    float out[4] = {c0, c1, c2, c3};
    const int rows[4] = {r0, r0, r1, r1};
    const int cols[4] = {col0, col0 + 1, col0, col0 + 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (rows[q] < B && cols[q] < N) {
            float v = out[q] + (bias ? bias[cols[q]] : 0.f);
            if (relu) v = v > 0.f ? v : 0.f;
            if (Z) Z[(size_t)rows[q] * N + cols[q]] = v;
            if (Zh) Zh[(size_t)rows[q] * N + cols[q]] = __float2bfloat16_rn(v);
        }
    }
}

// y[i] = Σ_j A2[i][j]·w3[j] + b3 (FP32; the last layer has one output)
__global__ void dot_out(const float *A, const float *w, const float *b, float *y, int B, int H) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    float s = b[0];
    for (int j = 0; j < H; ++j) s += A[(size_t)i * H + j] * w[j];
    y[i] = s;
}

inline dim3 gemm_grid(int M, int N) { return dim3((N + TILE - 1) / TILE, (M + TILE - 1) / TILE); }

struct Layout {
    size_t w1, b1, w2, b2, w3, b3, n;
};
Layout layout(uint32_t in, uint32_t hid) {
    Layout L;
    L.w1 = 0;
    L.b1 = L.w1 + (size_t)hid * in;
    L.w2 = L.b1 + hid;
    L.b2 = L.w2 + (size_t)hid * hid;
    L.w3 = L.b2 + hid;
    L.b3 = L.w3 + hid;
    L.n = L.b3 + 1;
    return L;
}

sge_status ensure_ws(sge_mlp *m, uint32_t B) {
    // X, Z1, A1, Z2, A2, y, t, dy, dA, loss
    size_t need = (size_t)B * m->in + 4ull * B * m->hid + 3ull * B + (size_t)B * m->hid + 64;
    if (m->ws_floats >= need) return SGE_OK;
    cudaFree(m->d_ws);
    m->d_ws = nullptr;
    CUDA_TRY(cudaMalloc(&m->d_ws, need * sizeof(float)));
    m->ws_floats = need;
    return SGE_OK;
}

// Forward in FP32; leaves Z1, A1, Z2, A2, y in the workspace.
void forward_fp32(sge_mlp *m, const Layout &L, float *X, float *Z1, float *A1, float *Z2, float *A2, float *y,
                  uint32_t B) {
    const dim3 blk(TILE, TILE);
    float *P = m->d_p;
    sgemm<false, true><<<gemm_grid(B, m->hid), blk, 0, m->stream>>>(X, P + L.w1, Z1, B, m->hid, m->in, P + L.b1, 0, 0.f);
    cudaMemcpyAsync(A1, Z1, sizeof(float) * B * m->hid, cudaMemcpyDeviceToDevice, m->stream);
    size_t nh = (size_t)B * m->hid;
    relu_grad<<<(unsigned)((nh + 255) / 256), 256, 0, m->stream>>>(A1, Z1, nh);  // A1 = relu(Z1)
    sgemm<false, true><<<gemm_grid(B, m->hid), blk, 0, m->stream>>>(A1, P + L.w2, Z2, B, m->hid, m->hid, P + L.b2, 0, 0.f);
    cudaMemcpyAsync(A2, Z2, sizeof(float) * nh, cudaMemcpyDeviceToDevice, m->stream);
    relu_grad<<<(unsigned)((nh + 255) / 256), 256, 0, m->stream>>>(A2, Z2, nh);
    dot_out<<<(B + 255) / 256, 256, 0, m->stream>>>(A2, P + L.w3, P + L.b3, y, B, m->hid);
}

}  // namespace

extern "C" {

sge_status sge_mlp_create(uint32_t in_dim, uint32_t hidden, uint64_t seed, int device, sge_mlp **out) {
    if (!out || in_dim == 0 || hidden == 0 || in_dim > 4096 || hidden > 4096)
        return fail(SGE_BAD_INPUT, "sge_mlp_create: bad dimensions");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return fail(SGE_NO_DEVICE, "no CUDA device visible"); }
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(device));
    sge_mlp *m = new sge_mlp();
    m->device = device;
    m->in = in_dim;
    m->hid = hidden;
    Layout L = layout(in_dim, hidden);
    m->np = L.n;
    std::vector<float> h(L.n, 0.f);
    Rng rng(seed);
    auto uni = [&](float a) { return (float)(((double)(rng.next() >> 11) / 9007199254740992.0) * 2.0 - 1.0) * a; };
    const float s1 = std::sqrt(6.f / (in_dim + hidden)), s2 = std::sqrt(6.f / (2.f * hidden)), s3 = std::sqrt(6.f / (hidden + 1.f));
    for (size_t i = 0; i < (size_t)hidden * in_dim; ++i) h[L.w1 + i] = uni(s1);
    for (size_t i = 0; i < (size_t)hidden * hidden; ++i) h[L.w2 + i] = uni(s2);
    for (size_t i = 0; i < hidden; ++i) h[L.w3 + i] = uni(s3);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_p, 4 * L.n * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(&m->d_w1h, sizeof(__nv_bfloat16) * hidden * in_dim)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_w2h, sizeof(__nv_bfloat16) * hidden * hidden)) != cudaSuccess) {
        sge_mlp_destroy(m);
        return fail(SGE_OOM, "sge_mlp_create: %s", cudaGetErrorString(e));
    }
    m->d_g = m->d_p + L.n;
    m->d_m = m->d_g + L.n;
    m->d_v = m->d_m + L.n;
    cudaMemcpy(m->d_p, h.data(), L.n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(m->d_m, 0, 2 * L.n * sizeof(float));
    *out = m;
    return SGE_OK;
}

sge_status sge_mlp_destroy(sge_mlp *m) {
    if (!m) return SGE_OK;
    DeviceGuard restore_device;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->d_p);
    cudaFree(m->d_w1h);
    cudaFree(m->d_w2h);
    cudaFree(m->d_ws);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SGE_OK;
}

sge_status sge_mlp_num_params(const sge_mlp *m, size_t *n) {
    if (!m || !n) return fail(SGE_BAD_INPUT, "null argument");
    *n = m->np;
    return SGE_OK;
}

sge_status sge_mlp_get_params(const sge_mlp *m, float *out) {
    if (!m || !out) return fail(SGE_BAD_INPUT, "null argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    CUDA_TRY(cudaMemcpy(out, m->d_p, m->np * sizeof(float), cudaMemcpyDeviceToHost));
    return SGE_OK;
}

sge_status sge_mlp_set_params(sge_mlp *m, const float *in) {
    if (!m || !in) return fail(SGE_BAD_INPUT, "null argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    CUDA_TRY(cudaMemcpy(m->d_p, in, m->np * sizeof(float), cudaMemcpyHostToDevice));
    m->bf16_stale = true;
    m->adam_t = 0;
    CUDA_TRY(cudaMemset(m->d_m, 0, 2 * m->np * sizeof(float)));
    return SGE_OK;
}

sge_status sge_mlp_forward(sge_mlp *m, const float *x, uint32_t B, float *y) {
    if (!m || (!x && B) || (!y && B)) return fail(SGE_BAD_INPUT, "null argument");
    if (B == 0) return SGE_OK;
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    sge_status st = ensure_ws(m, B);
    if (st != SGE_OK) return st;
    Layout L = layout(m->in, m->hid);
    float *X = m->d_ws, *Z1 = X + (size_t)B * m->in, *A1 = Z1 + (size_t)B * m->hid, *Z2 = A1 + (size_t)B * m->hid,
          *A2 = Z2 + (size_t)B * m->hid, *Y = A2 + (size_t)B * m->hid;
    CUDA_TRY(cudaMemcpyAsync(X, x, sizeof(float) * B * m->in, cudaMemcpyHostToDevice, m->stream));
    forward_fp32(m, L, X, Z1, A1, Z2, A2, Y, B);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(y, Y, sizeof(float) * B, cudaMemcpyDeviceToHost, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return SGE_OK;
}

sge_status sge_mlp_forward_bf16(sge_mlp *m, const float *x, uint32_t B, float *y) {
    if (!m || (!x && B) || (!y && B)) return fail(SGE_BAD_INPUT, "null argument");
    if (B == 0) return SGE_OK;
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    sge_status st = ensure_ws(m, B);
    if (st != SGE_OK) return st;
    Layout L = layout(m->in, m->hid);
    if (m->bf16_stale) {
        size_t n1 = (size_t)m->hid * m->in, n2 = (size_t)m->hid * m->hid;
        to_bf16<<<(unsigned)((n1 + 255) / 256), 256, 0, m->stream>>>(m->d_p + L.w1, m->d_w1h, n1);
        to_bf16<<<(unsigned)((n2 + 255) / 256), 256, 0, m->stream>>>(m->d_p + L.w2, m->d_w2h, n2);
        m->bf16_stale = false;
    }
    // workspace reuse: X (fp32) | Xh | A1h | A2 (fp32) | y
    float *X = m->d_ws;
    __nv_bfloat16 *Xh = reinterpret_cast<__nv_bfloat16 *>(X + (size_t)B * m->in);
    __nv_bfloat16 *A1h = Xh + (size_t)B * m->in + 8;
    float *A2 = reinterpret_cast<float *>(A1h + (size_t)B * m->hid + 8);
    A2 = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(A2) + 15) & ~(uintptr_t)15);
    float *Y = A2 + (size_t)B * m->hid;
    CUDA_TRY(cudaMemcpyAsync(X, x, sizeof(float) * B * m->in, cudaMemcpyHostToDevice, m->stream));
    size_t nx = (size_t)B * m->in;
    to_bf16<<<(unsigned)((nx + 255) / 256), 256, 0, m->stream>>>(X, Xh, nx);
    const int tiles = ((B + 15) / 16) * ((m->hid + 7) / 8);
    const int threads = 128, blocks = (tiles * 32 + threads - 1) / threads;
    bf16_linear<<<blocks, threads, 0, m->stream>>>(Xh, m->d_w1h, m->d_p + L.b1, nullptr, A1h, B, m->hid, m->in, 1);
    bf16_linear<<<blocks, threads, 0, m->stream>>>(A1h, m->d_w2h, m->d_p + L.b2, A2, nullptr, B, m->hid, m->hid, 1);
    dot_out<<<(B + 255) / 256, 256, 0, m->stream>>>(A2, m->d_p + L.w3, m->d_p + L.b3, Y, B, m->hid);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(y, Y, sizeof(float) * B, cudaMemcpyDeviceToHost, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return SGE_OK;
}

// Loss 0.5·mean((f(x)-t)²) and its gradient (flat, parameter layout) for one batch.
static sge_status loss_grad_dev(sge_mlp *m, const float *x, const float *t, uint32_t B, float *loss_out,
                                bool copy_grads, float *grads_out) {
    sge_status st = ensure_ws(m, B);
    if (st != SGE_OK) return st;
    Layout L = layout(m->in, m->hid);
    const uint32_t H = m->hid;
    float *X = m->d_ws, *Z1 = X + (size_t)B * m->in, *A1 = Z1 + (size_t)B * H, *Z2 = A1 + (size_t)B * H,
          *A2 = Z2 + (size_t)B * H, *Y = A2 + (size_t)B * H, *T = Y + B, *dY = T + B, *dA = dY + B,
          *loss = dA + (size_t)B * H;
    CUDA_TRY(cudaMemcpyAsync(X, x, sizeof(float) * B * m->in, cudaMemcpyHostToDevice, m->stream));
    CUDA_TRY(cudaMemcpyAsync(T, t, sizeof(float) * B, cudaMemcpyHostToDevice, m->stream));
    CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), m->stream));
    forward_fp32(m, L, X, Z1, A1, Z2, A2, Y, B);
    mse_grad<<<(B + 255) / 256, 256, 0, m->stream>>>(Y, T, dY, loss, (int)B);
    float *G = m->d_g;
    const dim3 blk(TILE, TILE);
    // layer 3: dW3[j] = Σ_i A2[i][j] dY[i] ; db3 = Σ dY ; dA2 = dY w3ᵀ
    sgemm<true, false><<<gemm_grid(H, 1), blk, 0, m->stream>>>(A2, dY, G + L.w3, H, 1, B, nullptr, 0, 0.f);
    colsum<<<1, 32, 0, m->stream>>>(dY, G + L.b3, B, 1);
    sgemm<false, false><<<gemm_grid(B, H), blk, 0, m->stream>>>(dY, m->d_p + L.w3, dA, B, H, 1, nullptr, 0, 0.f);
    size_t nh = (size_t)B * H;
    relu_grad<<<(unsigned)((nh + 255) / 256), 256, 0, m->stream>>>(dA, Z2, nh);  // dZ2
    // layer 2: dW2 = dZ2ᵀ A1 ; db2 = colsum dZ2 ; dA1 = dZ2 W2
    sgemm<true, false><<<gemm_grid(H, H), blk, 0, m->stream>>>(dA, A1, G + L.w2, H, H, B, nullptr, 0, 0.f);
    colsum<<<(H + 127) / 128, 128, 0, m->stream>>>(dA, G + L.b2, B, H);
    float *dA1 = Z2;  // Z2 no longer needed once dZ2 exists: reuse its storage
    sgemm<false, false><<<gemm_grid(B, H), blk, 0, m->stream>>>(dA, m->d_p + L.w2, dA1, B, H, H, nullptr, 0, 0.f);
    relu_grad<<<(unsigned)((nh + 255) / 256), 256, 0, m->stream>>>(dA1, Z1, nh);  // dZ1
    // layer 1: dW1 = dZ1ᵀ X ; db1 = colsum dZ1
    sgemm<true, false><<<gemm_grid(H, m->in), blk, 0, m->stream>>>(dA1, X, G + L.w1, H, m->in, B, nullptr, 0, 0.f);
    colsum<<<(H + 127) / 128, 128, 0, m->stream>>>(dA1, G + L.b1, B, H);
    CUDA_TRY(cudaGetLastError());
    if (loss_out) CUDA_TRY(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    if (copy_grads && grads_out)
        CUDA_TRY(cudaMemcpyAsync(grads_out, G, sizeof(float) * m->np, cudaMemcpyDeviceToHost, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return SGE_OK;
}

sge_status sge_mlp_loss_grad(sge_mlp *m, const float *x, const float *t, uint32_t B, float *loss, float *grads) {
    if (!m || !x || !t || B == 0) return fail(SGE_BAD_INPUT, "sge_mlp_loss_grad: bad argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    return loss_grad_dev(m, x, t, B, loss, true, grads);
}

sge_status sge_mlp_train(sge_mlp *m, const float *x, const float *t, uint32_t n, uint32_t epochs, uint32_t batch,
                         float lr, uint64_t seed, float *final_loss) {
    if (!m || !x || !t || n == 0 || batch == 0) return fail(SGE_BAD_INPUT, "sge_mlp_train: bad argument");
    DeviceGuard restore_device;
    CUDA_TRY(cudaSetDevice(m->device));
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::vector<float> bx((size_t)batch * m->in), bt(batch);
    Rng rng(seed);
    float last = 0.f;
    for (uint32_t ep = 0; ep < epochs; ++ep) {
        for (uint32_t i = n - 1; i > 0; --i) std::swap(idx[i], idx[(uint32_t)rng.below(i + 1)]);
        double ep_loss = 0;
        uint32_t nb = 0;
        for (uint32_t s = 0; s < n; s += batch) {
            const uint32_t B = std::min(batch, n - s);
            for (uint32_t r = 0; r < B; ++r) {
                memcpy(&bx[(size_t)r * m->in], x + (size_t)idx[s + r] * m->in, sizeof(float) * m->in);
                bt[r] = t[idx[s + r]];
            }
            float loss = 0.f;
            sge_status st = loss_grad_dev(m, bx.data(), bt.data(), B, &loss, false, nullptr);
            if (st != SGE_OK) return st;
            ++m->adam_t;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f - std::pow(b1, (float)m->adam_t), c2 = 1.f - std::pow(b2, (float)m->adam_t);
            adam<<<(unsigned)((m->np + 255) / 256), 256, 0, m->stream>>>(m->d_p, m->d_g, m->d_m, m->d_v, m->np, lr,
                                                                          b1, b2, 1e-8f, c1, c2);
            ep_loss += loss;
            ++nb;
        }
        last = (float)(ep_loss / std::max(nb, 1u));
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    m->bf16_stale = true;
    if (final_loss) *final_loss = last;
    return SGE_OK;
}

}  // extern "C"
