// mlp.cu -- the small multilayer perceptron of the learned cut ranking and dual
// warm start: FP32 forward, backward and Adam as hand-written sm_103a kernels.
//
// Network: x (d features) -> tanh(W1 x + b1) (h1) -> tanh(W2 . + b2) (h2) -> w3 . + b3.
// Loss: mean squared error over the batch.  Parameters live in one float vector
// [W1 (h1 x d, row-major) | b1 | W2 (h2 x h1) | b2 | w3 (h2) | b3].
//
// Gradients are deterministic: every block writes the sum of its samples'
// gradients (fixed order within the block) to its own row of a partials array,
// and the Adam kernel sums the rows in block order before the update (Adam:
// Kingma & Ba, 2015, with bias correction).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/mcbound.h"
#include "mcb_dev.cuh"
#include "mlp.h"

namespace mcb {
namespace {

constexpr int kTile = 128;  // samples per block of the gradient kernel

struct Dims {
    int d, h1, h2;
    __host__ __device__ int oW1() const { return 0; }
    __host__ __device__ int ob1() const { return h1 * d; }
    __host__ __device__ int oW2() const { return h1 * d + h1; }
    __host__ __device__ int ob2() const { return h1 * d + h1 + h2 * h1; }
    __host__ __device__ int ow3() const { return h1 * d + h1 + h2 * h1 + h2; }
    __host__ __device__ int ob3() const { return h1 * d + h1 + h2 * h1 + 2 * h2; }
    __host__ __device__ int P() const { return h1 * d + h1 + h2 * h1 + 2 * h2 + 1; }
};

// forward pass of one sample; a1 / a2 receive the hidden activations
__device__ __forceinline__ float fwd_one(const float *p, Dims D, const float *x, float *a1, float *a2) {
    for (int i = 0; i < D.h1; ++i) {
        float s = p[D.ob1() + i];
        const float *w = p + D.oW1() + i * D.d;
        for (int k = 0; k < D.d; ++k) s = fmaf(w[k], x[k], s);
        a1[i] = tanhf(s);
    }
    for (int j = 0; j < D.h2; ++j) {
        float s = p[D.ob2() + j];
        const float *w = p + D.oW2() + j * D.h1;
        for (int i = 0; i < D.h1; ++i) s = fmaf(w[i], a1[i], s);
        a2[j] = tanhf(s);
    }
    float y = p[D.ob3()];
    for (int j = 0; j < D.h2; ++j) y = fmaf(p[D.ow3() + j], a2[j], y);
    return y;
}

__global__ void __launch_bounds__(kTile) k_mlp_forward(const float *params, Dims D, const float *X, int n,
                                                       float *out) {
    extern __shared__ float sp[];
    const int P = D.P();
    for (int q = threadIdx.x; q < P; q += blockDim.x) sp[q] = params[q];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[kMlpMaxIn], a1[kMlpMaxHidden], a2[kMlpMaxHidden];
    for (int k = 0; k < D.d; ++k) x[k] = X[(size_t)s * D.d + k];
    out[s] = fwd_one(sp, D, x, a1, a2);
}

// Per-block gradient of sum_s (f(x_s) - y_s)^2 / n over the samples idx[b0 .. b0 + kTile)
// (idx = null: samples b0 ..), plus the block's share of the loss.
// Shared memory: the parameters, then per sample x (d), a1, d1 (h1), a2, d2 (h2).
__global__ void __launch_bounds__(kTile) k_mlp_grad(const float *params, Dims D, const float *X, const float *Y,
                                                    const int *idx, int n, int n_total, float *gpart,
                                                    float *lpart) {
    extern __shared__ float sm[];
    const int P = D.P();
    float *sp = sm;
    const int stride = D.d + 2 * D.h1 + 2 * D.h2;
    float *sv = sm + ((P + 3) & ~3);
    __shared__ float sdy[kTile];
    __shared__ float red[kTile];
    for (int q = threadIdx.x; q < P; q += blockDim.x) sp[q] = params[q];
    __syncthreads();
    const int t = threadIdx.x;
    const int b = blockIdx.x * kTile + t;
    float *xs = sv + (size_t)t * stride, *a1 = xs + D.d, *d1 = a1 + D.h1, *a2 = d1 + D.h1, *d2 = a2 + D.h2;
    float dy = 0.0f, l = 0.0f;
    if (b < n) {
        const int s = idx ? idx[b] : b;
        for (int k = 0; k < D.d; ++k) xs[k] = X[(size_t)s * D.d + k];
        float y = fwd_one(sp, D, xs, a1, a2);
        float r = y - Y[s];
        l = r * r / (float)n_total;
        dy = 2.0f * r / (float)n_total;
        for (int j = 0; j < D.h2; ++j) d2[j] = dy * sp[D.ow3() + j] * (1.0f - a2[j] * a2[j]);
        for (int i = 0; i < D.h1; ++i) {
            float s2 = 0.0f;
            for (int j = 0; j < D.h2; ++j) s2 = fmaf(d2[j], sp[D.oW2() + j * D.h1 + i], s2);
            d1[i] = s2 * (1.0f - a1[i] * a1[i]);
        }
    } else {
        for (int q = 0; q < stride; ++q) xs[q] = 0.0f;
    }
    sdy[t] = dy;
    red[t] = l;
    __syncthreads();
    // parameter sums over the tile's samples, in sample order
    const int cnt = min(kTile, n - (int)blockIdx.x * kTile);
    float *g = gpart + (size_t)blockIdx.x * P;
    for (int q = t; q < P; q += blockDim.x) {
        float acc = 0.0f;
        if (q < D.ob1()) {  // W1[i][k]
            int i = q / D.d, k = q - i * D.d;
            for (int u = 0; u < cnt; ++u) { const float *v = sv + (size_t)u * stride; acc = fmaf(v[D.d + D.h1 + i], v[k], acc); }
        } else if (q < D.oW2()) {  // b1[i]
            int i = q - D.ob1();
            for (int u = 0; u < cnt; ++u) acc += sv[(size_t)u * stride + D.d + D.h1 + i];
        } else if (q < D.ob2()) {  // W2[j][i]
            int r = q - D.oW2(), j = r / D.h1, i = r - j * D.h1;
            for (int u = 0; u < cnt; ++u) {
                const float *v = sv + (size_t)u * stride;
                acc = fmaf(v[D.d + 2 * D.h1 + D.h2 + j], v[D.d + i], acc);
            }
        } else if (q < D.ow3()) {  // b2[j]
            int j = q - D.ob2();
            for (int u = 0; u < cnt; ++u) acc += sv[(size_t)u * stride + D.d + 2 * D.h1 + D.h2 + j];
        } else if (q < D.ob3()) {  // w3[j]
            int j = q - D.ow3();
            for (int u = 0; u < cnt; ++u) acc = fmaf(sdy[u], sv[(size_t)u * stride + D.d + 2 * D.h1 + j], acc);
        } else {  // b3
            for (int u = 0; u < cnt; ++u) acc += sdy[u];
        }
        g[q] = acc;
    }
    if (t == 0) {
        float s = 0.0f;
        for (int u = 0; u < cnt; ++u) s += red[u];
        lpart[blockIdx.x] = s;
    }
}

// sum the block partials in block order; Adam update when lr > 0 (else gradient only)
__global__ void k_mlp_adam(float *params, float *m, float *v, const float *gpart, int nblk, int P, float lr,
                           float b1t, float b2t, float *grad_out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    float g = 0.0f;
    for (int k = 0; k < nblk; ++k) g += gpart[(size_t)k * P + q];
    if (grad_out) grad_out[q] = g;
    if (lr > 0.0f) {
        const float be1 = 0.9f, be2 = 0.999f, eps = 1e-8f;
        float mq = be1 * m[q] + (1.0f - be1) * g;
        float vq = be2 * v[q] + (1.0f - be2) * g * g;
        m[q] = mq;
        v[q] = vq;
        float mh = mq / (1.0f - b1t), vh = vq / (1.0f - b2t);
        params[q] -= lr * mh / (sqrtf(vh) + eps);
    }
}

__global__ void k_sum_loss(const float *lpart, int nblk, float *out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float s = 0.0f;
        for (int k = 0; k < nblk; ++k) s += lpart[k];
        *out = s;
    }
}

size_t grad_smem(Dims D) {
    return (size_t)(((D.P() + 3) & ~3) + kTile * (D.d + 2 * D.h1 + 2 * D.h2)) * sizeof(float);
}

}  // namespace

struct MlpImpl {
    Dims D{};
    float *p = nullptr, *m = nullptr, *v = nullptr, *gpart = nullptr, *lpart = nullptr, *gout = nullptr,
          *loss = nullptr;
    int nblk_cap = 0;
    float *dX = nullptr, *dY = nullptr, *dOut = nullptr;
    int *dIdx = nullptr;
    size_t cap = 0;
    long long step = 0;
};

int mlp_ensure(MlpImpl *M, size_t n) {
    const int nblk = (int)((n + kTile - 1) / kTile);
    if (nblk > M->nblk_cap) {
        if (M->gpart) cudaFree(M->gpart);
        if (M->lpart) cudaFree(M->lpart);
        M->gpart = M->lpart = nullptr;
        int c = std::max(nblk, 64);
        if (cudaMalloc(&M->gpart, (size_t)c * M->D.P() * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
        if (cudaMalloc(&M->lpart, (size_t)c * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
        M->nblk_cap = c;
    }
    if (n > M->cap) {
        if (M->dX) cudaFree(M->dX);
        if (M->dY) cudaFree(M->dY);
        if (M->dOut) cudaFree(M->dOut);
        if (M->dIdx) cudaFree(M->dIdx);
        M->dX = M->dY = M->dOut = nullptr;
        M->dIdx = nullptr;
        size_t c = std::max<size_t>(n, 4096);
        if (cudaMalloc(&M->dX, c * M->D.d * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
        if (cudaMalloc(&M->dY, c * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
        if (cudaMalloc(&M->dOut, c * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
        if (cudaMalloc(&M->dIdx, c * sizeof(int)) != cudaSuccess) return MCB_ERR_NOMEM;
        M->cap = c;
    }
    return MCB_OK;
}

void mlp_forward_device(const MlpImpl *M, const float *dX, int n, float *dOut, cudaStream_t st) {
    if (n <= 0) return;
    size_t sm = (size_t)M->D.P() * sizeof(float);
    k_mlp_forward<<<(n + kTile - 1) / kTile, kTile, sm, st>>>(M->p, M->D, dX, n, dOut);
}

// gradient of the loss over samples (idx or 0..n-1) into M->gout (and an Adam step if lr > 0)
int mlp_step_device(MlpImpl *M, const float *dX, const float *dY, const int *dIdx, int n, float lr, cudaStream_t st) {
    const int nblk = (n + kTile - 1) / kTile;
    const size_t sm = grad_smem(M->D);
    // per-device function attribute, set once on every device that trains
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCB_ERR_CUDA;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
    if (!bit || !(attr_set.load() & bit)) {
        if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
            return MCB_ERR_CUDA;
        attr_set.fetch_or(bit);
    }
    k_mlp_grad<<<nblk, kTile, sm, st>>>(M->p, M->D, dX, dY, dIdx, n, n, M->gpart, M->lpart);
    if (lr > 0.0f) M->step++;
    const float b1t = lr > 0.0f ? (float)pow(0.9, (double)M->step) : 0.0f;
    const float b2t = lr > 0.0f ? (float)pow(0.999, (double)M->step) : 0.0f;
    const int P = M->D.P();
    k_mlp_adam<<<(P + 255) / 256, 256, 0, st>>>(M->p, M->m, M->v, M->gpart, nblk, P, lr, b1t, b2t, M->gout);
    k_sum_loss<<<1, 32, 0, st>>>(M->lpart, nblk, M->loss);
    return cudaGetLastError() == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

}  // namespace mcb

using namespace mcb;

struct mcb_mlp {
    MlpImpl impl;
};

MlpImpl *mlp_impl(mcb_mlp *h) { return h ? &h->impl : nullptr; }
int mlp_inputs(const mcb_mlp *h) { return h ? h->impl.D.d : 0; }

extern "C" {

mcb_mlp *mcb_mlp_create(int d_in, int h1, int h2, uint64_t seed, int *status) {
    auto fail = [&](int c) -> mcb_mlp * {
        if (status) *status = c;
        return nullptr;
    };
    if (d_in < 1 || d_in > kMlpMaxIn || h1 < 1 || h1 > kMlpMaxHidden || h2 < 1 || h2 > kMlpMaxHidden)
        return fail(MCB_ERR_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MCB_ERR_NODEV);
    mcb_mlp *h = new mcb_mlp();
    MlpImpl &M = h->impl;
    M.D = Dims{d_in, h1, h2};
    const int P = M.D.P();
    bool ok = cudaMalloc(&M.p, P * sizeof(float)) == cudaSuccess && cudaMalloc(&M.m, P * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&M.v, P * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&M.gout, P * sizeof(float)) == cudaSuccess && cudaMalloc(&M.loss, sizeof(float)) == cudaSuccess;
    if (!ok || mlp_ensure(&M, 4096) != MCB_OK) {
        mcb_mlp_destroy(h);
        return fail(MCB_ERR_NOMEM);
    }
    // Glorot-uniform weights from a counter stream, zero biases
    std::vector<float> p(P, 0.0f);
    Stream rs{key2(seed, 0x4D4C50ull), 0};
    auto fill = [&](int off, int rows, int cols) {
        float s = sqrtf(6.0f / (float)(rows + cols));
        for (int q = 0; q < rows * cols; ++q) p[off + q] = (float)((2.0 * rs.next_unit() - 1.0) * s);
    };
    fill(M.D.oW1(), h1, d_in);
    fill(M.D.oW2(), h2, h1);
    fill(M.D.ow3(), 1, h2);
    cudaMemcpy(M.p, p.data(), P * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(M.m, 0, P * sizeof(float));
    cudaMemset(M.v, 0, P * sizeof(float));
    if (status) *status = MCB_OK;
    return h;
}

void mcb_mlp_destroy(mcb_mlp *h) {
    if (!h) return;
    MlpImpl &M = h->impl;
    void *ps[] = {M.p, M.m, M.v, M.gpart, M.lpart, M.gout, M.loss, M.dX, M.dY, M.dOut, M.dIdx};
    for (void *q : ps)
        if (q) cudaFree(q);
    delete h;
}

int mcb_mlp_num_params(const mcb_mlp *h) { return h ? h->impl.D.P() : 0; }

int mcb_mlp_get_params(const mcb_mlp *h, float *out) {
    if (!h || !out) return MCB_ERR_ARG;
    return cudaMemcpy(out, h->impl.p, h->impl.D.P() * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
               ? MCB_OK : MCB_ERR_CUDA;
}

int mcb_mlp_set_params(mcb_mlp *h, const float *in) {
    if (!h || !in) return MCB_ERR_ARG;
    MlpImpl &M = h->impl;
    const int P = M.D.P();
    M.step = 0;
    cudaMemset(M.m, 0, P * sizeof(float));
    cudaMemset(M.v, 0, P * sizeof(float));
    return cudaMemcpy(M.p, in, P * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

int mcb_mlp_predict(mcb_mlp *h, const float *X, int n, float *out) {
    if (!h || n < 0 || (n > 0 && (!X || !out))) return MCB_ERR_ARG;
    if (n == 0) return MCB_OK;
    MlpImpl &M = h->impl;
    if (int rc = mlp_ensure(&M, n)) return rc;
    cudaMemcpy(M.dX, X, (size_t)n * M.D.d * sizeof(float), cudaMemcpyHostToDevice);
    mlp_forward_device(&M, M.dX, n, M.dOut, 0);
    return cudaMemcpy(out, M.dOut, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? MCB_OK
                                                                                                    : MCB_ERR_CUDA;
}

int mcb_mlp_gradient(mcb_mlp *h, const float *X, const float *Y, int n, float *grad, float *loss) {
    if (!h || n < 1 || !X || !Y) return MCB_ERR_ARG;
    MlpImpl &M = h->impl;
    if (int rc = mlp_ensure(&M, n)) return rc;
    cudaMemcpy(M.dX, X, (size_t)n * M.D.d * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(M.dY, Y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    if (int rc = mlp_step_device(&M, M.dX, M.dY, nullptr, n, 0.0f, 0)) return rc;
    if (grad) cudaMemcpy(grad, M.gout, M.D.P() * sizeof(float), cudaMemcpyDeviceToHost);
    if (loss) cudaMemcpy(loss, M.loss, sizeof(float), cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

int mcb_mlp_train(mcb_mlp *h, const float *X, const float *Y, int n, int epochs, int batch, float lr, uint64_t seed,
                  float *final_loss) {
    if (!h || n < 1 || !X || !Y || epochs < 0 || batch < 1 || !(lr > 0.0f)) return MCB_ERR_ARG;
    MlpImpl &M = h->impl;
    if (int rc = mlp_ensure(&M, n)) return rc;
    cudaMemcpy(M.dX, X, (size_t)n * M.D.d * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(M.dY, Y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
    std::vector<int> perm(n);
    for (int e = 0; e < epochs; ++e) {
        // Fisher-Yates shuffle from a counter stream keyed by (seed, epoch)
        for (int i = 0; i < n; ++i) perm[i] = i;
        Stream rs{key2(seed, (uint64_t)e), 0};
        for (int i = n - 1; i > 0; --i) std::swap(perm[i], perm[rs.next() % (uint64_t)(i + 1)]);
        cudaMemcpy(M.dIdx, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        for (int b0 = 0; b0 < n; b0 += batch) {
            int nb = std::min(batch, n - b0);
            if (int rc = mlp_step_device(&M, M.dX, M.dY, M.dIdx + b0, nb, lr, 0)) return rc;
        }
    }
    if (final_loss) {
        // loss over the whole set with the trained parameters
        if (int rc = mlp_step_device(&M, M.dX, M.dY, nullptr, n, 0.0f, 0)) return rc;
        cudaMemcpy(final_loss, M.loss, sizeof(float), cudaMemcpyDeviceToHost);
    }
    return cudaDeviceSynchronize() == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

}  // extern "C"
