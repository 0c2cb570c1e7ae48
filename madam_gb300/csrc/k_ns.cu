// k_ns.cu -- kernels and host orchestration of the Newton-Schulz PSD projection
// (the chosen form, see ns.h) and of the GPU hyperplane rounding used by its
// heuristic.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/mcbound.h"
#include "mcb_dev.cuh"
#include "ns.h"
#include "tc.h"

namespace mcb {

namespace {
constexpr int TT = 32;  // tile edge of the copy kernels

// ||W||_F from the lower triangle (an upper bound on the spectral radius)
__global__ void __launch_bounds__(512) k_ns_alpha(Slot *slots, double *alpha_out, int gate) {
    Slot &s = slots[blockIdx.x];
    if (!gated(s, gate)) return;
    const int n = s.n;
    __shared__ double red[40];
    double a = 0.0;
    for (int j = threadIdx.x >> 5; j < n; j += blockDim.x >> 5) {
        const double *col = s.W + (size_t)j * n;
        for (int i = j + (threadIdx.x & 31); i < n; i += 32) {
            double w = col[i];
            a += (i == j ? 1.0 : 2.0) * w * w;
        }
    }
    a = block_sum(a, red);
    if (threadIdx.x == 0) {
        s.acc[ACC_NS_ALPHA] = sqrt(a);
        if (alpha_out) alpha_out[blockIdx.x] = sqrt(a);
    }
}

// Wd = W (full, FP64, padded to npad with zeros), S = W / alpha (FP32).
// W holds the lower triangle; upper tiles are read through their mirror and
// transposed in shared memory so that both reads and writes are coalesced.
__global__ void __launch_bounds__(256) k_ns_scale(Slot *slots, int npad, size_t stride, float *S, double *Wd,
                                                  int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const int n = s.n, nt = (npad + TT - 1) / TT;
    const int ti = blockIdx.x % nt, tj = blockIdx.x / nt;
    if (tj >= nt) return;
    const int I = ti >= tj ? ti : tj, J = ti >= tj ? tj : ti;
    __shared__ double sh[TT][TT + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int c = ty; c < TT; c += 8) {
        int r = I * TT + tx, q = J * TT + c;
        sh[c][tx] = (r < n && q < n) ? s.W[r + (size_t)q * n] : 0.0;
    }
    __syncthreads();
    const double alpha = s.acc[ACC_NS_ALPHA];
    const double inv = alpha > 0.0 ? 1.0 / alpha : 0.0;
    float *Sb = S + (size_t)blockIdx.y * stride;
    double *Wb = Wd + (size_t)blockIdx.y * stride;
    for (int c = ty; c < TT; c += 8) {
        int i = ti * TT + tx, j = tj * TT + c;
        if (i >= npad || j >= npad) continue;
        double v;
        if (ti > tj) v = sh[c][tx];
        else if (ti < tj) v = sh[tx][c];
        else v = tx >= c ? sh[c][tx] : sh[tx][c];
        if (i >= n || j >= n) v = 0.0;
        size_t o = i + (size_t)j * npad;
        Wb[o] = v;
        Sb[o] = (float)(v * inv);
    }
}

__global__ void k_ns_diag(Slot *slots, int npad, size_t stride, float *T, float a, int gate) {
    Slot &s = slots[blockIdx.x];
    if (!gated(s, gate)) return;
    float *Tb = T + (size_t)blockIdx.x * stride;
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) Tb[i + (size_t)i * npad] += a;
}

// Sd = S in FP64; M = number of positive eigenvalues = (n + trace S) / 2 rounded
__global__ void __launch_bounds__(256) k_ns_finish(Slot *slots, int npad, size_t stride, const float *S, double *Sd,
                                                   int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const float *Sb = S + (size_t)blockIdx.y * stride;
    double *Db = Sd ? Sd + (size_t)blockIdx.y * stride : nullptr;
    const size_t tot = (size_t)npad * npad;
    if (Sd)
        for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x)
            Db[q] = (double)Sb[q];
    if (blockIdx.x == 0) {
        __shared__ double red[40];
        double t = 0.0;
        for (int i = threadIdx.x; i < s.n; i += blockDim.x) t += (double)Sb[i + (size_t)i * npad];
        t = block_sum(t, red);
        if (threadIdx.x == 0) {
            s.acc[ACC_NS_TRACE] = t;
            int M = (int)llrint(0.5 * ((double)s.n + t));
            s.M = M < 0 ? 0 : (M > s.n ? s.n : M);
        }
    }
}

// --- heuristic: hyperplane signs of X v -------------------------------------
__global__ void __launch_bounds__(256) k_heur_xf(Slot *slots, const int *list, int npad, size_t stride, float *Xf) {
    const int si = list[blockIdx.y];
    Slot &s = slots[si];
    const int n = s.n;
    float *Xb = Xf + (size_t)si * stride;
    const size_t tot = (size_t)npad * npad;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(q / npad), i = (int)(q - (size_t)j * npad);
        Xb[q] = (i < n && j < n) ? (float)s.X[i + (size_t)j * n] : 0.0f;
    }
}

// V[:, c] = the n draws (uniform in [-0.5, 0.5)) of stream key2(key, c): draw i of a
// counter stream is mix64(key + (i + 1) * golden), see Stream::next; columns
// count .. rows - 1 are zero
__global__ void __launch_bounds__(256) k_heur_vec(Slot *slots, const int *list, const unsigned long long *keys,
                                                  int count, int rows, int npad, size_t stride, float *V) {
    const int si = list[blockIdx.y];
    const int n = slots[si].n;
    const uint64_t key = keys[blockIdx.y];
    float *Vb = V + (size_t)si * stride;
    const size_t tot = (size_t)npad * rows;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        int c = (int)(q / npad), i = (int)(q - (size_t)c * npad);
        float v = 0.0f;
        if (i < n && c < count) {
            uint64_t kc = key2(key, (uint64_t)c);
            uint64_t z = mix64(kc + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
            v = (float)((double)(z >> 11) * 0x1.0p-53 - 0.5);
        }
        Vb[q] = v;
    }
}

__global__ void __launch_bounds__(256) k_heur_sign(Slot *slots, const int *list, int count, int npad, size_t stride,
                                                   const float *H, unsigned char *out, size_t out_stride) {
    const int si = list[blockIdx.y];
    const int n = slots[si].n;
    const float *Hb = H + (size_t)si * stride;
    unsigned char *ob = out + (size_t)blockIdx.y * out_stride;
    const size_t tot = (size_t)n * count;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        int c = (int)(q / n), i = (int)(q - (size_t)c * n);
        ob[q] = Hb[i + (size_t)c * npad] < 0.0f ? 1 : 0;
    }
}

// One warp per (listed slot, hyperplane): the 1-opt local search of mc_1opt
// (heuristic.c) from the hyperplane's signs on the subproblem matrix L, then the
// cut value sol^T SL sol of the full 0/1 solution over the original variables
// (fixed ones from the node).  L and SL hold quarter-integers, so every FP64 sum
// here is exact and independent of order.  Lane l owns elements l + 32 j.
// signs: n bytes per hyperplane (1 = -1), overwritten with the 1-opt result;
// hval[q * count + h] = the cut value.
__global__ void __launch_bounds__(128) k_heur_1opt(const Slot *slots, const int *list, int count, const int *lists,
                                                   int list_stride, unsigned char *signs, size_t sstride,
                                                   double *hval) {
    constexpr int PER = kNmax / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int h = blockIdx.x * 4 + warp;
    const int q = blockIdx.y;
    __shared__ unsigned words[4][PER];
    if (h >= count) return;
    const int si = list[q];
    const Slot &s = slots[si];
    // the node's problem: P0->n hyperplanes (heuristic.c:24-91) of its own order N
    const int N = s.N;
    const double *SL = s.SL;
    if (h >= N) {
        if (lane == 0) hval[(size_t)q * count + h] = -kBig;
        return;
    }
    const int n = s.n;
    const double *L = s.L;
    unsigned char *sg = signs + (size_t)q * sstride + (size_t)h * n;
    unsigned xneg = 0;
    for (int j = 0; j < PER; ++j) {
        const int i = lane + 32 * j;
        if (i < n && sg[i]) xneg |= 1u << j;
    }
    for (int j = 0; j < PER; ++j) {
        unsigned w = __ballot_sync(0xffffffffu, (xneg >> j) & 1u);
        if (lane == 0) words[warp][j] = w;
    }
    __syncwarp();
    double lx[PER], dg[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) { lx[j] = 0.0; dg[j] = 0.0; }
    for (int k = 0; k < n; ++k) {
        const double xk = (words[warp][k >> 5] >> (k & 31)) & 1u ? -1.0 : 1.0;
        const double *col = L + (size_t)k * n;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int i = lane + 32 * j;
            if (i < n) lx[j] += col[i] * xk;
        }
    }
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const int i = lane + 32 * j;
        if (i < n) dg[j] = L[i + (size_t)i * n];
    }
    // flip the element of largest gain (first on ties) while the gain exceeds 0.001
    for (int it = 0; it < 16 * n + 64; ++it) {
        double best = -kBig;
        int idx = 0x7fffffff;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int i = lane + 32 * j;
            if (i >= n) continue;
            const double xi = (xneg >> j) & 1u ? -1.0 : 1.0;
            const double dl = dg[j] - xi * lx[j];
            if (dl > best) { best = dl; idx = i; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double ob = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, idx, o);
            if (ob > best || (ob == best && oi < idx)) { best = ob; idx = oi; }
        }
        if (!(best > 0.001)) break;
        const int ol = idx & 31, oj = idx >> 5;
        const unsigned on = __shfl_sync(0xffffffffu, xneg, ol);
        const double sgn = ((on >> oj) & 1u) ? 2.0 : -2.0;  // x = +1: Lx -= 2 L(idx, .), else +=
        const double *col = L + (size_t)idx * n;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int i = lane + 32 * j;
            if (i < n) {
                const double l = col[i];
                if (fabs(l) > 0.001) lx[j] += sgn * l;
            }
        }
        if (lane == ol) xneg ^= 1u << oj;
    }
    for (int j = 0; j < PER; ++j) {
        const int i = lane + 32 * j;
        if (i < n) sg[i] = (xneg >> j) & 1u;
    }
    // the full solution: free variables U[u] from element u, fixed ones from the node
    const int *ls = lists + (size_t)si * list_stride;
    const int nu = ls[0], nf1 = ls[1], nfx = ls[2];
    const int *U = ls + 3, *FX = U + nu + nf1, *FS = FX + nfx;
    __syncwarp();
    for (int j = lane; j < PER; j += 32) words[warp][j] = 0u;
    __syncwarp();
    for (int j = 0; j < PER; ++j) {
        const int u = lane + 32 * j;
        if (u < nu && !((xneg >> j) & 1u)) atomicOr(&words[warp][U[u] >> 5], 1u << (U[u] & 31));
    }
    for (int f = lane; f < nfx; f += 32)
        if (FS[f]) atomicOr(&words[warp][FX[f] >> 5], 1u << (FX[f] & 31));
    __syncwarp();
    const int pb = N - 1;
    double v = 0.0;
    for (int i = 0; i < pb; ++i) {
        if (!((words[warp][i >> 5] >> (i & 31)) & 1u)) continue;
        const double *row = SL + (size_t)i * N;
        for (int j = lane; j < pb; j += 32)
            if ((words[warp][j >> 5] >> (j & 31)) & 1u) v += row[j];
    }
    v = warp_sum(v);
    if (lane == 0) hval[(size_t)q * count + h] = v;
}

inline int cdiv(size_t a, int b) { return (int)((a + b - 1) / b); }
inline int grid_for(size_t tot) {
    int g = cdiv(tot, 256);
    return g < 1 ? 1 : (g > 1184 ? 1184 : g);
}

}  // namespace

void launch_ns_prep(Slot *d, int ns, int npad, size_t stride, float *S, double *Wd, double *alpha_out, int gate,
                    cudaStream_t st) {
    k_ns_alpha<<<ns, 512, 0, st>>>(d, alpha_out, gate);
    int nt = (npad + TT - 1) / TT;
    k_ns_scale<<<dim3(nt * nt, ns), 256, 0, st>>>(d, npad, stride, S, Wd, gate);
}
void launch_ns_diag(Slot *d, int ns, int npad, size_t stride, float *T, float a, int gate, cudaStream_t st) {
    (void)npad;
    k_ns_diag<<<ns, 256, 0, st>>>(d, npad, stride, T, a, gate);
}
void launch_ns_finish(Slot *d, int ns, int npad, size_t stride, const float *S, double *Sd, int gate,
                      cudaStream_t st) {
    int g = grid_for((size_t)npad * npad);
    g = g > 64 ? 64 : g;
    k_ns_finish<<<dim3(g, ns), 256, 0, st>>>(d, npad, stride, S, Sd, gate);
}
void launch_heur_xf(Slot *d, const int *slots, int nslots, int npad, size_t stride, float *Xf, cudaStream_t st) {
    int g = grid_for((size_t)npad * npad);
    g = g > 64 ? 64 : g;
    k_heur_xf<<<dim3(g, nslots), 256, 0, st>>>(d, slots, npad, stride, Xf);
}
void launch_heur_vectors(Slot *d, const int *slots, const unsigned long long *keys, int nslots, int count, int rows,
                         int npad, size_t stride, float *V, cudaStream_t st) {
    int g = grid_for((size_t)npad * rows);
    g = g > 64 ? 64 : g;
    k_heur_vec<<<dim3(g, nslots), 256, 0, st>>>(d, slots, keys, count, rows, npad, stride, V);
}
void launch_heur_1opt(const Slot *d, const int *slots, int nslots, int count, const int *lists, int list_stride,
                      unsigned char *signs, size_t sstride, double *hval, cudaStream_t st) {
    k_heur_1opt<<<dim3((count + 3) / 4, nslots), 128, 0, st>>>(d, slots, count, lists, list_stride, signs, sstride,
                                                                hval);
}
void launch_heur_signs(Slot *d, const int *slots, int nslots, int count, int npad, size_t stride, const float *H,
                       unsigned char *out, size_t out_stride, cudaStream_t st) {
    int g = grid_for((size_t)npad * count);
    g = g > 64 ? 64 : g;
    k_heur_sign<<<dim3(g, nslots), 256, 0, st>>>(d, slots, count, npad, stride, H, out, out_stride);
}

// --- schedule and host orchestration ---------------------------------------
std::vector<NsStep> ns_schedule(double l0, double safety, double eps) {
    std::vector<NsStep> st;
    double l = l0;
    auto p = [](double y) { return 1.5 * y - 0.5 * y * y * y; };
    while (1.0 - l > eps && st.size() < 64) {
        double k2 = 3.0 * (1.0 - safety) / (1.0 + l + l * l);
        double k = k2 > 1.0 ? sqrt(k2) : 1.0;
        NsStep s;
        s.a = (float)(1.5 * k);
        s.b = (float)(-0.5 * k * k * k);
        s.accurate = l > 0.9;
        double nl = p(k * l) < p(k) ? p(k * l) : p(k);
        st.push_back(s);
        l = nl;
    }
    // at least two accurate steps: they remove the low-precision rounding
    int acc = 0;
    for (auto &s : st) acc += s.accurate;
    while (acc < 2) {
        st.push_back({1.5f, -0.5f, 1});
        ++acc;
    }
    return st;
}

}  // namespace mcb

// the step schedule for a given l0 (host arithmetic only; no device needed)
extern "C" int mcb_ns_schedule_for(double l0, int cap, float *a, float *b, int *accurate) {
    if (!(l0 > 0.0 && l0 < 0.5)) return MCB_ERR_ARG;
    std::vector<mcb::NsStep> st = mcb::ns_schedule(l0, 0.02, 1e-7);
    for (int k = 0; k < (int)st.size() && k < cap; ++k) {
        if (a) a[k] = st[k].a;
        if (b) b[k] = st[k].b;
        if (accurate) accurate[k] = st[k].accurate;
    }
    return (int)st.size();
}

namespace mcb {

int NsProj::init(int form_, int nmax_, int cap_, cudaStream_t st) {
    form = form_;
    nmax = nmax_;
    cap = cap_;
    int np = (nmax + 127) / 128 * 128;
    stride = (size_t)np * np;
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) return MCB_ERR_CUDA;
    cublasSetStream(h, st);
    const size_t tot = stride * (size_t)cap;
    if (cudaMalloc(&S, tot * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&S2, tot * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&T, tot * sizeof(float)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&Wd, tot * sizeof(double)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&Sd, tot * sizeof(double)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&Gd, tot * sizeof(double)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&dptr, 6 * (size_t)cap * sizeof(void *)) != cudaSuccess) return MCB_ERR_NOMEM;
    hptr.assign(6 * (size_t)cap, nullptr);
    for (__nv_bfloat16 **b : {&Wp, &Sp, &S2p, &Tp})
        if (cudaMalloc(b, kTcPieces * tot * sizeof(__nv_bfloat16)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&d_alpha, cap * sizeof(double)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&d_live, cap * sizeof(int)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&d_n, cap * sizeof(int)) != cudaSuccess) return MCB_ERR_NOMEM;
    if (cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) return MCB_ERR_NOMEM;
    cudaMemset(d_err, 0, sizeof(int));
    maps_store.assign(4 * kTcPieces * 128 + 64, 0);
    maps = (unsigned char *)(((uintptr_t)maps_store.data() + 63) & ~(uintptr_t)63);
    steps = ns_schedule(l0, 0.02, 1e-7);
    return MCB_OK;
}

int NsProj::configure(int operands_, double l0_) {
    if (operands_ < MCB_NS_OPERANDS_NATIVE || operands_ > MCB_NS_OPERANDS_CUBLAS_SPLIT || !(l0_ > 0.0 && l0_ < 0.5))
        return MCB_ERR_ARG;
    operands = operands_;
    l0 = l0_;
    steps = ns_schedule(l0, 0.02, 1e-7);
    ++version;
    return MCB_OK;
}

void NsProj::destroy() {
    void *ps[] = {S, S2, T, Wd, Sd, Gd, dptr, Sp, S2p, Tp, Wp, d_live, d_n, d_err, d_alpha};
    for (void *p : ps)
        if (p) cudaFree(p);
    S = S2 = T = nullptr;
    Sp = S2p = Tp = Wp = nullptr;
    d_live = d_n = d_err = nullptr;
    d_alpha = nullptr;
    Wd = Sd = Gd = nullptr;
    dptr = nullptr;
    if (h) cublasDestroy(h);
    h = nullptr;
}

int NsProj::set_live(const std::vector<int> &slots, const std::vector<int> &ns, int npad_, cudaStream_t st) {
    live = (int)slots.size();
    npad = npad_;
    if (tc()) {
        if (npad % kTcTile) return MCB_ERR_ARG;
        if (live) {
            if (cudaMemcpyAsync(d_live, slots.data(), live * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess)
                return MCB_ERR_CUDA;
            if (cudaMemcpyAsync(d_n, ns.data(), live * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess)
                return MCB_ERR_CUDA;
        }
        if (map_npad != npad) {
            __nv_bfloat16 *bufs[4] = {Wp, Sp, S2p, Tp};
            const size_t tot = stride * (size_t)cap;
            for (int b = 0; b < 4; ++b)
                for (int p = 0; p < kTcPieces; ++p)
                    if (int rc = tc_make_map(maps + (kTcPieces * b + p) * 128, bufs[b] + p * tot, npad, stride, cap))
                        return rc;
            map_npad = npad;
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) return MCB_ERR_CUDA;
        if (live) {
            auto it = tuned.find({npad, bucket(live)});
            if (it == tuned.end()) return tune(st);
            variant = it->second.variant;
        }
        return MCB_OK;
    }
    for (int k = 0; k < live; ++k) {
        size_t o = slot_offset(slots[k]);
        hptr[0 * cap + k] = S + o;
        hptr[1 * cap + k] = S2 + o;
        hptr[2 * cap + k] = T + o;
        hptr[3 * cap + k] = Wd + o;
        hptr[4 * cap + k] = Sd + o;
        hptr[5 * cap + k] = Gd + o;
    }
    if (cudaMemcpyAsync(dptr, hptr.data(), 6 * (size_t)cap * sizeof(void *), cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
        return MCB_ERR_CUDA;
    // the staging vector is rewritten by the next call only: wait for the copy
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCB_ERR_CUDA;
    return MCB_OK;
}

namespace {
cublasStatus_t gemm32(cublasHandle_t h, int np, float alpha, void **A, void **B, float beta, void **C, int batch,
                      cublasComputeType_t ct) {
    return cublasGemmBatchedEx(h, CUBLAS_OP_N, CUBLAS_OP_N, np, np, np, &alpha, (const void *const *)A, CUDA_R_32F,
                               np, (const void *const *)B, CUDA_R_32F, np, &beta, (void *const *)C, CUDA_R_32F, np,
                               batch, ct, CUBLAS_GEMM_DEFAULT);
}
}  // namespace

namespace {
// plane scales of the tcgen05 path: S and S0 have |entries| <= ||S||_2 <= 1, so
// sigma = 2 (leading digits <= 64); T = a I + b S^2 has eigenvalues in [a + b, a]
// with a <= 1.5 sqrt(3) (the schedule's k^2 <= 3), so sigma = 4 (leading digits
// <= 83).  With digits that small the exact digit-sum groups of every product
// stay below 2^24 for K <= 1024.  The planes hold q = x 2^7 / sigma.
constexpr float kPscaleS = 64.0f, kPscaleT = 32.0f;
constexpr float kUnitSS = 1.0f / 4096.0f;  // sigma_S^2 2^-14
constexpr float kUnitST = 1.0f / 2048.0f;  // sigma_S sigma_T 2^-14
// the planes of one plane set (S0, S, S2 or T), tot elements apart
TcOut planes_out(__nv_bfloat16 *base, size_t tot, size_t stride, int *err, float pscale, float *f32 = nullptr) {
    TcOut o{f32, nullptr, {}, stride, err, pscale, nullptr};
    for (int p = 0; p < kTcPieces; ++p) o.p[p] = base + p * tot;
    return o;
}
}  // namespace

int NsProj::tune(cudaStream_t st) {
    const size_t tot = stride * (size_t)cap;
    TcOut ot = planes_out(Tp, tot, stride, d_err, kPscaleT);
    Tuned t{0, {0.0f, 0.0f}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = MCB_OK;
    // each variant: one launch to warm up, then rounds of kTuneLaunches launches queued
    // back to back between two events (the launches keep the GPU busy, so the time
    // is the kernels', not the host's submission), best round
    constexpr int kTuneLaunches = 8;
    for (int v = 0; v < kTcVariants && rc == MCB_OK; ++v) {
        rc = tc_gemm(maps, maps, ot, npad, live, d_live, d_n, 1.0f, 0.0f, kUnitSS, st, 1, v);
        float best = 1e30f;
        for (int rep = 0; rep < 3 && rc == MCB_OK; ++rep) {
            cudaEventRecord(e0, st);
            for (int k = 0; k < kTuneLaunches && rc == MCB_OK; ++k)
                rc = tc_gemm(maps, maps, ot, npad, live, d_live, d_n, 1.0f, 0.0f, kUnitSS, st, 1, v);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = MCB_ERR_CUDA;
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        t.us[v] = best * 1e3f / kTuneLaunches;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MCB_OK) return rc;
    t.variant = t.us[1] < t.us[0] ? 1 : 0;
    tuned[{npad, bucket(live)}] = t;
    variant = t.variant;
    return check_error(st);
}

int NsProj::check_error(cudaStream_t st) {
    if (!d_err) return MCB_OK;
    int e = 0;
    if (cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return MCB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCB_ERR_CUDA;
    if (e) cudaMemsetAsync(d_err, 0, sizeof(int), st);
    return e ? MCB_ERR_ITER : MCB_OK;
}

void NsProj::split_inputs(cudaStream_t st) {
    const size_t tot = stride * (size_t)cap;
    tc_split_f64(Wd, stride, planes_out(Wp, tot, stride, nullptr, kPscaleS), npad, live, d_live, d_alpha, st);
}

int NsProj::sign(Slot *d_slots, int ns, int gate, cudaStream_t st) {
    if (live == 0) return MCB_OK;
    if (tc()) {
        const size_t tot = stride * (size_t)cap;
        __nv_bfloat16 *bufs[4] = {Wp, Sp, S2p, Tp};
        auto mp = [&](int b) { return maps + kTcPieces * b * 128; };
        int c = 0, nx = 1;  // start from S0 (never overwritten: G needs it), then S and S2 in turn
        const double g = 2.0 * (double)npad * npad * npad * live;
        for (size_t i = 0; i < steps.size(); ++i) {
            const NsStep &stp = steps[i];
            // T = b S^2 + a I (planes), then S' = S T (planes; FP32 after the last step)
            TcOut ot = planes_out(Tp, tot, stride, d_err, kPscaleT);
            if (int rc = tc_gemm(mp(c), mp(c), ot, npad, live, d_live, d_n, stp.b, stp.a, kUnitSS, st, 1, variant))
                return rc;
            TcOut os = planes_out(bufs[nx], tot, stride, d_err, kPscaleS, i + 1 == steps.size() ? S : nullptr);
            if (int rc = tc_gemm(mp(c), mp(3), os, npad, live, d_live, d_n, 1.0f, 0.0f, kUnitST, st, 1, variant))
                return rc;
            flops_hi += 2.0 * g;  // algorithmic: two n^3 products per step (the mirror halves the MMAs)
            c = nx;
            nx = nx == 1 ? 2 : 1;
        }
        cur = c;
        launch_ns_finish(d_slots, ns, npad, stride, S, nullptr, gate, st);
        return MCB_OK;
    }
    cublasSetStream(h, st);
    void **pS = dptr, **pS2 = dptr + cap, **pT = dptr + 2 * cap;
    // cuBLAS forms: growth steps in one pass of the form's type (NATIVE), its
    // FP32-accurate split (CUBLAS_SPLIT: cuBLAS's three-piece BF16 emulation), or
    // FP32 FMA (FP32); the closing steps always FP32-accurate
    const cublasComputeType_t split = CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    cublasComputeType_t lo = form == MCB_PROJ_NS_TF32 ? CUBLAS_COMPUTE_32F_FAST_TF32 : CUBLAS_COMPUTE_32F_FAST_16BF;
    if (operands == MCB_NS_OPERANDS_CUBLAS_SPLIT) lo = split;
    if (operands == MCB_NS_OPERANDS_FP32) lo = CUBLAS_COMPUTE_32F;
    const cublasComputeType_t hi = operands == MCB_NS_OPERANDS_FP32 ? CUBLAS_COMPUTE_32F : split;
    float *cur = S, *nxt = S2;
    void **pc = pS, **pn = pS2;
    const double g = 2.0 * (double)npad * npad * npad * live;
    for (const NsStep &stp : steps) {
        cublasComputeType_t ct = stp.accurate ? hi : lo;
        // T = b S^2 + a I, then S' = S T
        if (gemm32(h, npad, stp.b, pc, pc, 0.0f, pT, live, ct) != CUBLAS_STATUS_SUCCESS) return MCB_ERR_CUDA;
        launch_ns_diag(d_slots, ns, npad, stride, T, stp.a, gate, st);
        if (gemm32(h, npad, 1.0f, pc, pT, 0.0f, pn, live, ct) != CUBLAS_STATUS_SUCCESS) return MCB_ERR_CUDA;
        (stp.accurate ? flops_hi : flops_lo) += 2.0 * g;
        float *t = cur; cur = nxt; nxt = t;
        void **tp = pc; pc = pn; pn = tp;
    }
    launch_ns_finish(d_slots, ns, npad, stride, cur, Sd, gate, st);
    return MCB_OK;
}

int NsProj::product(cudaStream_t st) {
    if (live == 0) return MCB_OK;
    if (tc()) {
        // G = W S = alpha (S0 S): the planes of S0 and of the final S, alpha per slot
        TcOut og{nullptr, Gd, {}, stride, d_err, 1.0f, d_alpha};
        int rc = tc_gemm(maps, maps + kTcPieces * cur * 128, og, npad, live, d_live, d_n, 1.0f, 0.0f, kUnitSS, st, 1,
                         variant);
        flops_hi += 2.0 * (double)npad * npad * npad * live;
        return rc;
    }
    cublasSetStream(h, st);
    void **pW = dptr + 3 * cap, **pSd = dptr + 4 * cap, **pG = dptr + 5 * cap;
    const double one = 1.0, zero = 0.0;
    if (cublasGemmBatchedEx(h, CUBLAS_OP_N, CUBLAS_OP_N, npad, npad, npad, &one, (const void *const *)pW, CUDA_R_64F,
                            npad, (const void *const *)pSd, CUDA_R_64F, npad, &zero, (void *const *)pG, CUDA_R_64F,
                            npad, live, CUBLAS_COMPUTE_64F, CUBLAS_GEMM_DEFAULT) != CUBLAS_STATUS_SUCCESS)
        return MCB_ERR_CUDA;
    flops_fp64 += 2.0 * (double)npad * npad * npad * live;
    return MCB_OK;
}

int NsProj::hyperplanes(Slot *d_slots, const std::vector<int> &slots, const int *d_list,
                        const unsigned long long *d_keys, int count, int npad_, unsigned char *d_out, size_t out_stride,
                        cudaStream_t st) {
    const int k = (int)slots.size();
    if (k == 0) return MCB_OK;
    for (int q = 0; q < k; ++q) {
        size_t o = slot_offset(slots[q]);
        hptr[0 * cap + q] = S + o;   // X in FP32
        hptr[1 * cap + q] = T + o;   // hyperplane normals
        hptr[2 * cap + q] = S2 + o;  // X V
    }
    if (tc()) {
        // H = V X on the library's tcgen05 kernel: the normals (rows of V, zero rows
        // past `count`) and X as digit planes in the projection's plane buffers,
        // both padded to a multiple of 128 that holds the subproblem and the count
        const int np2 = (std::max(npad_, count) + 127) / 128 * 128;
        const size_t tot = stride * (size_t)cap;
        launch_heur_xf(d_slots, d_list, k, np2, stride, S, st);
        launch_heur_vectors(d_slots, d_list, d_keys, k, count, np2, np2, stride, T, st);
        // |X_ij| <= 1 for the ADMM's X (unit diagonal, PSD) up to its tolerance: sigma = 4;
        // the normals lie in [-1/2, 1/2): sigma = 1
        TcOut ox = planes_out(Sp, tot, stride, nullptr, 32.0f), ov = planes_out(Tp, tot, stride, nullptr, 128.0f);
        tc_split_f32(S, stride, ox, np2, k, d_list, st);
        tc_split_f32(T, stride, ov, np2, k, d_list, st);
        alignas(64) unsigned char hm[2 * kTcPieces][128];
        for (int p = 0; p < kTcPieces; ++p) {
            if (int rc = tc_make_map(hm[p], ov.p[p], np2, stride, cap)) return rc;
            if (int rc = tc_make_map(hm[kTcPieces + p], ox.p[p], np2, stride, cap)) return rc;
        }
        map_npad = 0;  // the projection's maps are rebuilt at its next set_live
        TcOut oh{S2, nullptr, {}, stride, d_err, 1.0f, nullptr};
        // row c of the product is X v_c (X is symmetric); no diagonal term
        if (int rc = tc_gemm(hm[0], hm[kTcPieces], oh, np2, k, d_list, d_n, 1.0f, 0.0f, 4.0f / 16384.0f, st, 0, 0))
            return rc;
        launch_heur_signs(d_slots, d_list, k, count, np2, stride, S2, d_out, out_stride, st);
        return MCB_OK;
    }
    if (cudaMemcpyAsync(dptr, hptr.data(), 3 * (size_t)cap * sizeof(void *), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return MCB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCB_ERR_CUDA;
    live = 0;  // the live-slot arrays were overwritten
    launch_heur_xf(d_slots, d_list, k, npad_, stride, S, st);
    launch_heur_vectors(d_slots, d_list, d_keys, k, count, count, npad_, stride, T, st);
    cublasSetStream(h, st);
    const float one = 1.0f, zero = 0.0f;
    if (cublasGemmBatchedEx(h, CUBLAS_OP_N, CUBLAS_OP_N, npad_, count, npad_, &one, (const void *const *)dptr,
                            CUDA_R_32F, npad_, (const void *const *)(dptr + cap), CUDA_R_32F, npad_, &zero,
                            (void *const *)(dptr + 2 * cap), CUDA_R_32F, npad_, k, CUBLAS_COMPUTE_32F_FAST_TF32,
                            CUBLAS_GEMM_DEFAULT) != CUBLAS_STATUS_SUCCESS)
        return MCB_ERR_CUDA;
    launch_heur_signs(d_slots, d_list, k, count, npad_, stride, S2, d_out, out_stride, st);
    return MCB_OK;
}

}  // namespace mcb
