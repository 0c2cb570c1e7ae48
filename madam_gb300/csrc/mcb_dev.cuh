// mcb_dev.cuh -- device-side types and helpers shared by the sm_103a kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcb {

constexpr int kNmax = 1024;
constexpr double kBig = 1e9;        // BIG_NUMBER, admm.h:31
constexpr double kSaZero = 1e-11;   // |delta| below this is exactly zero in the SA

// One node being bounded ("slot").  All matrices are n x n column-major with
// leading dimension n, inside per-slot regions of Nmax*Nmax doubles.
struct Slot {
    const double *SL;  // the node's problem: SP->L (N x N, column-major) on the device
    int N;        // the problem's order (the original variables plus the fixed last one)
    int tri_k;    // triangle budget of the separation (TriIneq, twice that when the learned scorer ranks)
    int n;        // subproblem size
    int m;        // number of cuts (all families)
    int active;   // take part in the current launch
    int M;        // positive eigenvalues of the last projection
    double sigma; // ADMM penalty
    double tol;   // ADMM stopping tolerance
    int nbit;     // ADMM iteration counter of the current call
    int stop;     // ADMM finished (err < tol or itermax)
    int status;   // 0 or an error code set by a kernel (iteration cap, capacity)
    int cg_iters; // CG iterations of the last solve
    double normL; // ||L||_F (lower-triangle form, as dlansy 'F' 'L')
    double f;     // bound value of the last safe-bound evaluation
    double lmax;  // largest eigenvalue of the last safe-bound matrix
    // n x n
    double *L, *X, *Q, *W, *A, *V, *T1, *T2;
    // n-vectors
    double *y, *d, *e, *tau, *ev, *vtmp, *dy, *dy1;
    // cut data (m entries)
    int *cp;      // 8 ints per cut: k | (signmask << 8), p0..p6
    double *t, *s, *u, *v, *rhs, *cgr, *cgp, *cgq;
    // (B B^T + I) in CSR
    int *g_rp, *g_ci;
    double *g_v;
    float *g_v32;  // the values in FP32 (the inner CG)
    // B^T incidence: ne distinct lower elements e_idx[q] = i + j n (i > j), each with
    // the list e_rp[q]..e_rp[q+1] of (cut, coefficient) in cut order
    int ne;
    int *e_idx, *e_rp, *e_cut;
    double *e_coef;
    // reductions (per-slot accumulators, written by fixed-order reductions)
    double *acc;  // kAcc slots
    int *iwork;   // integer scratch
    double *dwork;// double scratch
};

// indices into Slot::acc
enum Acc {
    ACC_DUAL_T = 0,   // sum t
    ACC_SMT2,         // ||s - t||^2
    ACC_DRES2,        // ||X+ - X_old/sigma||_F^2 (lower form)
    ACC_PRIMAL,       // <L, X> (lower form)
    ACC_DIAG2,        // ||diag(X) - 1||^2
    ACC_BX2,          // ||(B(X) - 1)_+||^2
    ACC_SUMY,         // sum y
    ACC_SUMS,         // sum s
    ACC_ERR_P, ACC_ERR_D, ACC_GAP, ACC_ERR,
    ACC_LMAX_HI,      // upper end of the bisection bracket of lambda_max
    ACC_FNORM,        // ||A||_F of the safe-bound matrix
    ACC_SIGMA_LAST,   // sigma of the last ADMM iteration (scales the heuristic's factor)
    // IPM state (ipm_mc_pk.c)
    ACC_MU, ACC_PHI, ACC_PSI, ACC_AP, ACC_AD, ACC_IPM_IT, ACC_IPM_DONE, ACC_IPM_INFO,
    // Newton-Schulz projection: scale of W and trace of sign(W)
    ACC_NS_ALPHA, ACC_NS_TRACE,
    kAcc = 32
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum, result broadcast to all threads.  `red` needs 33 doubles of
// shared memory.  Deterministic for a fixed block size.
__device__ __forceinline__ double block_sum(double v, double *red) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        double x = lane < nw ? red[lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}
__device__ __forceinline__ double block_max(double v, double *red) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        double x = lane < nw ? red[lane] : -1e308;
        x = warp_max(x);
        if (lane == 0) red[32] = x;
    }
    __syncthreads();
    return red[32];
}

// splitmix64 finaliser and the counter streams shared with the host code
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t key2(uint64_t a, uint64_t b) {
    return mix64(a ^ mix64(b + 0x632BE59BD9B4E019ull));
}
struct Stream {
    uint64_t key, ctr;
    __host__ __device__ __forceinline__ uint64_t next() {
        ctr += 1;
        return mix64(key + ctr * 0x9E3779B97F4A7C15ull);
    }
    __host__ __device__ __forceinline__ int next_int() { return (int)(next() >> 33); }
    __host__ __device__ __forceinline__ double next_unit() { return (double)(next() >> 11) * 0x1.0p-53; }
};

// cut encoding: cp[0] = k | (signmask << 8); bit a of signmask set <=> e_a = -1
__host__ __device__ __forceinline__ int cut_k(int h) { return h & 0xff; }
__host__ __device__ __forceinline__ int cut_sign(int h, int a) { return ((h >> (8 + a)) & 1) ? -1 : 1; }
__host__ __device__ __forceinline__ double cut_scale(int k) {
    return k == 3 ? 1.0 : (k == 5 ? 0.5 : 1.0 / 3.0);
}

// inverse iteration (k_invit): threads per slot, one per cluster of eigenvalues
// at a time, and their workspace of 6 n doubles each
constexpr int kInvThreads = 128;
constexpr size_t eig_dwork_doubles_max(int n) { return (size_t)6 * kInvThreads * (size_t)n; }

// a slot takes part in a launch: active, and (when gated) its ADMM has not stopped
__device__ __forceinline__ bool gated(const Slot &s, int gate) { return s.active && !(gate && s.stop); }

// lower-triangle read of a full-storage matrix
__device__ __forceinline__ double lowr(const double *X, int n, int a, int b) {
    return a > b ? X[a + (size_t)b * n] : X[b + (size_t)a * n];
}

}  // namespace mcb
