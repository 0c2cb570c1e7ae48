// k_ipm.cu -- batched basic-SDP interior-point method on the GPU (FP64).
//
// Restates ipm_mc_pk.c (the Helmberg-Rendl-Vanderbei-Wolkowicz predictor-
// corrector for max <L,X> s.t. diag X = e, X psd) with one slot per node:
// Cholesky factorisations, inverses, solves and the line searches run one CTA
// per node; the two n^3 products Zi*tmp (ipm_mc_pk.c:181,249) run as a tiled
// multi-CTA FP64 GEMM.  Iterates: X (s.X), y (s.y), Z = Diag(y) - L (s.Q),
// Zi (s.W), factor of Zi o X (s.T1), dX1 (s.V), dX (s.A), scratch (s.T2).
#include "mcb_dev.cuh"
#include "kernels.h"

namespace mcb {

// Cholesky A = L L^T (lower, in place) of the n x n matrix at A with one CTA.
// Returns 0 on success or k+1 for a non-positive pivot (dpotrf's INFO).
__device__ int cta_cholesky(double *A, int n) {
    __shared__ int info;
    __shared__ double piv;
    if (threadIdx.x == 0) info = 0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            double a = A[k + (size_t)k * n];
            if (!(a > 0.0)) info = k + 1;
            piv = sqrt(a);
            A[k + (size_t)k * n] = piv;
        }
        __syncthreads();
        if (info) return info;
        double inv = 1.0 / piv;
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)k * n] *= inv;
        __syncthreads();
        const int m = n - k - 1;
        for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
            int jj = idx / m, ii = idx - jj * m;
            if (ii < jj) continue;
            int i = k + 1 + ii, j = k + 1 + jj;
            A[i + (size_t)j * n] -= A[i + (size_t)k * n] * A[j + (size_t)k * n];
        }
        __syncthreads();
    }
    return 0;
}

// b <- (L L^T)^{-1} b with the lower factor L, whole CTA (column oriented).
__device__ void cta_chol_solve(const double *Lf, int n, double *b) {
    for (int k = 0; k < n; ++k) {
        __syncthreads();
        double yk = b[k] / Lf[k + (size_t)k * n];
        __syncthreads();
        if (threadIdx.x == 0) b[k] = yk;
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) b[i] -= Lf[i + (size_t)k * n] * yk;
    }
    for (int k = n - 1; k >= 0; --k) {
        __syncthreads();
        double xk = b[k] / Lf[k + (size_t)k * n];
        __syncthreads();
        if (threadIdx.x == 0) b[k] = xk;
        for (int i = threadIdx.x; i < k; i += blockDim.x) b[i] -= Lf[k + (size_t)i * n] * xk;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Initial point, ipm_mc_pk.c:57-91
__global__ void k_ipm_init(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!s.active) return;
    const int n = s.n;
    __shared__ double red[40];
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double a = 0.0;
        for (int r = 0; r < n; ++r) a += fabs(s.L[r + (size_t)c * n]);
        s.y[c] = a + 1.1;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx / n, i = idx - j * n;
        s.X[idx] = i == j ? 1.0 : 0.0;
        s.Q[idx] = (i == j ? s.y[i] : 0.0) - s.L[idx];
    }
    __syncthreads();
    double py = 0.0, pl = 0.0, pz = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        py += s.y[i];
        pl += s.L[i + (size_t)i * n];
        pz += s.Q[i + (size_t)i * n];
    }
    py = block_sum(py, red);
    pl = block_sum(pl, red);
    pz = block_sum(pz, red);
    if (threadIdx.x == 0) {
        s.acc[ACC_PHI] = py;
        s.acc[ACC_PSI] = pl;
        s.acc[ACC_MU] = pz / (2.0 * n);
        s.acc[ACC_IPM_IT] = 0;
        s.acc[ACC_IPM_INFO] = 0;
        s.acc[ACC_IPM_DONE] = (py - pl > 1e-4) ? 0.0 : 1.0;
        // a non-finite objective (NaN or overflow in L) cannot start the IPM
        if (!isfinite(py) || !isfinite(pl)) {
            s.acc[ACC_IPM_DONE] = 1.0;
            s.status = -4;
        }
    }
}

__device__ __forceinline__ bool ipm_live(const Slot &s) { return s.active && s.acc[ACC_IPM_DONE] == 0.0; }

// Zi = Z^{-1} (ipm_mc_pk.c:121-142): A <- chol(Z); W <- inverse, full symmetric.
__global__ void __launch_bounds__(512) k_ipm_inverse(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!ipm_live(s)) return;
    const int n = s.n;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s.A[idx] = s.Q[idx];
    __syncthreads();
    int info = cta_cholesky(s.A, n);
    if (info) {
        if (threadIdx.x == 0) { s.acc[ACC_IPM_INFO] = 1; s.acc[ACC_IPM_DONE] = 1; s.status = -4; }
        return;
    }
    const double *Lf = s.A;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double *x = s.W + (size_t)c * n;
        for (int i = 0; i < c; ++i) x[i] = 0.0;
        for (int i = c; i < n; ++i) {
            double acc = i == c ? 1.0 : 0.0;
            for (int k = c; k < i; ++k) acc -= Lf[i + (size_t)k * n] * x[k];
            x[i] = acc / Lf[i + (size_t)i * n];
        }
        for (int i = n - 1; i >= 0; --i) {
            double acc = x[i];
            for (int k = i + 1; k < n; ++k) acc -= Lf[k + (size_t)i * n] * x[k];
            x[i] = acc / Lf[i + (size_t)i * n];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx / n, i = idx - j * n;
        if (i > j) {
            double a = 0.5 * (s.W[idx] + s.W[j + (size_t)i * n]);
            s.W[idx] = a;
            s.W[j + (size_t)i * n] = a;
        }
    }
}

// Predictor system (ipm_mc_pk.c:148-165): T1 <- chol(Zi o X); dy1 <- (Zi o X)^{-1}(-e);
// T2 <- -Diag(dy1) X.
__global__ void __launch_bounds__(512) k_ipm_predictor(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!ipm_live(s)) return;
    const int n = s.n;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s.T1[idx] = s.W[idx] * s.X[idx];
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.dy1[i] = -1.0;
    __syncthreads();
    if (cta_cholesky(s.T1, n)) {
        if (threadIdx.x == 0) { s.acc[ACC_IPM_INFO] = 2; s.acc[ACC_IPM_DONE] = 1; s.status = -4; }
        return;
    }
    cta_chol_solve(s.T1, n, s.dy1);
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int i = idx % n;
        s.T2[idx] = -(s.dy1[i]) * s.X[idx];
    }
}

// After dX1 = Zi*T2 (GEMM into V): dX1 -= X, symmetrise (ipm_mc_pk.c:184-191);
// corrector right-hand side and solve (:199-222); T2 <- -Diag(dy2) X - Diag(dy1) dX1.
__global__ void __launch_bounds__(512) k_ipm_corrector(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!ipm_live(s)) return;
    const int n = s.n;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s.V[idx] -= s.X[idx];
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx / n, i = idx - j * n;
        if (i > j) {
            double a = 0.5 * (s.V[idx] + s.V[j + (size_t)i * n]);
            s.V[idx] = a;
            s.V[j + (size_t)i * n] = a;
        }
    }
    __syncthreads();
    const double mu = s.acc[ACC_MU];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = 0.0;
        for (int j = 0; j < n; ++j) r += s.W[i + (size_t)j * n] * s.V[i + (size_t)j * n] * s.dy1[j];
        s.dy[i] = -r + mu * s.W[i + (size_t)i * n];
    }
    __syncthreads();
    cta_chol_solve(s.T1, n, s.dy);
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int i = idx % n;
        double t1 = -(s.dy[i]) * s.X[idx];
        double t2 = -(s.dy1[i]) * s.V[idx];
        s.T2[idx] = t1 + t2;
    }
}

// After dX = Zi*T2 (GEMM into A): dX += mu Zi; dy += dy1; dX += dX1; symmetrise
// (ipm_mc_pk.c:252-264); line searches (:272-301); update (:305-324).
__global__ void __launch_bounds__(512) k_ipm_step(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!ipm_live(s)) return;
    const int n = s.n;
    const double mu = s.acc[ACC_MU];
    __shared__ double red[40];
    __shared__ double ap_s, ad_s;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        double a = s.A[idx] + mu * s.W[idx];
        s.A[idx] = a + s.V[idx];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) s.dy[i] += s.dy1[i];
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx / n, i = idx - j * n;
        if (i > j) {
            double a = 0.5 * (s.A[idx] + s.A[j + (size_t)i * n]);
            s.A[idx] = a;
            s.A[j + (size_t)i * n] = a;
        }
    }
    __syncthreads();
    // primal line search: X + ap dX psd
    double ap = 1.0;
    for (int ls = 0;; ++ls) {
        if (ls > 400) {
            if (threadIdx.x == 0) { s.acc[ACC_IPM_INFO] = 3; s.acc[ACC_IPM_DONE] = 1; s.status = -6; }
            return;
        }
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s.T2[idx] = s.X[idx] + ap * s.A[idx];
        __syncthreads();
        if (cta_cholesky(s.T2, n) == 0) break;
        ap *= 0.8;
    }
    if (ap < 1.0) ap *= 0.95;
    double ad = 1.0;
    for (int ls = 0;; ++ls) {
        if (ls > 400) {
            if (threadIdx.x == 0) { s.acc[ACC_IPM_INFO] = 4; s.acc[ACC_IPM_DONE] = 1; s.status = -6; }
            return;
        }
        for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            int j = idx / n, i = idx - j * n;
            s.T2[idx] = s.Q[idx] + (i == j ? ad * s.dy[i] : 0.0);
        }
        __syncthreads();
        if (cta_cholesky(s.T2, n) == 0) break;
        ad *= 0.8;
    }
    if (ad < 1.0) ad *= 0.95;
    if (threadIdx.x == 0) { ap_s = ap; ad_s = ad; }
    __syncthreads();
    ap = ap_s;
    ad = ad_s;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) s.X[idx] += ap * s.A[idx];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        s.y[i] += ad * s.dy[i];
        s.Q[i + (size_t)i * n] += ad * s.dy[i];
    }
    __syncthreads();
    double pz = 0.0, pl = 0.0, py = 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        pz += s.Q[idx] * s.X[idx];
        pl += s.L[idx] * s.X[idx];
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) py += s.y[i];
    pz = block_sum(pz, red);
    pl = block_sum(pl, red);
    py = block_sum(py, red);
    if (threadIdx.x == 0) {
        double m2 = pz / (2.0 * n);
        if (ap + ad > 1.6) m2 *= 0.5;
        if (ap + ad > 1.9) m2 *= 0.2;
        s.acc[ACC_MU] = m2;
        s.acc[ACC_PHI] = py;
        s.acc[ACC_PSI] = pl;
        s.acc[ACC_AP] = ap;
        s.acc[ACC_AD] = ad;
        s.acc[ACC_IPM_IT] += 1.0;
        if (!(py - pl > 1e-4)) s.acc[ACC_IPM_DONE] = 1.0;
        if (s.acc[ACC_IPM_IT] >= 500) { s.acc[ACC_IPM_DONE] = 1.0; s.status = -6; }
    }
}

// ---------------------------------------------------------------------------
// Batched FP64 GEMM, C = A * B for the IPM products (square n x n per slot).
// which: 0 -> V = W * T2 ; 1 -> A = W * T2.  64x64 tiles, 256 threads, 4x4 per thread.
__global__ void __launch_bounds__(256) k_ipm_gemm(Slot *slots, int which) {
    Slot &s = slots[blockIdx.z];
    if (!ipm_live(s)) return;
    const int n = s.n;
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    if (i0 >= n || j0 >= n) return;
    const double *Am = s.W, *Bm = s.T2;
    double *Cm = which == 0 ? s.V : s.A;
    __shared__ double As[16][64 + 1], Bs[16][64 + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < n; k0 += 16) {
        for (int q = threadIdx.x; q < 16 * 64; q += 256) {
            int r = q & 63, kk = q >> 6;
            int ia = i0 + r, ka = k0 + kk;
            As[kk][r] = (ia < n && ka < n) ? Am[ia + (size_t)ka * n] : 0.0;
            int kb = k0 + (q & 15), jb = j0 + (q >> 4);
            Bs[q & 15][q >> 4] = (kb < n && jb < n) ? Bm[kb + (size_t)jb * n] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            int i = i0 + ty * 4 + r, j = j0 + tx * 4 + c;
            if (i < n && j < n) Cm[i + (size_t)j * n] = acc[r][c];
        }
}

// ---------------------------------------------------------------------------
void launch_ipm_init(Slot *d, int ns, cudaStream_t st) { k_ipm_init<<<ns, 256, 0, st>>>(d); }
void launch_ipm_iteration(Slot *d, int ns, int nmax, cudaStream_t st) {
    k_ipm_inverse<<<ns, 512, 0, st>>>(d);
    k_ipm_predictor<<<ns, 512, 0, st>>>(d);
    dim3 g((nmax + 63) / 64, (nmax + 63) / 64, ns);
    k_ipm_gemm<<<g, 256, 0, st>>>(d, 0);
    k_ipm_corrector<<<ns, 512, 0, st>>>(d);
    k_ipm_gemm<<<g, 256, 0, st>>>(d, 1);
    k_ipm_step<<<ns, 512, 0, st>>>(d);
}

}  // namespace mcb
