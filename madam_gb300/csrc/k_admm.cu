// k_admm.cu -- one ADMM iteration of admm.c:520-704 for a batch of nodes, and
// the safe-bound post-processing of admm.c:718-763.
//
// Every kernel skips slots that are inactive or have already met the stopping
// test, so a fixed sequence of iterations can be launched (or captured in a CUDA
// graph) without a host round trip; a stopped slot keeps exactly the state of
// its stopping iteration, as the reference's `break` does.
//
// Cuts are signed cliques (k = 3/5/7 vertices p, signs e): the reference's
// op_B term is  scale * sum_{a<b} (-e_a e_b) X[p_a, p_b]  (operators.c:62-150)
// and op_Bt adds  0.5 * scale * e_a e_b * t  to both X[p_a,p_b] and X[p_b,p_a]
// (operators.c:171-513).  B^T t is formed by a gather over an edge-keyed CSR
// whose lists are in cut order, so each X entry receives its contributions in
// the same order as the reference's sequential scatter.
#include "mcb_dev.cuh"
#include "kernels.h"

namespace mcb {

__device__ __forceinline__ bool live(const Slot &s) { return s.active && !s.stop; }

// signed-clique sum of a matrix over one cut, in the reference's term order
__device__ __forceinline__ double clique_sum(const int *cp, const double *X, int n) {
    int h = cp[0], k = cut_k(h);
    double acc = 0.0;
    for (int a = 0; a < k; ++a)
        for (int b = a + 1; b < k; ++b) {
            double x = lowr(X, n, cp[1 + a], cp[1 + b]);
            acc += (cut_sign(h, a) * cut_sign(h, b) > 0) ? -x : x;
        }
    return cut_scale(k) * acc;
}

// rhs (admm.c:526-543): y = diag(L + Q + X/sigma) - e/sigma ;
// rhs_c = s_c + B(L + Q + X/sigma)_c + (u_c - 1)/sigma.  Also the per-cut data the
// first iteration of a call needs: u = 0 and t = s = initial duals (host-uploaded).
__global__ void k_admm_rhs(Slot *slots) {
    Slot &s = slots[blockIdx.y];
    if (!live(s)) return;
    const int n = s.n, m = s.m;
    const double sg = s.sigma;
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < n) {
        size_t ii = g + (size_t)g * n;
        s.y[g] = s.L[ii] + s.Q[ii] + (s.X[ii] - 1.0) / sg;
    }
    if (g < m) {
        const int *cp = s.cp + 8 * (size_t)g;
        int h = cp[0], k = cut_k(h);
        double acc = 0.0;
        for (int a = 0; a < k; ++a)
            for (int b = a + 1; b < k; ++b) {
                int i = cp[1 + a], j = cp[1 + b];
                size_t e = i > j ? i + (size_t)j * n : j + (size_t)i * n;
                double x = s.L[e] + s.Q[e] + s.X[e] / sg;
                acc += (cut_sign(h, a) * cut_sign(h, b) > 0) ? -x : x;
            }
        double r = s.s[g] + cut_scale(k) * acc;
        s.rhs[g] = r + (s.u[g] - 1.0) / sg;
    }
}

// (B B^T + I) t = rhs (the reference factors with CHOLMOD, admm.c:546) to
// ||rhs - A t|| <= rtol ||rhs|| (the plain form uses rtol = 1e-13), warm-started
// from the current t, by mixed-precision iterative refinement: the true residual
// r = rhs - A t and the stopping test in FP64, the correction A d = r by
// conjugate gradients in FP32 (its rate is ~64x FP64's on this part) to 1e-5 of
// ||r||, then t += d.  A has eigenvalues in [1, ~11], so each outer step gains
// about five digits and two or three reach 1e-13.  One CTA per slot, one thread
// per matrix row.  The system is small and fixed for the whole solve (m cuts,
// a few nonzeros per row), so the solve is a chain of short, synchronised
// steps whose cost is latency: the kernel copies the CSR structure and the FP32
// values into shared memory once, next to the FP32 work vectors (direction p,
// product q, scaled residual, correction), when they fit in kCgShBytes; the
// vectors alone when only they fit; otherwise everything stays in the slot's
// arrays (cgp / cgq hold two floats per double).  The iteration cap counts the
// FP32 CG iterations; reaching it before the tolerance sets status and leaves t
// as far as it got.
constexpr int kCgOuter = 12;             // refinement steps at most
constexpr double kCgInnerRel2 = 1e-10;   // (1e-5)^2: the inner CG's relative target
constexpr int kCgShBytes = 200 * 1024;   // dynamic shared memory of k_cg
__global__ void __launch_bounds__(1024) k_cg(Slot *slots, int maxit, double rtol2) {
    Slot &s = slots[blockIdx.x];
    if (!live(s)) return;
    const int m = s.m;
    if (m == 0) return;
    __shared__ double red[40];
    extern __shared__ float csh[];
    const int nnz = s.g_rp[m];
    const size_t vec_words = 4 * (size_t)m, csr_words = (size_t)m + 1 + 2 * (size_t)nnz;
    const bool vec_sh = vec_words * 4 <= kCgShBytes, csr_sh = (vec_words + csr_words) * 4 <= kCgShBytes;
    double *x = s.t, *r = s.cgr;
    float *p = vec_sh ? csh : (float *)s.cgq, *q = vec_sh ? csh + m : (float *)s.cgq + m;
    float *ri = vec_sh ? csh + 2 * m : (float *)s.cgp, *d = vec_sh ? csh + 3 * m : (float *)s.cgp + m;
    const int *rp = s.g_rp, *ci = s.g_ci;
    const float *gf = s.g_v32;
    if (csr_sh) {
        int *rps = (int *)(csh + vec_words), *cis = rps + m + 1;
        float *gfs = (float *)(cis + nnz);
        for (int k = threadIdx.x; k <= m; k += blockDim.x) rps[k] = s.g_rp[k];
        for (int k = threadIdx.x; k < nnz; k += blockDim.x) {
            cis[k] = s.g_ci[k];
            gfs[k] = s.g_v32[k];
        }
        rp = rps;
        ci = cis;
        gf = gfs;
    }
    const double *gv = s.g_v;
    double lbb = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) lbb += s.rhs[i] * s.rhs[i];
    const double bb = block_sum(lbb, red);  // (its barriers also publish the copies above)
    const double stop2 = rtol2 * bb;
    int it = 0;
    double rr = 0.0;
    for (int outer = 0;; ++outer) {
        double lrr = 0.0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            double acc = 0.0;
            for (int k = rp[i]; k < rp[i + 1]; ++k) acc += gv[k] * x[ci[k]];
            const double res = s.rhs[i] - acc;
            r[i] = res;
            lrr += res * res;
        }
        rr = block_sum(lrr, red);
        if (rr <= stop2 || it >= maxit || outer >= kCgOuter) break;
        // the correction, on the residual scaled to unit norm (FP32's range)
        const double nr = sqrt(rr), inv = 1.0 / nr;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const float v = (float)(r[i] * inv);
            ri[i] = v;
            p[i] = v;
            d[i] = 0.0f;
        }
        __syncthreads();
        double rz = 1.0;  // the scaled residual's squared norm
        while (rz > kCgInnerRel2 && it < maxit) {
            double lpq = 0.0;
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                float acc = 0.0f;
                for (int k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(gf[k], p[ci[k]], acc);
                q[i] = acc;
                lpq += (double)(p[i] * acc);
            }
            const double pq = block_sum(lpq, red);
            const float alpha = (float)(rz / pq);
            double l2 = 0.0;
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                d[i] = fmaf(alpha, p[i], d[i]);
                const float v = fmaf(-alpha, q[i], ri[i]);
                ri[i] = v;
                l2 += (double)(v * v);
            }
            const double rz2 = block_sum(l2, red);
            const float beta = (float)(rz2 / rz);
            for (int i = threadIdx.x; i < m; i += blockDim.x) p[i] = fmaf(beta, p[i], ri[i]);
            __syncthreads();
            rz = rz2;
            ++it;
        }
        for (int i = threadIdx.x; i < m; i += blockDim.x) x[i] += nr * (double)d[i];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s.cg_iters = it;
        if (rr > stop2) s.status = -6;
    }
}

// the FP32 copy of A's values for the inner CG (k_cg), per live slot
__global__ void k_cg_values(Slot *slots) {
    Slot &s = slots[blockIdx.y];
    if (!s.active) return;
    const int nnz = s.m > 0 ? s.g_rp[s.m] : 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x)
        s.g_v32[k] = (float)s.g_v[k];
}

// admm.c:556-560, 587-591: v = t - u/sigma, s = v_+, u = -sigma v_- ; and W (admm.c:564-568):
// W = L + X/sigma - Diag(y) - B^T(t), lower triangle (one thread per element).
__global__ void k_admm_su(Slot *slots) {
    Slot &s = slots[blockIdx.y];
    if (!live(s)) return;
    const double sg = s.sigma;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < s.m; g += gridDim.x * blockDim.x) {
        double v = s.t[g] - s.u[g] / sg;
        s.v[g] = v;
        s.s[g] = v > 0 ? v : 0;
        s.u[g] = v < 0 ? -sg * v : 0;
    }
}

// mat = 0: W = L + X/sigma - Diag(y)   (ADMM step, lower triangle)
// mat = 1: A = L - Diag(y)              (safe bound, admm.c:727-728, full symmetric)
// B^T of t (mat 0) or s (mat 1) is added afterwards by k_apply_edges.
__global__ void k_build_W(Slot *slots, int mat) {
    Slot &s = slots[blockIdx.y];
    if (mat == 0 ? !live(s) : !s.active) return;
    const int n = s.n;
    const double sg = s.sigma;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * n; idx += gridDim.x * blockDim.x) {
        int j = idx / n, i = idx - j * n;
        if (mat == 0) {
            if (i < j) continue;
            double w = s.L[idx] + s.X[idx] / sg;
            if (i == j) w -= s.y[i];
            s.W[idx] = w;
        } else {
            double w = s.L[idx];
            if (i == j) w -= s.y[i];
            s.A[idx] = w;
        }
    }
}

// W[e] (mat 0) or A[e] and its mirror (mat 1) += sum over the cuts through e of
// coef * t_c (resp. s_c), added one at a time in cut order (op_Bt, operators.c:171-513).
__global__ void k_apply_edges(Slot *slots, int mat) {
    Slot &s = slots[blockIdx.y];
    if (mat == 0 ? !live(s) : !s.active) return;
    const int n = s.n;
    const double *tv = mat == 0 ? s.t : s.s;
    double *M = mat == 0 ? s.W : s.A;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < s.ne; q += gridDim.x * blockDim.x) {
        int idx = s.e_idx[q];
        double w = M[idx];
        for (int r = s.e_rp[q]; r < s.e_rp[q + 1]; ++r) w += s.e_coef[r] * tv[s.e_cut[r]];
        M[idx] = w;
        if (mat == 1) {
            int j = idx / n, i = idx - j * n;
            M[j + (size_t)i * n] = w;
        }
    }
}

// Operator-level forms on an arbitrary matrix of slot 0 (KATs):
// y_c += B(X)_c (X lower) and X -= B^T(t) on both triangles.
__global__ void k_op_B(Slot *slots, const double *X, double *y) {
    Slot &s = slots[0];
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < s.m; g += gridDim.x * blockDim.x)
        y[g] += clique_sum(s.cp + 8 * (size_t)g, X, s.n);
}
__global__ void k_op_Bt(Slot *slots, double *X, const double *t) {
    Slot &s = slots[0];
    const int n = s.n;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < s.ne; q += gridDim.x * blockDim.x) {
        int idx = s.e_idx[q];
        int j = idx / n, i = idx - j * n;
        double a = X[idx], b = X[j + (size_t)i * n];
        for (int r = s.e_rp[q]; r < s.e_rp[q + 1]; ++r) {
            double c = s.e_coef[r] * t[s.e_cut[r]];
            a += c;
            b += c;
        }
        X[idx] = a;
        X[j + (size_t)i * n] = b;
    }
}

// admm.c:607-617: b_c = -1 + B(X)_c, kept in cgq for the residual reduction
__global__ void k_admm_bx(Slot *slots) {
    Slot &s = slots[blockIdx.y];
    if (!live(s)) return;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < s.m; g += gridDim.x * blockDim.x) {
        const int *cp = s.cp + 8 * (size_t)g;
        s.cgq[g] = -1.0 + clique_sum(cp, s.X, s.n);
    }
}

// Residuals, objectives, sigma update and the stopping test (admm.c:594-702).
__global__ void __launch_bounds__(512) k_admm_finish(Slot *slots, double scaleSigma, int itermax) {
    Slot &s = slots[blockIdx.x];
    if (!live(s)) return;
    const int n = s.n, m = s.m;
    __shared__ double red[40];
    double sy = 0, st = 0, smt = 0, bx = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sy += s.y[i];
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        st += s.t[i];
        double d = s.s[i] - s.t[i];
        smt += d * d;
        double b = s.cgq[i];
        if (b > 0) bx += b * b;
    }
    sy = block_sum(sy, red);
    st = block_sum(st, red);
    smt = block_sum(smt, red);
    bx = block_sum(bx, red);
    if (threadIdx.x == 0) {
        s.nbit += 1;
        double err_p = (sqrt(s.acc[ACC_DIAG2]) + sqrt(bx)) / (1.0 + sqrt((double)n));
        double err_d = (sqrt(smt) + sqrt(s.acc[ACC_DRES2])) / (1.0 + s.normL);
        double primal = s.acc[ACC_PRIMAL];
        double dual = sy + st;
        double gap = fabs(dual - primal) / (1.0 + fabs(dual) + fabs(primal));
        double err = err_p > err_d ? (err_p > gap ? err_p : gap) : (err_d > gap ? err_d : gap);
        s.acc[ACC_ERR_P] = err_p;
        s.acc[ACC_ERR_D] = err_d;
        s.acc[ACC_GAP] = gap;
        s.acc[ACC_ERR] = err;
        s.acc[ACC_SUMY] = sy;
        s.acc[ACC_DUAL_T] = st;
        s.acc[ACC_SIGMA_LAST] = s.sigma;
        double dp = log10(err_p), dd = log10(err_d);
        if (dd - dp < -0.5) s.sigma /= scaleSigma;
        else if (dd - dp > 0.5) s.sigma *= scaleSigma;
        if (err < s.tol || s.nbit > itermax) s.stop = 1;
        if (!(err == err)) { s.stop = 1; s.status = -4; }
        if (s.status) s.stop = 1;  // a failed step (e.g. the CG cap) ends this node's ADMM
    }
}

// Safe bound (admm.c:757-763): f = n * lambda_max(L - Diag y - B^T s) + sum y + sum s,
// with lambda_max replaced by a rigorous upper bound: the top of the bisection
// bracket plus 8 n eps ||A||_F for the tridiagonal reduction's backward error.
__global__ void __launch_bounds__(512) k_safe_norm(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!s.active) return;
    const int n = s.n;
    __shared__ double red[40];
    double a = 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) a += s.A[idx] * s.A[idx];
    a = block_sum(a, red);
    if (threadIdx.x == 0) s.acc[ACC_FNORM] = sqrt(a);
}
__global__ void __launch_bounds__(512) k_safe_finish(Slot *slots) {
    Slot &s = slots[blockIdx.x];
    if (!s.active) return;
    const int n = s.n, m = s.m;
    __shared__ double red[40];
    double sy = 0, ss = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sy += s.y[i];
    for (int i = threadIdx.x; i < m; i += blockDim.x) ss += s.s[i];
    sy = block_sum(sy, red);
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) {
        double lam = s.acc[ACC_LMAX_HI] + 8.0 * n * 2.220446049250313e-16 * s.acc[ACC_FNORM];
        s.f = n * lam + sy + ss;
        s.acc[ACC_SUMY] = sy;
        s.acc[ACC_SUMS] = ss;
    }
}

// ---------------------------------------------------------------------------
static inline int cdiv(int a, int b) { return (a + b - 1) / b; }

void launch_admm_rhs(Slot *d, int ns, int nmax, int mmax, cudaStream_t st) {
    int tot = nmax > mmax ? nmax : mmax;
    dim3 g(cdiv(tot, 256), ns);
    k_admm_rhs<<<g, 256, 0, st>>>(d);
}
int cg_prepare() {
    return cudaFuncSetAttribute(k_cg, cudaFuncAttributeMaxDynamicSharedMemorySize, kCgShBytes) == cudaSuccess ? 0
                                                                                                                : -1;
}
void launch_cg(Slot *d, int ns, int mmax, int maxit, double rtol, cudaStream_t st) {
    (void)mmax;
    k_cg<<<ns, 1024, kCgShBytes, st>>>(d, maxit, rtol * rtol);
}
void launch_cg_values(Slot *d, int ns, cudaStream_t st) { k_cg_values<<<dim3(64, ns), 256, 0, st>>>(d); }
void launch_admm_su(Slot *d, int ns, int mmax, cudaStream_t st) {
    dim3 g(cdiv(mmax > 1 ? mmax : 1, 256) < 512 ? cdiv(mmax > 1 ? mmax : 1, 256) : 512, ns);
    k_admm_su<<<g, 256, 0, st>>>(d);
}
void launch_build_W(Slot *d, int ns, int nmax, int emax, int mat, cudaStream_t st) {
    int b = cdiv(nmax * nmax, 256);
    dim3 g(b < 1024 ? b : 1024, ns);
    k_build_W<<<g, 256, 0, st>>>(d, mat);
    int be = cdiv(emax > 1 ? emax : 1, 256);
    dim3 ge(be < 512 ? be : 512, ns);
    k_apply_edges<<<ge, 256, 0, st>>>(d, mat);
}
void launch_op_B(Slot *d, int m, const double *X, double *y, cudaStream_t st) {
    k_op_B<<<cdiv(m > 1 ? m : 1, 256), 256, 0, st>>>(d, X, y);
}
void launch_op_Bt(Slot *d, int ne, double *X, const double *t, cudaStream_t st) {
    k_op_Bt<<<cdiv(ne > 1 ? ne : 1, 256), 256, 0, st>>>(d, X, t);
}
void launch_admm_bx(Slot *d, int ns, int mmax, cudaStream_t st) {
    dim3 g(cdiv(mmax > 1 ? mmax : 1, 256) < 512 ? cdiv(mmax > 1 ? mmax : 1, 256) : 512, ns);
    k_admm_bx<<<g, 256, 0, st>>>(d);
}
void launch_admm_finish(Slot *d, int ns, double scaleSigma, int itermax, cudaStream_t st) {
    k_admm_finish<<<ns, 512, 0, st>>>(d, scaleSigma, itermax);
}
void launch_safe_norm(Slot *d, int ns, cudaStream_t st) { k_safe_norm<<<ns, 512, 0, st>>>(d); }
void launch_safe_finish(Slot *d, int ns, cudaStream_t st) { k_safe_finish<<<ns, 512, 0, st>>>(d); }

}  // namespace mcb
