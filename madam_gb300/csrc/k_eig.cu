// k_eig.cu -- FP64 symmetric eigensolver for the PSD projection (plain form).
//
// The reference projects with LAPACK dsyevr, RANGE='V' over (1e-8, VU]
// (operators.c:521-619).  For a value range dsyevr reduces to tridiagonal form
// (dsytrd), finds the eigenvalues by Sturm bisection (dstebz) and the vectors
// by inverse iteration with re-orthogonalisation inside clusters (dstein), then
// back-transforms (dormtr).  These kernels do the same four steps on the GPU,
// one CTA per node, FP64 throughout, with full-precision bisection.
#include <cooperative_groups.h>

#include "mcb_dev.cuh"
#include "ns.h"
#include "kernels.h"

namespace mcb {

// ---------------------------------------------------------------------------
// W (lower triangle authoritative) -> A (full symmetric copy)
__global__ void k_sym_copy(Slot *slots, int src, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    int n = s.n;
    const double *W = src == 0 ? s.W : s.A;
    double *A = s.A;
    int total = n * n;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        int j = idx / n, i = idx - j * n;
        A[idx] = i >= j ? W[i + (size_t)j * n] : W[j + (size_t)i * n];
    }
}

// ---------------------------------------------------------------------------
// Householder tridiagonalisation of A (full symmetric, overwritten).  On exit
// d[0..n-1], e[0..n-2], tau[0..n-3]; reflector k has v[k+1] = 1 and
// v[i] = A[i + k n] for i >= k+2.
__global__ void __launch_bounds__(512) k_tridiag(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.x];
    if (!gated(s, gate)) return;
    const int n = s.n, tid = threadIdx.x, bs = blockDim.x;
    double *A = s.A;
    extern __shared__ double sh[];
    double *v = sh, *w = sh + n, *red = sh + 2 * n;
    for (int k = 0; k < n - 2; ++k) {
        const int m = n - k - 1;
        double *x = A + (k + 1) + (size_t)k * n;
        double loc = 0.0;
        for (int i = 1 + tid; i < m; i += bs) loc += x[i] * x[i];
        double sig2 = block_sum(loc, red);
        double alpha = x[0];
        double beta, tau, scal;
        if (sig2 == 0.0) {
            beta = alpha;
            tau = 0.0;
            scal = 0.0;
        } else {
            beta = -copysign(sqrt(alpha * alpha + sig2), alpha);
            tau = (beta - alpha) / beta;
            scal = 1.0 / (alpha - beta);
        }
        for (int i = tid; i < m; i += bs) v[i] = i == 0 ? 1.0 : x[i] * scal;
        __syncthreads();
        if (tau != 0.0) {
            const double *A22 = A + (k + 1) + (size_t)(k + 1) * n;
            for (int i = tid; i < m; i += bs) {
                double acc = 0.0;
                for (int j = 0; j < m; ++j) acc += A22[i + (size_t)j * n] * v[j];
                w[i] = tau * acc;
            }
            loc = 0.0;
            for (int i = tid; i < m; i += bs) loc += w[i] * v[i];
            double pv = block_sum(loc, red);
            double K = -0.5 * tau * pv;
            for (int i = tid; i < m; i += bs) w[i] += K * v[i];
            __syncthreads();
            double *U = A + (k + 1) + (size_t)(k + 1) * n;
            for (int idx = tid; idx < m * m; idx += bs) {
                int j = idx / m, i = idx - j * m;
                U[i + (size_t)j * n] -= v[i] * w[j] + w[i] * v[j];
            }
        }
        if (tid == 0) {
            s.d[k] = A[k + (size_t)k * n];
            s.e[k] = beta;
            s.tau[k] = tau;
        }
        for (int i = 1 + tid; i < m; i += bs) x[i] = v[i];
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            s.d[n - 2] = A[(n - 2) + (size_t)(n - 2) * n];
            s.d[n - 1] = A[(n - 1) + (size_t)(n - 1) * n];
            s.e[n - 2] = A[(n - 1) + (size_t)(n - 2) * n];
            s.tau[n - 2] = 0.0;
        } else if (n == 1) {
            s.d[0] = A[0];
        }
    }
}

// ---------------------------------------------------------------------------
// The same reduction with a slot's rows spread over the C CTAs of a thread-block
// cluster (C = gridDim.x), so that a node's 4/3 n^3 FP64 flops run on C SMs'
// FP64 pipes.  Rows are owned statically, in blocks of 32: block b (rows 32 b ..
// 32 b + 31) belongs to CTA b mod C for the whole reduction, which reads and
// writes only its own rows of A, so the product w = tau A22 v and the rank-2
// update need no exchange of matrix data, and the column-k entries a CTA sums for
// sigma^2 at step k are ones it updated itself at step k - 1.  The exchanges go
// through the slot's work array s.dwork (w, and per-CTA partial sums added in CTA
// order, so every CTA gets the same sigma^2 and v^T w), with two cluster barriers
// per step (release / acquire at cluster scope): after the sigma^2 partials
// (which also publishes the previous step's update to every CTA before any of
// them reads column k or the rows of another CTA) and after w.  Every CTA of a
// cluster runs the same loop with the same barrier sequence (the slot, n and tau
// are common to the cluster), so the barriers always match.  Within a CTA the
// warps split the columns of A22 v and of the update, and the lanes take 32
// consecutive rows of an own block (coalesced column reads).
constexpr int kTrMaxBlk = 4;  // own row blocks per CTA: ceil(ceil(n / 32) / C) <= 4 for n <= 1024
__global__ void __launch_bounds__(512) k_tridiag_cl(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;  // common to the cluster: the CTAs of one slot
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int n = s.n, tid = threadIdx.x, bs = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = bs >> 5;
    const int C = gridDim.x, c = blockIdx.x;
    const int nblk = (n + 31) >> 5;
    const int myblk = (nblk - c + C - 1) / C;  // blocks c, c + C, c + 2C, ...
    double *A = s.A;
    extern __shared__ double sh[];
    double *v = sh, *w = sh + n, *red = sh + 2 * n, *part = red + 40;  // part: nw x 32 kTrMaxBlk
    double *gw = s.dwork, *gp = s.dwork + n;  // w; partials: [0, C) sigma^2, [C, 2C) v^T w
    auto own_row = [&](int q) { return (c + q * C) * 32 + lane; };
    for (int k = 0; k < n - 2; ++k) {
        const int m = n - k - 1, r0 = k + 1;  // trailing rows / columns r0 .. n-1, local i = r - r0
        const double *colk = A + (size_t)k * n;
        double loc = 0.0;
        for (int q = wid; q < myblk; q += nw) {
            const int r = own_row(q);
            if (r >= k + 2 && r < n) loc += colk[r] * colk[r];
        }
        loc = block_sum(loc, red);
        if (tid == 0) gp[c] = loc;
        cl.sync();
        double sig2 = 0.0;
        for (int q = 0; q < C; ++q) sig2 += gp[q];
        const double alpha = colk[r0];
        double beta, tau, scal;
        if (sig2 == 0.0) {
            beta = alpha;
            tau = 0.0;
            scal = 0.0;
        } else {
            beta = -copysign(sqrt(alpha * alpha + sig2), alpha);
            tau = (beta - alpha) / beta;
            scal = 1.0 / (alpha - beta);
        }
        for (int i = tid; i < m; i += bs) v[i] = i == 0 ? 1.0 : colk[r0 + i] * scal;
        __syncthreads();
        if (tau != 0.0) {
            double acc[kTrMaxBlk];
#pragma unroll
            for (int q = 0; q < kTrMaxBlk; ++q) acc[q] = 0.0;
            for (int j = wid; j < m; j += nw) {
                const double vj = v[j];
                const double *col = A + (size_t)(r0 + j) * n;
#pragma unroll
                for (int q = 0; q < kTrMaxBlk; ++q) {
                    const int r = own_row(q);
                    if (q < myblk && r >= r0 && r < n) acc[q] += col[r] * vj;
                }
            }
#pragma unroll
            for (int q = 0; q < kTrMaxBlk; ++q) part[(wid * kTrMaxBlk + q) * 32 + lane] = acc[q];
            __syncthreads();
            double lp = 0.0;
            for (int t = tid; t < myblk * 32; t += bs) {
                const int q = t >> 5, r = (c + q * C) * 32 + (t & 31);
                if (r >= r0 && r < n) {
                    double a = 0.0;
                    for (int u = 0; u < nw; ++u) a += part[(u * kTrMaxBlk + q) * 32 + (t & 31)];
                    const double wi = tau * a;
                    gw[r - r0] = wi;
                    lp += wi * v[r - r0];
                }
            }
            lp = block_sum(lp, red);
            if (tid == 0) gp[C + c] = lp;
        }
        cl.sync();
        // every CTA has read column k: store the reflector in its own rows
        for (int q = wid; q < myblk; q += nw) {
            const int r = own_row(q);
            if (r >= k + 2 && r < n) A[r + (size_t)k * n] = v[r - r0];
        }
        if (c == 0 && tid == 0) {
            s.d[k] = A[k + (size_t)k * n];
            s.e[k] = beta;
            s.tau[k] = tau;
        }
        if (tau != 0.0) {
            double pv = 0.0;
            for (int q = 0; q < C; ++q) pv += gp[C + q];
            const double K = -0.5 * tau * pv;
            for (int i = tid; i < m; i += bs) w[i] = gw[i] + K * v[i];
            __syncthreads();
            for (int j = wid; j < m; j += nw) {
                const double vj = v[j], wj = w[j];
                double *col = A + (size_t)(r0 + j) * n;
#pragma unroll
                for (int q = 0; q < kTrMaxBlk; ++q) {
                    const int r = own_row(q);
                    if (q < myblk && r >= r0 && r < n) col[r] -= v[r - r0] * wj + w[r - r0] * vj;
                }
            }
        }
        __syncthreads();
    }
    cl.sync();
    if (c == 0 && tid == 0) {
        if (n >= 2) {
            s.d[n - 2] = A[(n - 2) + (size_t)(n - 2) * n];
            s.d[n - 1] = A[(n - 1) + (size_t)(n - 1) * n];
            s.e[n - 2] = A[(n - 1) + (size_t)(n - 2) * n];
            s.tau[n - 2] = 0.0;
        } else if (n == 1) {
            s.d[0] = A[0];
        }
    }
}

// ---------------------------------------------------------------------------
// Sturm counts: eigenvalues of T strictly below x.
//
// sturm(): dstebz's pivot recurrence q_i = d_i - x - e_{i-1}^2 / q_{i-1} with
// pivmin, one FP64 division per step; used for the largest eigenvalue of the
// safe bound, whose rigorous error term follows dstebz's analysis.
__device__ __forceinline__ int sturm(const double *d, const double *e2, int n, double x, double pivmin) {
    int cnt = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int i = 1; i < n; ++i) {
        q = d[i] - x - e2[i - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0) ++cnt;
    }
    return cnt;
}

// sturm3(): the same count from the three-term Sturm sequence p_0 = 1,
// p_1 = d_0 - x, p_{i+1} = (d_i - x) p_i - e_{i-1}^2 p_{i-1} (the method of Barth,
// Martin and Wilkinson, 1967): the number of sign changes.  No division, three
// FP64 operations per step (FP64 division costs about ten on this part).  The pair
// (p_i, p_{i+1}) is rescaled by an exact power of two when the larger exponent
// leaves [-400, 400], and an exact zero takes the sign opposite to its
// predecessor.  Used for the projection's eigenvalues, which only need to be
// accurate to a few units in the last place of ||T||.
__device__ __forceinline__ int sturm3(const double *d, const double *e2, int n, double x) {
    double p0 = 1.0, p1 = d[0] - x;
    if (p1 == 0.0) p1 = -0x1p-900;
    int cnt = p1 < 0.0;
    for (int i = 1; i < n; ++i) {
        double p2 = fma(d[i] - x, p1, -e2[i - 1] * p0);
        if (p2 == 0.0) p2 = p1 < 0.0 ? 0x1p-900 : -0x1p-900;
        cnt += (__double2hiint(p2) ^ __double2hiint(p1)) < 0;
        p0 = p1;
        p1 = p2;
        const int e0 = (__double2hiint(p0) >> 20) & 0x7ff, e1 = (__double2hiint(p1) >> 20) & 0x7ff;
        const int em = e0 > e1 ? e0 : e1;
        if (em > 1023 + 400 || em < 1023 - 400) {
            const double sc = __hiloint2double((2046 - em) << 20, 0);  // 2^(1023 - em)
            p0 *= sc;
            p1 *= sc;
        }
    }
    return cnt;
}

// Gershgorin interval of T, the largest e_i^2, and d / e^2 into shared memory
__device__ void tri_setup(const Slot &s, double *d, double *e2, double *red, double &gl, double &gu, double &emax) {
    const int n = s.n;
    double lo_g = 1e308, hi_g = -1e308, em = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] = s.d[i];
        double el = i > 0 ? fabs(s.e[i - 1]) : 0.0, er = i < n - 1 ? fabs(s.e[i]) : 0.0;
        if (i < n - 1) {
            e2[i] = s.e[i] * s.e[i];
            em = fmax(em, e2[i]);
        }
        lo_g = fmin(lo_g, d[i] - el - er);
        hi_g = fmax(hi_g, d[i] + el + er);
    }
    gl = -block_max(-lo_g, red);
    gu = block_max(hi_g, red);
    emax = block_max(em, red);
}

// Eigenvalues of T above vl (ascending) into ev[0..M-1]; M into s.M.  The CTAs
// of a slot (blockIdx.x) split the eigenvalue indices in chunks of blockDim.x,
// so that a batch of nodes spreads over every SM; each thread bisects one
// eigenvalue to dstebz's tolerance.
__global__ void __launch_bounds__(64) k_bisect(Slot *slots, double vl, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const int n = s.n, tid = threadIdx.x;
    const int first = blockIdx.x * blockDim.x;
    if (first >= n) return;
    extern __shared__ double sh[];
    double *d = sh, *e2 = sh + n, *red = sh + 2 * n;
    __shared__ int c0;
    double gl, gu, emax;
    tri_setup(s, d, e2, red, gl, gu, emax);
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, emax);
    const double tnorm = fmax(fabs(gl), fabs(gu));
    gl -= 2.0 * tnorm * 2.220446049250313e-16 * n + 2.0 * pivmin;
    gu += 2.0 * tnorm * 2.220446049250313e-16 * n + 2.0 * pivmin;
    // dstebz with ABSTOL <= 0 stops at ULP * max(|gl|, |gu|) (plus the pivmin guard)
    const double atol = 2.220446049250313e-16 * tnorm + 4.0 * pivmin;
    if (tid == 0) c0 = vl <= gl ? 0 : sturm3(d, e2, n, vl);
    __syncthreads();
    const int M = n - c0;
    if (blockIdx.x == 0 && tid == 0) s.M = M;
    const int j = first + tid;
    if (j >= M) return;
    const int idx = c0 + j;
    double lo = fmax(vl, gl), hi = gu;
    int it = 0;
    for (; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm3(d, e2, n, mid) > idx) hi = mid;
        else lo = mid;
        if (hi - lo <= 2.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + atol) break;
    }
    if (it >= 200) s.status = -6;
    s.ev[j] = 0.5 * (lo + hi);
}

// The largest eigenvalue of T into s.lmax, and the upper end of its final
// bisection bracket into acc[ACC_LMAX_HI] (the safe bound, admm.c:731-752).
__global__ void k_bisect_max(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.x];
    if (!gated(s, gate)) return;
    const int n = s.n;
    extern __shared__ double sh[];
    double *d = sh, *e2 = sh + n, *red = sh + 2 * n;
    double gl, gu, emax;
    tri_setup(s, d, e2, red, gl, gu, emax);
    if (threadIdx.x != 0) return;
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, emax);
    const double tnorm = fmax(fabs(gl), fabs(gu));
    gl -= 2.0 * tnorm * 2.220446049250313e-16 * n + 2.0 * pivmin;
    gu += 2.0 * tnorm * 2.220446049250313e-16 * n + 2.0 * pivmin;
    const double atol = 2.220446049250313e-16 * tnorm + 4.0 * pivmin;
    double lo = gl, hi = gu;
    int it = 0;
    for (; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm(d, e2, n, mid, pivmin) >= n) hi = mid;  // all eigenvalues below mid
        else lo = mid;
        if (hi - lo <= 2.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + atol) break;
    }
    s.lmax = 0.5 * (lo + hi);
    s.acc[ACC_LMAX_HI] = hi;  // upper end of the final bracket
    if (it >= 200) s.status = -6;
}

// ---------------------------------------------------------------------------
// Inverse iteration for the M eigenvectors of T (dstein's method): LU of
// (T - lambda I) with partial pivoting, three solves from a fixed pseudo-random
// start, modified Gram-Schmidt against earlier vectors of the same cluster
// (eigenvalues closer than 1e-3 ||T||_1).  Vectors go to V (n x M).
//
// One thread per cluster (a cluster's vectors depend on each other in order;
// different clusters do not), kInvThreads threads per slot spread over
// kInvThreads / 64 CTAs, striding over the clusters.  The thread's work arrays
// (dl, dd, du, du2, piv, b: 6 n doubles) live in s.dwork interleaved across the
// slot's threads (element i of array k of thread t at (k n + i) kInvThreads + t),
// so that a warp's accesses are coalesced.
struct Strided {
    double *p;
    __device__ double &operator[](int i) const { return p[(size_t)i * kInvThreads]; }
};

__device__ void tri_lu(const double *d, const double *e, int n, double lam, double tiny, Strided dl, Strided dd,
                       Strided du, Strided du2, Strided piv) {
    for (int i = 0; i < n; ++i) dd[i] = d[i] - lam;
    for (int i = 0; i < n - 1; ++i) {
        dl[i] = e[i];
        du[i] = e[i];
    }
    for (int i = 0; i < n - 1; ++i) {
        if (fabs(dd[i]) >= fabs(dl[i])) {
            if (dd[i] == 0.0) dd[i] = tiny;
            double fact = dl[i] / dd[i];
            dl[i] = fact;
            dd[i + 1] -= fact * du[i];
            if (i < n - 2) du2[i] = 0.0;
            piv[i] = 0.0;
        } else {
            double fact = dd[i] / dl[i];
            dd[i] = dl[i];
            dl[i] = fact;
            double temp = du[i];
            du[i] = dd[i + 1];
            dd[i + 1] = temp - fact * dd[i + 1];
            if (i < n - 2) {
                du2[i] = du[i + 1];
                du[i + 1] = -fact * du[i + 1];
            }
            piv[i] = 1.0;
        }
    }
    for (int i = 0; i < n; ++i)
        if (fabs(dd[i]) < tiny) dd[i] = dd[i] < 0 ? -tiny : tiny;
}

__device__ void tri_solve(int n, Strided dl, Strided dd, Strided du, Strided du2, Strided piv, Strided b) {
    for (int i = 0; i < n - 1; ++i) {
        if (piv[i] == 0.0) {
            b[i + 1] -= dl[i] * b[i];
        } else {
            double temp = b[i];
            b[i] = b[i + 1];
            b[i + 1] = temp - dl[i] * b[i];
        }
    }
    b[n - 1] /= dd[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / dd[n - 2];
    for (int i = n - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) / dd[i];
}

__global__ void __launch_bounds__(64) k_invit(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const int n = s.n, M = s.M;
    if (M <= 0) return;
    extern __shared__ double sh[];
    double *d = sh, *e = sh + n, *red = sh + 2 * n;
    int *cstart = (int *)(red + 40);  // M+1 ints
    __shared__ int ncl;
    double nrm = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] = s.d[i];
        if (i < n - 1) e[i] = s.e[i];
        double el = i > 0 ? fabs(s.e[i - 1]) : 0.0, er = i < n - 1 ? fabs(s.e[i]) : 0.0;
        nrm = fmax(nrm, fabs(s.d[i]) + el + er);
    }
    const double onenrm = block_max(nrm, red);
    const double ortol = 1e-3 * onenrm;
    const double tiny = 2.220446049250313e-16 * fmax(onenrm, 1e-300);
    if (threadIdx.x == 0) {
        int c = 0;
        for (int j = 0; j < M; ++j)
            if (j == 0 || s.ev[j] - s.ev[j - 1] > ortol) cstart[c++] = j;
        cstart[c] = M;
        ncl = c;
    }
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;  // the slot's thread, < kInvThreads
    double *base = s.dwork + t;
    const size_t stride = (size_t)n * kInvThreads;
    Strided dl{base}, dd{base + stride}, du{base + 2 * stride}, du2{base + 3 * stride}, piv{base + 4 * stride},
        b{base + 5 * stride};
    for (int cl = t; cl < ncl; cl += kInvThreads) {
        const int j0 = cstart[cl], j1 = cstart[cl + 1];
        for (int j = j0; j < j1; ++j) {
            tri_lu(d, e, n, s.ev[j], tiny, dl, dd, du, du2, piv);
            for (int i = 0; i < n; ++i) {
                uint64_t h = mix64(((uint64_t)(j + 1) << 32) ^ (uint64_t)(i + 1));
                b[i] = 2.0 * ((double)(h >> 11) * 0x1.0p-53) - 1.0;
            }
            double *vj = s.V + (size_t)j * n;
            for (int it = 0; it < 3; ++it) {
                tri_solve(n, dl, dd, du, du2, piv, b);
                double ss = 0.0;
                for (int i = 0; i < n; ++i) ss += b[i] * b[i];
                double inv = ss > 0 ? 1.0 / sqrt(ss) : 0.0;
                for (int i = 0; i < n; ++i) b[i] *= inv;
                for (int jp = j0; jp < j; ++jp) {
                    const double *vp = s.V + (size_t)jp * n;
                    double dot = 0.0;
                    for (int i = 0; i < n; ++i) dot += vp[i] * b[i];
                    for (int i = 0; i < n; ++i) b[i] -= dot * vp[i];
                }
                if (j > j0) {
                    ss = 0.0;
                    for (int i = 0; i < n; ++i) ss += b[i] * b[i];
                    inv = ss > 0 ? 1.0 / sqrt(ss) : 0.0;
                    for (int i = 0; i < n; ++i) b[i] *= inv;
                }
            }
            for (int i = 0; i < n; ++i) vj[i] = b[i];
        }
    }
}

// ---------------------------------------------------------------------------
// V (n x M) <- Q V with Q = H_0 H_1 ... H_{n-3} (dormtr).
// The columns of V are independent: CTA blockIdx.x takes columns
// [kBtCols blockIdx.x, kBtCols (blockIdx.x + 1)) of its slot, so that a node's
// 2 n^2 M FP64 flops spread over several SMs.
constexpr int kBtCols = 32;
__global__ void __launch_bounds__(256) k_backtrans(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const int n = s.n, M = s.M, lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int c0 = blockIdx.x * kBtCols, c1 = min(M, c0 + kBtCols), nc = c1 - c0;
    if (nc <= 0 || n < 3) return;
    extern __shared__ double sh[];
    double *v = sh, *sc = sh + n;
    const double *A = s.A;
    double *V = s.V;
    for (int k = n - 3; k >= 0; --k) {
        double tau = s.tau[k];
        if (tau == 0.0) continue;
        const int m = n - k - 1;
        for (int i = threadIdx.x; i < m; i += blockDim.x) v[i] = i == 0 ? 1.0 : A[(k + 1 + i) + (size_t)k * n];
        __syncthreads();
        for (int c = c0 + wid; c < c1; c += nw) {
            const double *col = V + (size_t)c * n + k + 1;
            double acc = 0.0;
            for (int i = lane; i < m; i += 32) acc += v[i] * col[i];
            acc = warp_sum(acc);
            if (lane == 0) sc[c - c0] = tau * acc;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < m * nc; idx += blockDim.x) {
            int c = idx / m, i = idx - c * m;
            V[(size_t)(c0 + c) * n + k + 1 + i] -= sc[c] * v[i];
        }
        __syncthreads();
    }
}

// Canonical sign (largest-magnitude entry positive, first on ties) and scaling
// of column j by sqrt(ev[j]) * extra (extra = 1, or sqrt(sigma) for the factor
// the heuristic reads, admm.c:582-585).
__global__ void k_canon_scale(Slot *slots, int gate) {
    Slot &s = slots[blockIdx.y];
    if (!gated(s, gate)) return;
    const int n = s.n, M = s.M, lane = threadIdx.x & 31;
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= M) return;
    double *col = s.V + (size_t)c * n;
    double best = -1.0;
    int arg = n;
    for (int i = lane; i < n; i += 32) {
        double a = fabs(col[i]);
        if (a > best) { best = a; arg = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
    }
    double sgn = col[arg] < 0 ? -1.0 : 1.0;
    double sc = sgn * sqrt(s.ev[c]);
    for (int i = lane; i < n; i += 32) col[i] *= sc;
}

// ---------------------------------------------------------------------------
// X+ = Y Y^T (Y = V after k_canon_scale, n x M) on 32x32 lower tiles, with the
// epilogue of the caller:
//   mode 0 (projection only): Xp = X+ full symmetric into s.X, Q = X+ - W lower into s.Q
//   mode 1 (ADMM step, admm.c:574-585 and the residual terms of :600-665):
//           X <- sigma X+ (full), Q <- X+ - W (full), partial sums per tile
//           of ||X+ - X_old/sigma||^2, <L, X>, ||diag X - 1||^2 into s.dwork2
//   modes 2 / 3: as 1 / 0, with X+ = (W + (G + G^T) / 2) / 2 from G = W sign(W)
//           (the Newton-Schulz form; G padded with leading dimension gld)
constexpr int TS = 32;
__global__ void __launch_bounds__(256) k_syrk_post(Slot *slots, int mode, double *partials, int ptile,
                                                   const double *G, int gld, size_t gstride) {
    Slot &s = slots[blockIdx.y];
    const int admm = mode == 1 || mode == 2;
    if (!gated(s, admm)) return;
    const int n = s.n, M = mode >= 2 ? 0 : s.M;
    const int nt = (n + TS - 1) / TS;
    const int tile = blockIdx.x;
    if (tile >= nt * (nt + 1) / 2) return;
    int ti = 0;
    while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
    int tj = tile - ti * (ti + 1) / 2;
    const int i0 = ti * TS, j0 = tj * TS;
    __shared__ double Ya[16][TS + 1], Yb[16][TS + 1];
    __shared__ double red[40];
    // 32 x 8 threads: lane tx takes row i0 + tx (the column-major reads and the
    // direct writes coalesce across the warp), four columns j0 + 4 ty + r each
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    double acc[4] = {0, 0, 0, 0};
    const double *Y = s.V;
    for (int k0 = 0; k0 < M; k0 += 16) {
        for (int q = threadIdx.x; q < 16 * TS; q += blockDim.x) {
            int kk = q / TS, r = q - kk * TS;
            int ia = i0 + r, ja = j0 + r, kc = k0 + kk;
            Ya[kk][r] = (ia < n && kc < M) ? Y[ia + (size_t)kc * n] : 0.0;
            Yb[kk][r] = (ja < n && kc < M) ? Y[ja + (size_t)kc * n] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            const double ai = Ya[kk][tx];
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[r] += ai * Yb[kk][ty * 4 + r];
        }
        __syncthreads();
    }
    double p_dres = 0.0, p_primal = 0.0, p_diag = 0.0;
    const double sg = s.sigma;
    for (int r = 0; r < 4; ++r) {
        int i = i0 + tx, j = j0 + ty * 4 + r;
        if (i >= n || j >= n || i < j) continue;
        size_t ij = i + (size_t)j * n, ji = j + (size_t)i * n;
        double w = s.W[ij];
        double xp = acc[r];
        if (mode >= 2) {
            const double *Gb = G + (size_t)blockIdx.y * gstride;
            xp = 0.5 * (w + 0.5 * (Gb[i + (size_t)j * gld] + Gb[j + (size_t)i * gld]));
        }
        if (!admm) {
            s.X[ij] = xp;
            s.X[ji] = xp;
            s.Q[ij] = xp - w;
        } else {
            double xo = s.X[ij];
            double xn = sg * xp;
            double q = xp - w;
            s.X[ij] = xn;
            s.X[ji] = xn;
            s.Q[ij] = q;
            s.Q[ji] = q;
            double dr = xp - xo / sg;
            double mult = i == j ? 1.0 : 2.0;
            p_dres += mult * dr * dr;
            p_primal += mult * s.L[ij] * xn;
            if (i == j) p_diag += (xn - 1.0) * (xn - 1.0);
        }
    }
    if (admm) {
        double a = block_sum(p_dres, red);
        double b = block_sum(p_primal, red);
        double c = block_sum(p_diag, red);
        if (threadIdx.x == 0) {
            double *pp = partials + ((size_t)blockIdx.y * ptile + tile) * 3;
            pp[0] = a;
            pp[1] = b;
            pp[2] = c;
        }
    }
}

// Sum the per-tile partials of k_syrk_post in a fixed order.
__global__ void k_syrk_reduce(Slot *slots, const double *partials, int ptile) {
    Slot &s = slots[blockIdx.x];
    if (!gated(s, 1)) return;
    const int nt = (s.n + TS - 1) / TS, T = nt * (nt + 1) / 2;
    __shared__ double red[40];
    double a = 0, b = 0, c = 0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const double *pp = partials + ((size_t)blockIdx.x * ptile + t) * 3;
        a += pp[0];
        b += pp[1];
        c += pp[2];
    }
    a = block_sum(a, red);
    b = block_sum(b, red);
    c = block_sum(c, red);
    if (threadIdx.x == 0) {
        s.acc[ACC_DRES2] = a;
        s.acc[ACC_PRIMAL] = b;
        s.acc[ACC_DIAG2] = c;
    }
}

// ---------------------------------------------------------------------------
// host-side launchers
void launch_sym_copy(Slot *d_slots, int nslots, int nmax, int src, int gate, cudaStream_t st) {
    dim3 g((nmax * nmax + 255) / 256 < 1024 ? (nmax * nmax + 255) / 256 : 1024, nslots);
    k_sym_copy<<<g, 256, 0, st>>>(d_slots, src, gate);
}
void launch_tridiag(Slot *d_slots, int nslots, int nmax, int gate, cudaStream_t st) {
    size_t sm = (2 * (size_t)nmax + 40) * sizeof(double);
    // a cluster of C CTAs per slot (about 64 rows per CTA, at most the portable 8)
    const int C = nmax >= 384 ? 8 : (nmax >= 192 ? 4 : (nmax >= 96 ? 2 : 1));
    if (C == 1) {
        k_tridiag<<<nslots, 512, sm, st>>>(d_slots, gate);
        return;
    }
    // the cluster kernel's own row blocks: at most kTrMaxBlk per CTA (n <= 1024)
    if (((nmax + 31) / 32 + C - 1) / C > kTrMaxBlk) {
        k_tridiag<<<nslots, 512, sm, st>>>(d_slots, gate);
        return;
    }
    sm += (size_t)(512 / 32) * kTrMaxBlk * 32 * sizeof(double);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C, nslots);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_tridiag_cl, d_slots, gate);
}
void launch_bisect(Slot *d_slots, int nslots, int nmax, double vl, int largest_only, int gate,
                   cudaStream_t st) {
    size_t sm = (2 * (size_t)nmax + 40) * sizeof(double);
    if (largest_only)
        k_bisect_max<<<nslots, 256, sm, st>>>(d_slots, gate);
    else
        k_bisect<<<dim3((nmax + 63) / 64, nslots), 64, sm, st>>>(d_slots, vl, gate);
}
void launch_invit(Slot *d_slots, int nslots, int nmax, int gate, cudaStream_t st) {
    size_t sm = (2 * (size_t)nmax + 40) * sizeof(double) + ((size_t)nmax + 1) * sizeof(int);
    k_invit<<<dim3(kInvThreads / 64, nslots), 64, sm, st>>>(d_slots, gate);
}
void launch_backtrans(Slot *d_slots, int nslots, int nmax, int gate, cudaStream_t st) {
    size_t sm = (2 * (size_t)nmax) * sizeof(double);
    k_backtrans<<<dim3((nmax + kBtCols - 1) / kBtCols, nslots), 256, sm, st>>>(d_slots, gate);
}
void launch_canon_scale(Slot *d_slots, int nslots, int nmax, int gate, cudaStream_t st) {
    dim3 g((nmax + 7) / 8, nslots);
    k_canon_scale<<<g, 256, 0, st>>>(d_slots, gate);
}
int syrk_tiles(int nmax) {
    int nt = (nmax + TS - 1) / TS;
    return nt * (nt + 1) / 2;
}
void launch_syrk_post(Slot *d_slots, int nslots, int nmax, int mode, double *partials, cudaStream_t st) {
    int T = syrk_tiles(nmax);
    dim3 g(T, nslots);
    k_syrk_post<<<g, 256, 0, st>>>(d_slots, mode, partials, T, nullptr, 0, 0);
    if (mode == 1) k_syrk_reduce<<<nslots, 256, 0, st>>>(d_slots, partials, T);
}
void launch_ns_post(Slot *d_slots, int nslots, int nmax, double *partials, const double *G, int npad, size_t stride,
                    cudaStream_t st) {
    int T = syrk_tiles(nmax);
    k_syrk_post<<<dim3(T, nslots), 256, 0, st>>>(d_slots, 2, partials, T, G, npad, stride);
    k_syrk_reduce<<<nslots, 256, 0, st>>>(d_slots, partials, T);
}
void launch_ns_post0(Slot *d_slots, int nslots, int nmax, const double *G, int npad, size_t stride, cudaStream_t st) {
    int T = syrk_tiles(nmax);
    k_syrk_post<<<dim3(T, nslots), 256, 0, st>>>(d_slots, 3, nullptr, T, G, npad, stride);
}

size_t eig_dwork_doubles(int nmax) { return eig_dwork_doubles_max(nmax); }

}  // namespace mcb
