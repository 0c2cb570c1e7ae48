// k_sub.cu -- createSubproblem (evaluate.c:39-116) and getFixedValue
// (evaluate.c:124-139) on the GPU, one CTA per node, from the resident SP->L.
//
// Per-slot index lists (list_stride ints): [nu, nf1, nfx, U[nu], F1[nf1], FX[nfx], FS[nfx]]
// with U the unfixed vertices, F1 the vertices fixed to 1, FX/FS the fixed
// vertices and their values, all ascending, so every sum runs in the
// reference's order.
#include "mcb_dev.cuh"
#include "kernels.h"

namespace mcb {

__global__ void __launch_bounds__(256) k_subproblem(Slot *slots, const int *lists, int stride, double *fixedval) {
    Slot &s = slots[blockIdx.x];
    if (!s.active) return;
    const double *SL = s.SL;  // the slot's own problem
    const int N = s.N;
    const int *ls = lists + (size_t)blockIdx.x * stride;
    const int nu = ls[0], nf1 = ls[1], nfx = ls[2];
    const int *U = ls + 3, *F1 = U + nu, *FX = F1 + nf1, *FS = FX + nfx;
    const int n = nu + 1;
    double *L = s.L;
    double *fixedRow = s.vtmp;
    for (int c = threadIdx.x; c < nu; c += blockDim.x) {
        const double *col = SL + (size_t)U[c] * N;
        double row_sum = 0.0;
        for (int r = 0; r < nu; ++r) {
            double v = col[U[r]];
            L[r + (size_t)c * n] = v;
            row_sum += v;
        }
        L[(n - 1) + (size_t)c * n] = row_sum;
        double fr = 0.0;
        for (int q = 0; q < nf1; ++q) fr += SL[U[c] + (size_t)F1[q] * N];
        fixedRow[c] = fr;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nu; c += blockDim.x) {
        double fr2 = 2 * fixedRow[c];
        L[c + (size_t)c * n] += fr2;
        double lastrow = L[(n - 1) + (size_t)c * n] + fr2;
        L[(n - 1) + (size_t)c * n] = lastrow;
        L[c + (size_t)(n - 1) * n] = lastrow;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int c = 0; c < nu; ++c) sum += L[c + (size_t)(n - 1) * n];
        L[(n - 1) + (size_t)(n - 1) * n] = sum;
        double fv = 0.0;
        for (int a = 0; a < nfx; ++a)
            for (int b = 0; b < nfx; ++b) fv += SL[FX[b] + (size_t)FX[a] * N] * FS[a] * FS[b];
        fixedval[blockIdx.x] = fv;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) L[idx] *= 0.25;
    __syncthreads();
    // ||L||_F as dlansy('F', 'L') sees it (admm.c:640): diagonal + 2 x strict lower
    __shared__ double red[40];
    double dg = 0.0, lo = 0.0;
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
        int j = idx / n, i = idx - j * n;
        double v = L[idx];
        if (i == j) dg += v * v;
        else if (i > j) lo += v * v;
    }
    dg = block_sum(dg, red);
    lo = block_sum(lo, red);
    if (threadIdx.x == 0) s.normL = sqrt(dg + 2.0 * lo);
}

void launch_subproblem(Slot *d, int ns, const int *d_lists, int list_stride, double *d_fixed, cudaStream_t st) {
    k_subproblem<<<ns, 256, 0, st>>>(d, d_lists, list_stride, d_fixed);
}

}  // namespace mcb
