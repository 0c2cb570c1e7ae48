// k_learn.cu -- per-cut features of the learned models, computed on the GPU from
// the node's current X and its subproblem matrix L.
//
// A cut c (any family, packed as in Slot::cp) constrains <B_c, X> <= 1 with
// <B_c, X> = -scale_k sum_{a<b} e_a e_b X[p_a, p_b].  Its features (kCutFeatures):
//   0  k / 7                                  (family)
//   1  <B_c, X> - 1                           (violation; > 0 when violated)
//   2  mean_{a<b} e_a e_b X_ab                 3  min of the same   4  max of the same
//   5  mean_{a<b} e_a e_b 4 L_ab / (1 + max |4 L_ab|)   (edge weights seen by the cut)
//   6  fraction of the pairs that are edges (L_ab != 0)
//   7  n / N                                   (subproblem size)
//   8  log(1 + extra)                          (the cut's dual in the parent node, or 0)
//   9  1 if the cut uses the subproblem's last (fixed-side) vertex
#include <cuda_runtime.h>

#include "learn.h"
#include "mcb_dev.cuh"

namespace mcb {
namespace {

__global__ void __launch_bounds__(128) k_cut_features(const Slot *slots, const int *slot_of, const int *cps, int ncut,
                                                      const double *extra, float *F) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ncut) return;
    const Slot &s = slots[slot_of[q]];
    const int *cp = cps + 8 * (size_t)q;
    const int h = cp[0], k = cut_k(h), n = s.n;
    double sum = 0.0, mn = 1e300, mx = -1e300, wsum = 0.0, wmax = 0.0;
    int edges = 0, last = 0, pairs = 0;
    for (int a = 0; a < k; ++a) {
        int pa = cp[1 + a];
        if (pa == n - 1) last = 1;
        for (int b = a + 1; b < k; ++b) {
            int pb = cp[1 + b];
            double eab = (double)(cut_sign(h, a) * cut_sign(h, b));
            double x = eab * lowr(s.X, n, pa, pb);
            double l = 4.0 * lowr(s.L, n, pa, pb);
            sum += x;
            mn = fmin(mn, x);
            mx = fmax(mx, x);
            wsum += eab * l;
            wmax = fmax(wmax, fabs(l));
            edges += l != 0.0;
            ++pairs;
        }
    }
    const double mean = sum / pairs;
    float *f = F + (size_t)q * kCutFeatures;
    f[0] = (float)k / 7.0f;
    f[1] = (float)(-cut_scale(k) * sum - 1.0);
    f[2] = (float)mean;
    f[3] = (float)mn;
    f[4] = (float)mx;
    f[5] = (float)(wsum / pairs / (1.0 + wmax));
    f[6] = (float)edges / (float)pairs;
    f[7] = (float)n / (float)s.N;
    f[8] = extra ? (float)log1p(fmax(extra[q], 0.0)) : 0.0f;
    f[9] = (float)last;
}

}  // namespace

void launch_cut_features(const Slot *d_slots, const int *slot_of, const int *cps, int ncut, const double *extra,
                         float *F, cudaStream_t st) {
    if (ncut <= 0) return;
    k_cut_features<<<(ncut + 127) / 128, 128, 0, st>>>(d_slots, slot_of, cps, ncut, extra, F);
}

}  // namespace mcb
