// learn.h -- features of the learned cut ranking and dual warm start (k_learn.cu).
#pragma once
#include <cuda_runtime.h>

namespace mcb {
struct Slot;
constexpr int kCutFeatures = 10;
// F[q, :] = features of cut q (packed cps[8 q ..]) of slot slot_of[q], from that
// slot's X and L; extra[q] = the cut's dual in the parent node (may be null)
void launch_cut_features(const Slot *d_slots, const int *slot_of, const int *cps, int ncut, const double *extra,
                         float *F, cudaStream_t st);
}  // namespace mcb
