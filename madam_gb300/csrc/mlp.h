// mlp.h -- device-side interface of the learned models (mlp.cu) for the engine.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace mcb {
constexpr int kMlpMaxIn = 16;
constexpr int kMlpMaxHidden = 32;
struct MlpImpl;
// buffers for n samples (inputs, targets, outputs, index list, block partials)
int mlp_ensure(MlpImpl *M, size_t n);
// out[s] = f(X[s, :]) for s < n, on the device
void mlp_forward_device(const MlpImpl *M, const float *dX, int n, float *dOut, cudaStream_t st);
}  // namespace mcb

struct mcb_mlp;
mcb::MlpImpl *mlp_impl(mcb_mlp *h);
int mlp_inputs(const mcb_mlp *h);
