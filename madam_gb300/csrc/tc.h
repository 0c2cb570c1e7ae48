// tc.h -- the tcgen05 split-BF16 GEMM of the Newton-Schulz form (k_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace mcb {

// outputs of one GEMM (row-major npad x npad per slot, `stride` elements apart);
// any of f32, f64 and the pieces p may be null
struct TcOut {
    float *f32;
    double *f64;
    __nv_bfloat16 *p[3];
    size_t stride;
    int *err;  // set to MCB_ERR_ITER when a bounded wait expires
};

constexpr int kTcTile = 128;  // npad must be a multiple of this
size_t tc_map_bytes();
// TMA descriptor (tc_map_bytes() bytes, 64-byte aligned) of `slots` BF16 matrices
int tc_make_map(void *map, const __nv_bfloat16 *base, int npad, size_t stride, int slots);
// C = alpha A B^T + diag I_n (n = d_n[k] for live slot d_live[k]); amaps / bmaps: three maps each.
// sym = 1: the product is symmetric; the lower tiles are computed and mirrored
// variant: 0 = one stage, two CTAs per SM; 1 = two stages, one CTA per SM
constexpr int kTcVariants = 2;
int tc_gemm(const void *amaps, const void *bmaps, const TcOut &out, int npad, int nlive, const int *d_live,
            const int *d_n, float alpha, float diag, cudaStream_t st, int sym, int variant);
// 1 while the expiry test of the bounded waits is on (mcb_tc_test_expiry)
int tc_test_expiry();
// three BF16 pieces of FP32 / FP64 matrices (row-major, source slots `sstride` apart)
void tc_split_f32(const float *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st);
void tc_split_f64(const double *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st);
}  // namespace mcb
