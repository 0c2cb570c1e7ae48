// tc.h -- the tcgen05 GEMM of the Newton-Schulz form (k_tc.cu).
//
// Operand format.  A matrix x with a power-of-two scale sigma (|x| <= sigma / 2
// for the exactness bounds below) is carried as q = x 2^7 / sigma cut into five
// signed digits, q = d0 + d1 2^-7 + d2 2^-14 + d3 2^-21 + d4 2^-28 (each rounded
// to nearest, |d_a| <= 64; d3 may reach 68 where a float pair is cut, and only
// enters the FP32 group below), digit a stored as the BF16 value d_a 2^-7a
// (exact): five BF16 planes per matrix, q to within 2^-29.  A product of two such
// matrices is a sum over digit pairs; the pairs of digit sum 0, 1 and 2 give
// integer multiples of 2^0, 2^-7, 2^-14 below 2^24 in magnitude (for K <= 1024),
// which FP32 accumulators hold exactly, and the pairs of digit sum 3 to 5 are
// ~2^-12 of the total, so their FP32 rounding stays near 2^-36.  The product is
// accurate to ~5e-10 of its norm (pairs of digit sum 6 and above are dropped).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace mcb {

constexpr int kTcPieces = 5;  // the digit planes d0 .. d4

// outputs of one GEMM (row-major npad x npad per slot, `stride` elements apart);
// any of f32, f64 and the planes p may be null
struct TcOut {
    float *f32;
    double *f64;
    __nv_bfloat16 *p[kTcPieces];  // the output's planes, q = x pscale (see above)
    size_t stride;
    int *err;                     // set to MCB_ERR_ITER when a bounded wait expires
    float pscale;                 // 2^7 / sigma of the output planes
    const double *slot_scale;     // per-slot factor of the f64 output (indexed by slot), or null
};

constexpr int kTcTile = 128;  // npad must be a multiple of this
size_t tc_map_bytes();
// TMA descriptor (tc_map_bytes() bytes, 64-byte aligned) of `slots` BF16 matrices
int tc_make_map(void *map, const __nv_bfloat16 *base, int npad, size_t stride, int slots);
// C = alpha A B^T + diag I_n (n = d_n[k] for live slot d_live[k]); amaps / bmaps: five
// maps each (the planes); in_scale = sigma_A sigma_B 2^-14 (the unit of d0 . d0').
// sym = 1: the product is symmetric; the lower tiles are computed and mirrored
// variant: 0 = two pipeline stages, 1 = one stage (one CTA per SM either way)
constexpr int kTcVariants = 2;
int tc_gemm(const void *amaps, const void *bmaps, const TcOut &out, int npad, int nlive, const int *d_live,
            const int *d_n, float alpha, float diag, float in_scale, cudaStream_t st, int sym, int variant);
// 1 while the expiry test of the bounded waits is on (mcb_tc_test_expiry)
int tc_test_expiry();
// the five planes of FP32 / FP64 matrices (row-major, source slots `sstride` apart);
// out.pscale is the planes' 2^7 / sigma; the FP64 values are divided by
// slot_div[slot] first when it is given
void tc_split_f32(const float *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st);
void tc_split_f64(const double *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  const double *slot_div, cudaStream_t st);
}  // namespace mcb
