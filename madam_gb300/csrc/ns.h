// ns.h -- the chosen form of the PSD projection: a scaled Newton-Schulz sign
// iteration on the tensor cores, then an FP64 assembly of X+ = (W + W sign(W)) / 2.
//
// operators.c:521-619 projects W onto the PSD cone through a full
// eigendecomposition (dsyevr).  Here sign(W) is computed instead: W is scaled
// by an upper bound alpha of its spectral radius, then every step maps
// S <- a S + b S^3 (two batched GEMMs, FP32 accumulation).  The steps follow the
// scaled Newton-Schulz iteration of Chen & Chow (2014, "A stable scaling of
// Newton-Schulz for improving the sign function computation of a Hermitian
// matrix"): for eigenvalues of S known to lie in [l, 1] the step uses
// p(x) = 1.5 k x - 0.5 (k x)^3 with k^2 = 3 (1 - safety) / (1 + l + l^2), which
// maps both ends of the interval to the same value and so raises l fastest.
// The schedule starts from l0 (eigenvalues below l0 * alpha in magnitude are
// not resolved; they change X+ by at most l0 * alpha / 2 each) and ends once
// 1 - l < 1e-7.  By default (MCB_NS_OPERANDS_SPLIT) every product runs on the
// library's tcgen05 kernel (k_tc.cu) with operands carried as five BF16 digit
// planes whose leading digit-sum groups accumulate exactly (tc.h), accurate to
// ~5e-10 of the product: one pass of BF16 or TF32 operands cannot resolve
// eigenvalues below its rounding (~1e-3 of alpha).  The planes of S0 = W / alpha
// are cut from the FP64 W.  The cuBLAS modes (NATIVE: one-pass growth steps and
// FP32-accurate closing steps, l > 0.9; FP32; CUBLAS_SPLIT) are kept as reference
// points.  G = W S = alpha S0 S leaves the accumulators as FP64 (a cuBLAS DGEMM in
// the cuBLAS modes) and the epilogue forms X+ = (W + (G + G^T)/2) / 2 and
// Q = X+ - W in FP64.
#pragma once
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <map>
#include <utility>
#include <vector>

#include "../../include/mcbound.h"

namespace mcb {
struct Slot;

struct NsStep {
    float a, b;    // S <- a S + b S^3
    int accurate;  // FP32-accurate operands (else the form's low precision)
};

// Step schedule from l0; `safety` shrinks k^2 to keep rounding away from the
// p(x) = 0 end at x = sqrt(3).
std::vector<NsStep> ns_schedule(double l0, double safety, double eps);

struct NsProj {
    int form = 0;        // MCB_PROJ_NS_BF16 or MCB_PROJ_NS_TF32
    int operands = 1;    // MCB_NS_OPERANDS_* of the growth steps
    // SPLIT operands run on the library's own tcgen05 kernel (k_tc.cu): every
    // matrix as five BF16 digit planes (tc.h), npad a multiple of 128, G = alpha S0 S
    bool tc() const { return operands == MCB_NS_OPERANDS_SPLIT; }
    // planes (kTcPieces * cap * stride each): S0 = W / alpha, the iterates S and S2
    // in turn, and T = b S^2 + a I
    __nv_bfloat16 *Wp = nullptr, *Sp = nullptr, *S2p = nullptr, *Tp = nullptr;
    int *d_live = nullptr, *d_n = nullptr, *d_err = nullptr;
    double *d_alpha = nullptr;      // alpha = ||W||_F per slot
    unsigned char *maps = nullptr;  // TMA descriptors: the planes of W, S, S2, T (64-byte aligned)
    std::vector<unsigned char> maps_store;
    int map_npad = 0;
    int cur = 0;                    // which plane set (1: S, 2: S2) holds the result of sign()
    // autotuner: tcgen05 kernel variant per (npad, live-slot bucket), with the
    // timings (microseconds per launch) that chose it
    struct Tuned {
        int variant;
        float us[2];
    };
    std::map<std::pair<int, int>, Tuned> tuned;
    int variant = 0;                // variant of the current launch configuration
    int version = 0;                // bumped when the schedule or operands change (graph keys)
    static int bucket(int nlive) {
        int b = 1;
        while (b < nlive) b <<= 1;
        return b;
    }
    // time both variants on the live set (outside any stream capture) and keep the faster
    int tune(cudaStream_t st);
    int nmax = 0;        // largest matrix order
    int cap = 0;         // slots
    size_t stride = 0;   // elements per slot region (npad_max^2)
    cublasHandle_t h = nullptr;
    float *S = nullptr, *S2 = nullptr, *T = nullptr;  // cap * stride
    double *Wd = nullptr, *Sd = nullptr, *Gd = nullptr;
    void **dptr = nullptr;       // 6 * cap device pointers (S, S2, T, Wd, Sd, Gd per live slot)
    std::vector<void *> hptr;    // host staging of dptr
    std::vector<NsStep> steps;
    int live = 0;                // live slots in the current pointer arrays
    int npad = 0;                // order of the padded matrices of the current launch
    double l0 = 1e-6;
    // algorithmic work of the last run: low-precision GEMM flops, accurate FP32 GEMM flops, FP64 flops
    double flops_lo = 0, flops_hi = 0, flops_fp64 = 0;

    int init(int form_, int nmax_, int cap_, cudaStream_t st);
    // growth-step operands and the smallest resolved |eigenvalue| / alpha
    int configure(int operands_, double l0_);
    void destroy();
    // set the live slots (indices into the slot array) and the padded order
    int set_live(const std::vector<int> &slots, const std::vector<int> &ns, int npad_, cudaStream_t st);
    // sign(W) for the live slots from the scaled W of launch_ns_prep (gate = 1
    // skips slots whose ADMM has stopped), into Sd in FP64, and M per slot
    int sign(Slot *d_slots, int ns, int gate, cudaStream_t st);
    // G = W sign(W) in FP64 for the live slots
    int product(cudaStream_t st);
    // signs of X v for `count` hyperplane normals per listed slot (d_list / d_keys:
    // the same list on the device and the streams' keys); overwrites the live arrays
    int hyperplanes(Slot *d_slots, const std::vector<int> &slots, const int *d_list,
                    const unsigned long long *d_keys, int count, int npad_, unsigned char *d_out, size_t out_stride,
                    cudaStream_t st);
    size_t slot_offset(int slot) const { return (size_t)slot * stride; }
    // order of the padded matrices for the live slots' largest n
    int pad(int nmax_live) const { return tc() ? (nmax_live + 127) / 128 * 128 : (nmax_live + 15) / 16 * 16; }
    // the planes of S0 = W / alpha for the live slots, from the FP64 W (tcgen05 path)
    void split_inputs(cudaStream_t st);
    // MCB_ERR_ITER when a bounded wait of a tcgen05 kernel expired (flag reset)
    int check_error(cudaStream_t st);
};

// kernels (k_ns.cu)
// alpha = ||W||_F into s.acc and alpha_out[slot]; Wd = W (FP64, padded), S = W / alpha (FP32)
void launch_ns_prep(Slot *d, int ns, int npad, size_t stride, float *S, double *Wd, double *alpha_out, int gate,
                    cudaStream_t st);
void launch_ns_diag(Slot *d, int ns, int npad, size_t stride, float *T, float a, int gate, cudaStream_t st);
void launch_ns_finish(Slot *d, int ns, int npad, size_t stride, const float *S, double *Sd, int gate,
                      cudaStream_t st);
// X+ from G = W S (k_eig.cu, the epilogue of k_syrk_post): mode 1 semantics
void launch_ns_post(Slot *d, int ns, int nmax, double *partials, const double *G, int npad, size_t stride,
                    cudaStream_t st);
// mode 0 semantics (projection only: Xp full, Q lower)
void launch_ns_post0(Slot *d, int ns, int nmax, const double *G, int npad, size_t stride, cudaStream_t st);

// hyperplane rounding of the heuristic on the GPU: signs of X v for `count`
// counter-stream vectors v per slot (the vectors of the plain form's host
// heuristic, drawn in dimension n); out: n x count bytes per slot, 1 = negative
void launch_heur_vectors(Slot *d, const int *slots, const unsigned long long *keys, int nslots, int count, int rows,
                         int npad, size_t stride, float *V, cudaStream_t st);
void launch_heur_xf(Slot *d, const int *slots, int nslots, int npad, size_t stride, float *Xf, cudaStream_t st);
void launch_heur_signs(Slot *d, const int *slots, int nslots, int count, int npad, size_t stride, const float *H,
                       unsigned char *out, size_t out_stride, cudaStream_t st);
// 1-opt from each hyperplane's signs (overwritten) and the cut value of the full
// solution, over the first N of the `count` hyperplanes of each listed slot (N the
// order of the slot's own problem; the others get -inf)
void launch_heur_1opt(const Slot *d, const int *slots, int nslots, int count, const int *lists, int list_stride,
                      unsigned char *signs, size_t sstride, double *hval, cudaStream_t st);
}  // namespace mcb
