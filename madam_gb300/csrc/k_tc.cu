// k_tc.cu -- the Newton-Schulz GEMMs on the 5th-generation tensor cores
// (tcgen05.mma, operands staged by TMA, accumulators in tensor memory).
//
// C = alpha * A * B^T + diag * I_n for a batch of npad x npad row-major matrices
// (one per live slot).  In the projection A and B are symmetric and commute
// (B is a polynomial in A, or A = W and B = sign(W)), so A B^T = A B is
// symmetric: only the lower 128 x 128 tiles are computed and each is stored with
// its mirror, which keeps the iterates exactly symmetric.  (Without it the
// rounding's antisymmetric part would grow by the step's slope, ~2.6x, every
// step, since X (aI + b X X^T) is not a polynomial in X once X is not symmetric.)
//
// Operands are the five BF16 digit planes of tc.h: q = x 2^7 / sigma =
// sum_a d_a 2^-7a with signed 7-bit digits, plane a holding d_a 2^-7a.  A product
// is the sum of the nineteen plane products of digit sum <= 5, in four FP32
// accumulators in tensor memory:
//   acc0 <- d0 . d0'                 (digit sum 0: integers below 2^24, exact)
//   acc1 <- d0 . d1' + d1 . d0'       (digit sum 1: multiples of 2^-7, exact)
//   acc2 <- the three of digit sum 2  (multiples of 2^-14, exact)
//   acc3 <- the thirteen of digit sum 3, 4, 5 (FP32, ~2^-12 of the total)
// so C = alpha sigma_A sigma_B 2^-14 (acc0 + acc1 + acc2 + acc3), accurate to
// ~5e-10 of its norm: FP32 rounding touches only acc3, far below the floor of a
// three-piece BF16 split accumulated in FP32 (~1e-7 per product), which the
// Newton-Schulz iteration compounded to ~1e-6 in the projection.  The epilogue
// sums the four accumulators as an unevaluated float pair (no FP64 arithmetic,
// which is slow on this part) and writes C as FP32, as FP64 (times a per-slot
// factor) and/or as the next step's five digit planes.
//
// Tiling: one CTA of eight warps per 128 x 128 tile of C and slot; K in chunks of
// 32 BF16 (one 64-byte swizzle row).  A stage holds the five planes of the A and
// B chunks (80 KB).  The four accumulators take all 512 tensor-memory columns, so
// one CTA runs per SM; the autotuner times two variants: two pipeline stages or
// one.  One thread of warp 1 issues the TMA copies (waiting only for a stage to be
// released), one thread of warp 0 issues the MMAs (waiting only for a stage to
// land), so the MMAs of the next chunk queue behind those of this one.  All eight
// warps drain the accumulators with tcgen05.ld (warp w: lanes 32 (w mod 4) .. +31,
// columns 64 (w / 4) .. +63) in two phases.  Phase A sums each element's four
// accumulators to a float pair; an off-diagonal tile stores its rows from
// registers (16 consecutive columns per thread: vector stores of whole 32-byte
// sectors), and a symmetric product stages the pairs, transposed, in shared
// memory.  Phase B writes, again as whole rows, the diagonal tiles (every element
// from the lower triangle, so the result is exactly symmetric) and the mirrors of
// the off-diagonal tiles.  Every wait on an mbarrier is bounded: on expiry the CTA records an
// error code, gives the TMA loads it still has in flight their own bounded wait,
// skips the rest and releases its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>

#include "../../include/mcbound.h"
#include "mcb_dev.cuh"
#include "tc.h"

namespace mcb {
namespace {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int kPieces = kTcPieces;
constexpr int kTileBytes = BM * BK * 2;                // one plane of one operand chunk (8 KB)
constexpr int kStageBytes = 2 * kPieces * kTileBytes;  // A and B, five planes each (80 KB)
constexpr int kThreads = 256;                          // eight warps
constexpr int kChunk = 16;                             // epilogue: columns per tcgen05.ld
constexpr int kLdF = BM + 1;                           // epilogue staging F[c][r], in float pairs
constexpr int kEpiBytes = BN * kLdF * 8;               // 132,096 B: the whole tile as float pairs
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
// variant 0: two stages; variant 1: one stage.  The four accumulators hold all 512
// tensor-memory columns, so the shared memory asked for is at least kOneCtaBytes,
// more than half an SM's: a second CTA never lands on the SM to wait for them.
constexpr int kStages0 = 2, kStages1 = 1;
constexpr int kOneCtaBytes = 120 * 1024;
constexpr int smem_bytes(int stages) {
    return cmax(cmax(stages * kStageBytes, kEpiBytes) + 1024 + 128, kOneCtaBytes);
}
constexpr int kAccs = 4;
constexpr uint32_t kTmemCols = kAccs * BN;   // 512: acc0 .. acc3
constexpr long long kSpinLimit = 1ll << 26;  // bounded waits (~a second)
// the expiry test: no TMA loads are issued (nothing is ever in flight), so the
// first wait on a full stage runs out after this many polls (~a millisecond)
constexpr long long kTestSpinLimit = 1ll << 16;
std::atomic<int> g_test_expiry{0};

// the nineteen plane products (A plane, B plane, accumulator) of digit sum <= 5;
// kFirst: the product that starts each accumulator
constexpr int kProducts = 19;
__constant__ int kProdA[kProducts] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4, 1, 2, 3, 4};
__constant__ int kProdB[kProducts] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0, 4, 3, 2, 1, 0, 4, 3, 2, 1};
__constant__ int kProdAcc[kProducts] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3};
__constant__ int kFirst[kAccs] = {0, 1, 3, 6};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// true when the phase with the given parity has completed; false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit) {
    for (long long it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// shared-memory matrix descriptor: K-major, 64-byte swizzle (rows of 64 bytes,
// the pattern repeats every 8 rows = 512 bytes), 8-row groups 512 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);  // start address
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused with this swizzle)
    d |= (uint64_t)(512 >> 4) << 32;         // stride byte offset
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)4 << 61;                  // 64-byte swizzle
    return d;
}

// instruction descriptor: kind::f16 with BF16 A/B, FP32 accumulator, both K-major, M x N
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// s + e = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// the five digits of q = qh + ql (|q| <= 64, |ql| <= ulp(qh) / 2), each times its
// weight 2^-7a: d_a = rint of the remainder scaled by 2^7a.  r - rint(r) and the
// scaling by 2^7 are exact, so d0, d1, d2 are exact digits of qh (|d| <= 64); ql
// (at most 2^-18 when |qh| < 64) joins the remainder after them, which rounds
// once at ~2^-39 of q, and d3 may reach 68 (its pairs are summed in FP32 in any
// case).  The five digits leave q - sum d_a 2^-7a within 2^-29.
__device__ __forceinline__ void digits(float qh, float ql, float *o) {
    float r = qh;
#pragma unroll
    for (int a = 0; a < kPieces; ++a) {
        const float d = rintf(r);
        o[a] = d * __int_as_float((127 - 7 * a) << 23);  // d 2^-7a: exact
        r = a == 2 ? fmaf(ql, 2097152.0f, (r - d) * 128.0f) : (r - d) * 128.0f;
    }
}
// the same as BF16 planes (d 2^-7a has at most 7 significant bits: exact in BF16)
__device__ __forceinline__ void planes(float qh, float ql, __nv_bfloat16 *o) {
    float v[kPieces];
    digits(qh, ql, v);
#pragma unroll
    for (int a = 0; a < kPieces; ++a) o[a] = __float2bfloat16_rn(v[a]);
}

// coef (acc0 + acc1 + acc2 + acc3) + d as an unevaluated float pair (h, l): the
// exact accumulators summed by two-sums, the product's rounding error recovered
// by an FMA, the diagonal added by a two-sum
__device__ __forceinline__ float2 ff_value(float a0, float a1, float a2, float a3, float coef, float d) {
    float s, e, e2;
    two_sum(a0, a1, s, e);
    two_sum(s, a2, s, e2);
    e += e2;
    two_sum(s, a3, s, e2);
    e += e2;
    float h = coef * s;
    float l = fmaf(coef, e, fmaf(coef, s, -h));
    if (d != 0.0f) {
        two_sum(h, d, h, e2);
        l += e2;
    }
    two_sum(h, l, h, l);
    return make_float2(h, l);
}

struct Maps {
    CUtensorMap a[kPieces], b[kPieces];
};

// a bounded wait that also ends when *abort is set (by the CTA's other role)
__device__ __forceinline__ bool mbar_wait_or(uint64_t *bar, uint32_t parity, long long limit, volatile int *abort) {
    for (long long it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
    }
    return false;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

template <int kStages>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ Maps maps, TcOut out, int npad, const int *live, const int *nlist, float alpha,
              float diag, float in_scale, int sym, long long spin_limit, int issue_loads) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + cmax(kStages * kStageBytes, kEpiBytes));
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    __shared__ int s_fail, s_issued, s_landed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_n = npad / BN;
    int ti = blockIdx.x / tiles_n, tj = blockIdx.x % tiles_n;
    if (sym) {  // lower tiles only: blockIdx.x = ti (ti + 1) / 2 + tj, tj <= ti
        ti = 0;
        while ((ti + 1) * (ti + 2) / 2 <= (int)blockIdx.x) ++ti;
        tj = blockIdx.x - ti * (ti + 1) / 2;
    }
    const int m0 = ti * BM, n0 = tj * BN;
    const int slot = live[blockIdx.y];
    const int nk = npad / BK;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        s_fail = 0;
        s_issued = 0;
        s_landed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int *fail = &s_fail;

    if (warp == 1 && lane == 0) {
        // TMA producer: chunk kc goes to stage kc mod kStages once the MMAs of chunk
        // kc - kStages have released it (the expiry test issues nothing)
        int issued = 0;
        for (int kc = 0; kc < nk && issue_loads; ++kc) {
            const int s = kc % kStages;
            if (kc >= kStages && !mbar_wait_or(&empty[s], (uint32_t)(kc / kStages - 1) & 1u, spin_limit, fail)) {
                *fail = 1;
                break;
            }
            if (*fail) break;
            unsigned char *st = smem + s * kStageBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            for (int p = 0; p < kPieces; ++p) {
                tma_load_3d(st + p * kTileBytes, &maps.a[p], kc * BK, m0, slot, &full[s]);
                tma_load_3d(st + (kPieces + p) * kTileBytes, &maps.b[p], kc * BK, n0, slot, &full[s]);
            }
            ++issued;
        }
        s_issued = issued;
    } else if (warp == 0 && lane == 0) {
        // MMA issuer: the nineteen plane products of each landed chunk, then its stage
        // is released by a commit
        const uint32_t idesc = instr_desc(BM, BN);
        int landed = 0;
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc % kStages;
            if (!mbar_wait_or(&full[s], (uint32_t)(kc / kStages) & 1u, spin_limit, fail)) {
                *fail = 1;
                break;
            }
            ++landed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(smem + s * kStageBytes);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
#pragma unroll
                for (int q = 0; q < kProducts; ++q) {
                    // each accumulator starts with its first product of the first chunk
                    const int ac = kProdAcc[q];
                    const uint64_t ad = smem_desc(base + kProdA[q] * kTileBytes + kk * 32);
                    const uint64_t bd = smem_desc(base + (kPieces + kProdB[q]) * kTileBytes + kk * 32);
                    const uint32_t acc = !(kc == 0 && kk == 0 && q == kFirst[ac]);
                    mma_bf16(tmem + (uint32_t)(ac * BN), ad, bd, idesc, acc);
                }
            mma_commit(&empty[s]);
        }
        s_landed = landed;
        mma_commit(done);
    }
    __syncwarp();
    // every thread waits for the accumulators; the outcome is made block-uniform
    bool ok = mbar_wait(done, 0, kSpinLimit);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int bad = __syncthreads_or(!ok || s_fail);
    if (bad) {
        if (tid == 0) {
            if (out.err) atomicExch(out.err, MCB_ERR_ITER);
            // loads still in flight write this CTA's shared memory: give them their
            // own bounded wait before the block can exit and the memory is reused
            for (int j = s_landed; j < s_issued; ++j)
                mbar_wait(&full[j % kStages], (uint32_t)(j / kStages) & 1u, kSpinLimit);
        }
    } else {
        const int n = nlist[blockIdx.y];
        const float coef = alpha * in_scale;
        const double fscale = out.slot_scale ? out.slot_scale[slot] : 1.0;
        const int g = warp & 3;         // tensor-memory lanes 32 g .. 32 g + 31: tile rows
        const int r = g * 32 + lane;    // this thread's tile row (phase A) / row of its output (phase B)
        const int cbeg = (warp >> 2) * (BN / 2);
        const bool diag_tile = sym && ti == tj;
        const size_t sb = (size_t)slot * out.stride;
        const bool want_planes = out.p[0] != nullptr;
        // F[c kLdF + rr] = C(m0 + rr, n0 + c) as a float pair: the stage buffers are free
        // once the MMAs are done
        float2 *F = (float2 *)smem;
        // the outputs of 16 consecutive columns of one output row at element offset o,
        // from their float pairs: whole 32-byte sectors per thread
        auto store_row = [&](size_t o, const float *h, const float *l) {
            if (out.f32) {
                float4 *o4 = reinterpret_cast<float4 *>(out.f32 + o);
#pragma unroll
                for (int q = 0; q < kChunk / 4; ++q)
                    o4[q] = make_float4(h[4 * q] + l[4 * q], h[4 * q + 1] + l[4 * q + 1], h[4 * q + 2] + l[4 * q + 2],
                                        h[4 * q + 3] + l[4 * q + 3]);
            }
            if (out.f64) {
                double2 *o2 = reinterpret_cast<double2 *>(out.f64 + o);
#pragma unroll
                for (int q = 0; q < kChunk / 2; ++q)
                    o2[q] = make_double2(fscale * ((double)h[2 * q] + (double)l[2 * q]),
                                         fscale * ((double)h[2 * q + 1] + (double)l[2 * q + 1]));
            }
            if (want_planes) {
                uint32_t pk[kPieces][kChunk / 2];
#pragma unroll
                for (int j = 0; j < kChunk; j += 2) {
                    float d0[kPieces], d1[kPieces];
                    digits(h[j] * out.pscale, l[j] * out.pscale, d0);
                    digits(h[j + 1] * out.pscale, l[j + 1] * out.pscale, d1);
#pragma unroll
                    for (int p = 0; p < kPieces; ++p) pk[p][j / 2] = pack_bf16(d0[p], d1[p]);
                }
#pragma unroll
                for (int p = 0; p < kPieces; ++p) {
                    uint4 *o4 = reinterpret_cast<uint4 *>(out.p[p] + o);
                    o4[0] = make_uint4(pk[p][0], pk[p][1], pk[p][2], pk[p][3]);
                    o4[1] = make_uint4(pk[p][4], pk[p][5], pk[p][6], pk[p][7]);
                }
            }
        };
        // phase A: the accumulators of this thread's row, 16 columns at a time, summed to
        // float pairs; an off-diagonal tile stores them in place, and a symmetric product
        // stages them (transposed) for phase B
        for (int c0 = cbeg; c0 < cbeg + BN / 2; c0 += kChunk) {
            float h[kChunk], l[kChunk];
            {
                float v[kAccs][kChunk];
#pragma unroll
                for (int a = 0; a < kAccs; ++a)
                    tmem_ld16(tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)(a * BN + c0), v[a]);
#pragma unroll
                for (int j = 0; j < kChunk; ++j) {
                    const int row = m0 + r, col = n0 + c0 + j;
                    const float2 x =
                        ff_value(v[0][j], v[1][j], v[2][j], v[3][j], coef, (row == col && row < n) ? diag : 0.0f);
                    h[j] = x.x;
                    l[j] = x.y;
                    if (sym) F[(c0 + j) * kLdF + r] = x;
                }
            }
            if (!diag_tile) store_row(sb + (size_t)(m0 + r) * npad + n0 + c0, h, l);
        }
        if (sym) {
            __syncthreads();
            // phase B: a diagonal tile writes its rows whole, each element taken from the
            // lower triangle (C(c, r) for c > r), so the result is exactly symmetric; an
            // off-diagonal tile writes its mirror: output row n0 + r holds C(m0 + k, n0 + r)
            for (int c0 = cbeg; c0 < cbeg + BN / 2; c0 += kChunk) {
                float h[kChunk], l[kChunk];
#pragma unroll
                for (int j = 0; j < kChunk; ++j) {
                    const int c = c0 + j;
                    const float2 x = diag_tile ? (c <= r ? F[c * kLdF + r] : F[r * kLdF + c]) : F[r * kLdF + c];
                    h[j] = x.x;
                    l[j] = x.y;
                }
                if (diag_tile)
                    store_row(sb + (size_t)(m0 + r) * npad + n0 + c0, h, l);
                else
                    store_row(sb + (size_t)(n0 + r) * npad + m0 + c0, h, l);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// FP32 (or FP64) matrices -> the five digit planes of q = x pscale (/ slot_div[slot]),
// row-major npad x npad per listed slot
template <typename T>
__global__ void k_tc_split(const T *src, size_t sstride, TcOut out, int npad, const int *live,
                           const double *slot_div) {
    const int slot = live[blockIdx.y];
    const size_t tot = (size_t)npad * npad;
    const T *s = src + (size_t)slot * sstride;
    const double inv = slot_div && slot_div[slot] != 0.0 ? 1.0 / slot_div[slot] : 1.0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        const size_t o = (size_t)slot * out.stride + q;
        __nv_bfloat16 pl[kPieces];
        if (sizeof(T) == 4 && !slot_div) {
            planes((float)s[q] * out.pscale, 0.0f, pl);  // a power-of-two scale: exact
        } else {
            // the FP64 value as a float pair (h + l to 2^-48), then the digits in FP32:
            // three FP64 operations per element instead of four per digit
            const double x = (double)s[q] * inv * (double)out.pscale;
            const float h = (float)x;
            planes(h, (float)(x - (double)h), pl);
        }
#pragma unroll
        for (int p = 0; p < kPieces; ++p) out.p[p][o] = pl[p];
    }
}

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
    }
    return fn;
}

}  // namespace

// a 3D tensor map over `slots` row-major npad x npad BF16 matrices spaced `stride`
// elements apart; boxes of 32 x 128 elements (64-byte rows, 64-byte swizzle)
int tc_make_map(void *map, const __nv_bfloat16 *base, int npad, size_t stride, int slots) {
    EncodeTiled enc = encoder();
    if (!enc) return MCB_ERR_CUDA;
    if (npad % BN || ((uintptr_t)base & 15) || (stride * 2) % 16) return MCB_ERR_ARG;
    cuuint64_t dims[3] = {(cuuint64_t)npad, (cuuint64_t)npad, (cuuint64_t)slots};
    cuuint64_t strides[2] = {(cuuint64_t)npad * 2, (cuuint64_t)stride * 2};
    cuuint32_t box[3] = {BK, BM, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc((CUtensorMap *)map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? MCB_OK : MCB_ERR_CUDA;
}

size_t tc_map_bytes() { return sizeof(CUtensorMap); }

int tc_gemm(const void *amaps, const void *bmaps, const TcOut &out, int npad, int nlive, const int *d_live,
            const int *d_n, float alpha, float diag, float in_scale, cudaStream_t st, int sym, int variant) {
    if (nlive <= 0) return MCB_OK;
    if (npad % BM || npad % BK || npad > 1024 || variant < 0 || variant >= kTcVariants) return MCB_ERR_ARG;
    // the shared-memory limit is a per-device function attribute: set it once on
    // every device that launches the kernel
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCB_ERR_CUDA;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
    if (!bit || !(attr_set.load() & bit)) {
        if (cudaFuncSetAttribute(k_tc_gemm<kStages0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_bytes(kStages0)) != cudaSuccess ||
            cudaFuncSetAttribute(k_tc_gemm<kStages1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_bytes(kStages1)) != cudaSuccess)
            return MCB_ERR_CUDA;
        attr_set.fetch_or(bit);
    }
    Maps m;
    memcpy(m.a, amaps, sizeof(m.a));
    memcpy(m.b, bmaps, sizeof(m.b));
    const int nt = npad / BM;
    dim3 grid(sym ? nt * (nt + 1) / 2 : nt * nt, nlive);
    const int test = g_test_expiry.load();
    const long long spins = test ? kTestSpinLimit : kSpinLimit;
    if (variant == 0)
        k_tc_gemm<kStages0><<<grid, kThreads, smem_bytes(kStages0), st>>>(m, out, npad, d_live, d_n, alpha, diag, in_scale,
                                                                     sym, spins, !test);
    else
        k_tc_gemm<kStages1><<<grid, kThreads, smem_bytes(kStages1), st>>>(m, out, npad, d_live, d_n, alpha, diag, in_scale,
                                                                     sym, spins, !test);
    return cudaGetLastError() == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

int tc_test_expiry() { return g_test_expiry.load(); }

void tc_split_f32(const float *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st) {
    if (nlive <= 0) return;
    int g = (int)(((size_t)npad * npad + 255) / 256);
    g = g > 128 ? 128 : g;
    k_tc_split<float><<<dim3(g, nlive), 256, 0, st>>>(src, sstride, out, npad, d_live, nullptr);
}
void tc_split_f64(const double *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  const double *slot_div, cudaStream_t st) {
    if (nlive <= 0) return;
    int g = (int)(((size_t)npad * npad + 255) / 256);
    g = g > 128 ? 128 : g;
    k_tc_split<double><<<dim3(g, nlive), 256, 0, st>>>(src, sstride, out, npad, d_live, slot_div);
}

}  // namespace mcb

// The expiry test of the bounded waits (see mcbound.h).
extern "C" void mcb_tc_test_expiry(int on) { mcb::g_test_expiry.store(on ? 1 : 0); }
