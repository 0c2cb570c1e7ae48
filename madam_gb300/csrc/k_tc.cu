// k_tc.cu -- the Newton-Schulz GEMMs on the 5th-generation tensor cores
// (tcgen05.mma, operands staged by TMA, accumulator in tensor memory).
//
// C = alpha * A * B^T + diag * I_n for a batch of npad x npad row-major matrices
// (one per live slot).  In the projection A and B are symmetric and commute
// (B is a polynomial in A, or A = W and B = sign(W)), so A B^T = A B is
// symmetric: only the lower 128 x 128 tiles are computed and each is stored with
// its mirror, which keeps the iterates exactly symmetric.  (Without it the
// rounding's antisymmetric part would grow by the step's slope, ~2.6x, every
// step, since X (aI + b X X^T) is not a polynomial in X once X is not symmetric.)
// Every FP32 operand X is carried as three BF16 pieces x_hi + x_mid + x_lo
// (each the BF16 rounding of what the previous pieces leave), which together
// hold 24 significant bits.  The product keeps the six piece products whose
// weight is at least 2^-16 of the leading one -- hi.hi, hi.mid, mid.hi, mid.mid,
// hi.lo, lo.hi -- and accumulates them in FP32 in tensor memory (hi.hi and the
// five corrections in two accumulators), so C is FP32-accurate.  The epilogue
// writes C as FP32, as its own three pieces (the next step's operands) and/or
// widened to FP64.
//
// Tiling: one CTA per 128 x 128 tile of C and slot; K in chunks of 64 BF16
// (one 128-byte swizzle row).  A stage holds the three pieces of the A and B
// chunks (96 KB).  Two variants, timed by the autotuner: one stage per CTA, so
// that two CTAs fit on an SM (shared memory and the 512 tensor-memory columns)
// and one CTA's TMA loads overlap the other's MMAs; or two stages with one CTA
// per SM.  One thread issues the TMA copies and the MMAs; all four warps drain
// the accumulators (32 lanes each) with tcgen05.ld, through shared-memory tiles
// (row-major for the direct half, column-major for the mirror) so that every
// global store is coalesced and 64 or 128 bits wide.  Every wait on an
// mbarrier is bounded: on expiry the CTA records an error code, gives the TMA
// loads it still has in flight their own bounded wait, skips the rest and
// releases its tensor memory.
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

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int kPieces = 3;
constexpr int kTileBytes = BM * BK * 2;                   // one piece of one operand chunk (16 KB)
constexpr int kStageBytes = 2 * kPieces * kTileBytes;    // A and B, three pieces each (96 KB)
// two variants, picked per matrix order by the autotuner (tc_variant): one stage
// per CTA with two CTAs per SM, or two stages (TMA of chunk k+1 under the MMAs of
// chunk k) with one CTA per SM
constexpr int smem_bytes(int stages) { return stages * kStageBytes + 1024 + 128; }
constexpr uint32_t kTmemCols = 256;  // two 128-column FP32 accumulators: hi.hi, and the corrections
constexpr long long kSpinLimit = 1ll << 26;  // bounded waits (~a second)
// the expiry test: no TMA loads are issued (nothing is ever in flight), so the
// first wait on a full stage runs out after this many polls (~a millisecond)
constexpr long long kTestSpinLimit = 1ll << 16;
std::atomic<int> g_test_expiry{0};

// the six piece products (A piece, B piece)
__constant__ int kProdA[6] = {0, 0, 1, 1, 0, 2};
__constant__ int kProdB[6] = {0, 1, 0, 1, 2, 0};

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

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);   // start address
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused with this swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // 128-byte swizzle
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

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    h = __float2bfloat16_rn(x);
    float r = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r);
    l = __float2bfloat16_rn(r - __bfloat162float(m));
}

// three BF16 pieces of four values, packed for 64-bit stores
__device__ __forceinline__ void split3x4(float4 x, uint2 &h, uint2 &m, uint2 &l) {
    const float xs[4] = {x.x, x.y, x.z, x.w};
    __nv_bfloat162 hp[2], mp[2], lp[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float a = xs[2 * k], b = xs[2 * k + 1];
        hp[k] = __floats2bfloat162_rn(a, b);
        const float ra = a - __low2float(hp[k]), rb = b - __high2float(hp[k]);
        mp[k] = __floats2bfloat162_rn(ra, rb);
        lp[k] = __floats2bfloat162_rn(ra - __low2float(mp[k]), rb - __high2float(mp[k]));
    }
    h = make_uint2(*reinterpret_cast<uint32_t *>(&hp[0]), *reinterpret_cast<uint32_t *>(&hp[1]));
    m = make_uint2(*reinterpret_cast<uint32_t *>(&mp[0]), *reinterpret_cast<uint32_t *>(&mp[1]));
    l = make_uint2(*reinterpret_cast<uint32_t *>(&lp[0]), *reinterpret_cast<uint32_t *>(&lp[1]));
}

struct Maps {
    CUtensorMap a[kPieces], b[kPieces];
};


template <int kStages>
__global__ void __launch_bounds__(128, 3 - kStages) k_tc_gemm(const __grid_constant__ Maps maps, TcOut out, int npad,
                                                   const int *live, const int *nlist, float alpha, float diag,
                                                   int sym, long long spin_limit, int issue_loads) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    __shared__ int s_fail;

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

    if (tid == 0) {
        const uint32_t idesc = instr_desc(BM, BN);
        int issued = 0, landed = 0;  // chunks whose loads were issued / have been waited for
        auto load = [&](int kc) {
            if (!issue_loads) return;  // the expiry test: nothing is issued, nothing is in flight
            const int s = kc % kStages;
            unsigned char *st = smem + s * kStageBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            for (int p = 0; p < kPieces; ++p) {
                tma_load_3d(st + p * kTileBytes, &maps.a[p], kc * BK, m0, slot, &full[s]);
                tma_load_3d(st + (kPieces + p) * kTileBytes, &maps.b[p], kc * BK, n0, slot, &full[s]);
            }
            ++issued;
        };
        bool ok = true;
        for (int kc = 0; kc < kStages && kc < nk; ++kc) load(kc);
        for (int kc = 0; kc < nk && ok; ++kc) {
            const int s = kc % kStages;
            const uint32_t use = (uint32_t)(kc / kStages) & 1u;
            ok = mbar_wait(&full[s], use, spin_limit);
            if (!ok) break;
            ++landed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(smem + s * kStageBytes);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    // hi.hi into the first accumulator, the five correction products
                    // (2^-8 of it or less) into the second, so that their bits are
                    // not lost against the leading term; the epilogue adds the two
                    uint64_t ad = smem_desc(base + kProdA[q] * kTileBytes + kk * 32);
                    uint64_t bd = smem_desc(base + (kPieces + kProdB[q]) * kTileBytes + kk * 32);
                    const uint32_t acc = q == 0 ? (kc | kk) != 0 : !(kc == 0 && kk == 0 && q == 1);
                    mma_bf16(tmem + (q == 0 ? 0u : (uint32_t)BN), ad, bd, idesc, acc);
                }
            mma_commit(&empty[s]);
            // refill this stage once its MMAs have read it
            if (kc + kStages < nk) {
                ok = mbar_wait(&empty[s], use, spin_limit);
                if (!ok) break;
                load(kc + kStages);
            }
        }
        if (!ok) {
            s_fail = 1;
            // loads still in flight write this CTA's shared memory: give them their
            // own bounded wait before the block can exit and the memory is reused
            for (int j = landed; j < issued; ++j) mbar_wait(&full[j % kStages], (uint32_t)(j / kStages) & 1u, kSpinLimit);
        }
        mma_commit(done);
    }
    __syncwarp();
    // every thread waits for the accumulator; the outcome is made block-uniform
    bool ok = mbar_wait(done, 0, kSpinLimit);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int bad = __syncthreads_or(!ok || s_fail);
    if (bad) {
        if (tid == 0 && out.err) atomicExch(out.err, MCB_ERR_ITER);
    } else {
        const int n = nlist[blockIdx.y];
        // Stores go through a shared-memory tile (the stage buffers are free once
        // the MMAs are done) so that every global store is coalesced and 64 or
        // 128 bits wide.  Symmetric products: the lower triangle is stored twice,
        // as (row, col) from a row-major tile and mirrored to (col, row) from a
        // column-major one (the accumulators are read a second time for it), so
        // the result is exactly symmetric; diagonal tiles store their lower part.
        constexpr int LD = BN + 4;  // 16-byte rows, conflict-free 128-bit accesses
        float *F = (float *)smem;
        const int r = warp * 32 + lane;
        const bool diag_tile = sym && ti == tj;
        const size_t sb = (size_t)slot * out.stride;
        auto value = [&](float acc, int row, int col) {
            return alpha * acc + ((row == col && row < n) ? diag : 0.0f);
        };
        // store elements valid_from .. valid_to of four consecutive values (all of
        // them as vectors); unrolled with register selects, no local memory
        auto store4 = [&](size_t o, float4 x, int valid_from, int valid_to) {
            if (valid_from == 0 && valid_to == 3) {
                if (out.f32) *reinterpret_cast<float4 *>(out.f32 + o) = x;
                if (out.f64) {
                    reinterpret_cast<double2 *>(out.f64 + o)[0] = make_double2(x.x, x.y);
                    reinterpret_cast<double2 *>(out.f64 + o)[1] = make_double2(x.z, x.w);
                }
                if (out.p[0]) {
                    uint2 h, m, l;
                    split3x4(x, h, m, l);
                    *reinterpret_cast<uint2 *>(out.p[0] + o) = h;
                    *reinterpret_cast<uint2 *>(out.p[1] + o) = m;
                    *reinterpret_cast<uint2 *>(out.p[2] + o) = l;
                }
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    if (e < valid_from || e > valid_to) continue;
                    const float xe = e == 0 ? x.x : (e == 1 ? x.y : (e == 2 ? x.z : x.w));
                    if (out.f32) out.f32[o + e] = xe;
                    if (out.f64) out.f64[o + e] = (double)xe;
                    if (out.p[0]) {
                        __nv_bfloat16 h, m, l;
                        split3(xe, h, m, l);
                        out.p[0][o + e] = h;
                        out.p[1][o + e] = m;
                        out.p[2][o + e] = l;
                    }
                }
            }
        };
        // (1) row-major tile F[r][c] = C(m0 + r, n0 + c)
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32], w[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(BN + c0), w);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int c = c0 + 4 * q;
                float4 x = make_float4(value(v[4 * q] + w[4 * q], m0 + r, n0 + c),
                                       value(v[4 * q + 1] + w[4 * q + 1], m0 + r, n0 + c + 1),
                                       value(v[4 * q + 2] + w[4 * q + 2], m0 + r, n0 + c + 2),
                                       value(v[4 * q + 3] + w[4 * q + 3], m0 + r, n0 + c + 3));
                *reinterpret_cast<float4 *>(F + r * LD + c) = x;
            }
        }
        __syncthreads();
        // direct half: warp per row, lane per 4 columns; diagonal tiles keep col <= row
        for (int rr = warp; rr < BM; rr += 4) {
            const int c = 4 * lane;
            if (diag_tile && c > rr) continue;
            const float4 x = *reinterpret_cast<const float4 *>(F + rr * LD + c);
            // on a diagonal tile, columns c .. min(c + 3, rr)
            store4(sb + (size_t)(m0 + rr) * npad + n0 + c, x, 0, diag_tile ? min(3, rr - c) : 3);
        }
        if (sym) {
            __syncthreads();
            // (2) column-major tile F[c][r] = C(m0 + r, n0 + c), from the accumulators again
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float v[32], w[32];
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
                tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(BN + c0), w);
#pragma unroll
                for (int j = 0; j < 32; ++j) F[(c0 + j) * LD + r] = value(v[j] + w[j], m0 + r, n0 + c0 + j);
            }
            __syncthreads();
            // mirrored half: output row n0 + cc, lane per 4 rows of the tile; diagonal
            // tiles keep rows strictly below the diagonal (rr > cc)
            for (int cc = warp; cc < BN; cc += 4) {
                const int rr0 = 4 * lane;
                const int from = diag_tile ? max(0, cc + 1 - rr0) : 0;
                if (from >= 4) continue;
                const float4 x = *reinterpret_cast<const float4 *>(F + cc * LD + rr0);
                store4(sb + (size_t)(n0 + cc) * npad + m0 + rr0, x, from, 3);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// FP32 (or FP64) matrices -> three BF16 pieces, row-major npad x npad per listed slot
template <typename T>
__global__ void k_tc_split(const T *src, size_t sstride, TcOut out, int npad, const int *live) {
    const int slot = live[blockIdx.y];
    const size_t tot = (size_t)npad * npad;
    const T *s = src + (size_t)slot * sstride;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
        const size_t o = (size_t)slot * out.stride + q;
        double x = (double)s[q];
        __nv_bfloat16 h = __double2bfloat16(x);
        double r = x - (double)__bfloat162float(h);
        __nv_bfloat16 m = __double2bfloat16(r);
        double r2 = r - (double)__bfloat162float(m);
        out.p[0][o] = h;
        out.p[1][o] = m;
        out.p[2][o] = __double2bfloat16(r2);
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

// a 3D tensor map over `slots` row-major npad x npad BF16 matrices spaced `stride` elements apart
int tc_make_map(void *map, const __nv_bfloat16 *base, int npad, size_t stride, int slots) {
    EncodeTiled enc = encoder();
    if (!enc) return MCB_ERR_CUDA;
    if (npad % BN || ((uintptr_t)base & 15) || (stride * 2) % 16) return MCB_ERR_ARG;
    cuuint64_t dims[3] = {(cuuint64_t)npad, (cuuint64_t)npad, (cuuint64_t)slots};
    cuuint64_t strides[2] = {(cuuint64_t)npad * 2, (cuuint64_t)stride * 2};
    cuuint32_t box[3] = {BK, BM, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = enc((CUtensorMap *)map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? MCB_OK : MCB_ERR_CUDA;
}

size_t tc_map_bytes() { return sizeof(CUtensorMap); }

int tc_gemm(const void *amaps, const void *bmaps, const TcOut &out, int npad, int nlive, const int *d_live,
            const int *d_n, float alpha, float diag, cudaStream_t st, int sym, int variant) {
    if (nlive <= 0) return MCB_OK;
    if (npad % BM || npad % BK || variant < 0 || variant >= kTcVariants) return MCB_ERR_ARG;
    // the shared-memory limit is a per-device function attribute: set it once on
    // every device that launches the kernel
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCB_ERR_CUDA;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
    if (!bit || !(attr_set.load() & bit)) {
        if (cudaFuncSetAttribute(k_tc_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(1)) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(2)) !=
                cudaSuccess)
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
        k_tc_gemm<1><<<grid, 128, smem_bytes(1), st>>>(m, out, npad, d_live, d_n, alpha, diag, sym, spins, !test);
    else
        k_tc_gemm<2><<<grid, 128, smem_bytes(2), st>>>(m, out, npad, d_live, d_n, alpha, diag, sym, spins, !test);
    return cudaGetLastError() == cudaSuccess ? MCB_OK : MCB_ERR_CUDA;
}

int tc_test_expiry() { return g_test_expiry.load(); }

void tc_split_f32(const float *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st) {
    if (nlive <= 0) return;
    int g = (int)(((size_t)npad * npad + 255) / 256);
    g = g > 128 ? 128 : g;
    k_tc_split<float><<<dim3(g, nlive), 256, 0, st>>>(src, sstride, out, npad, d_live);
}
void tc_split_f64(const double *src, size_t sstride, const TcOut &out, int npad, int nlive, const int *d_live,
                  cudaStream_t st) {
    if (nlive <= 0) return;
    int g = (int)(((size_t)npad * npad + 255) / 256);
    g = g > 128 ? 128 : g;
    k_tc_split<double><<<dim3(g, nlive), 256, 0, st>>>(src, sstride, out, npad, d_live);
}


}  // namespace mcb

// The expiry test of the bounded waits (see mcbound.h).
extern "C" void mcb_tc_test_expiry(int on) { mcb::g_test_expiry.store(on ? 1 : 0); }
