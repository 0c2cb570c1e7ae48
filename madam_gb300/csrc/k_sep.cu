// k_sep.cu -- cut separation on the GPU.
//
// Triangles (cutting_planes.c:48-127): all 4 * C(n,3) inequalities are
// evaluated; the K most violated above the threshold are selected exactly by a
// two-level radix select on the bit patterns of the (positive) violations, in
// three passes over the triples: (1) 2048-bin histogram + maximum, (2) collect
// the bins above the K-th and histogram the boundary bin on the next 11 bits,
// (3) collect the boundary bin above its K-th sub-bin plus that sub-bin.
// Candidates are packed as (type-1)<<30 | i<<20 | j<<10 | k, whose numeric order
// is the reference's scan order.  X is read as a full symmetric matrix so that
// the inner index k walks down columns (coalesced).
//
// k-gonal inequalities (qap_simulated_annealing.c): one thread per SA run, each
// with its own counter stream; every run is independent, so all
// Pent_Trials*3 + Hepta_Trials*4 runs of all nodes go in one launch.
#include "mcb_dev.cuh"
#include "kernels.h"

namespace mcb {

constexpr int kHistBins = 2048;
constexpr int kShift1 = 45;
constexpr int kSaMaxSweeps = 80;

__device__ __forceinline__ unsigned long long ord_key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// per-slot selection state, in TriSel (device)
struct TriSel {
    unsigned long long maxkey;
    int hist1[kHistBins];
    int hist2[kHistBins];
    int b1, need1, b2, need2, take_all, total;
    int n_out, n_bnd;
};

__device__ __forceinline__ void tri_vals(double a, double b, double c, double v[4]) {
    v[0] = -a - b - c - 1.0;
    v[1] = -a + b + c - 1.0;
    v[2] = a - b + c - 1.0;
    v[3] = a + b - c - 1.0;
}

template <int PASS>
__global__ void __launch_bounds__(256) k_tri_pass(Slot *slots, TriSel *sel, double thr, unsigned int *out,
                                                  double *outv, unsigned int *bnd, double *bndv, int cap_out,
                                                  int cap_bnd) {
    Slot &s = slots[blockIdx.y];
    if (!s.active) return;
    const int n = s.n, ii = blockIdx.x;
    if (ii < 2 || ii >= n) return;
    TriSel &T = sel[blockIdx.y];
    if (PASS > 1 && T.total == 0) return;
    if (PASS == 3 && T.take_all) return;
    __shared__ int hist[kHistBins];
    __shared__ double red[40];
    if (PASS != 3)
        for (int q = threadIdx.x; q < kHistBins; q += blockDim.x) hist[q] = 0;
    __syncthreads();
    const double *X = s.X;
    const unsigned long long base = (unsigned long long)__double_as_longlong(thr);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double vmax = -1e308;
    const int b1 = T.b1, b2 = T.b2, take_all = T.take_all;
    unsigned int *outp = out + (size_t)blockIdx.y * cap_out;
    double *outvp = outv + (size_t)blockIdx.y * cap_out;
    unsigned int *bndp = bnd + (size_t)blockIdx.y * cap_bnd;
    double *bndvp = bndv + (size_t)blockIdx.y * cap_bnd;
    const double *colI = X + (size_t)ii * n;
    for (int jj = 1 + wid; jj < ii; jj += 8) {
        const double a = X[ii + (size_t)jj * n];
        const double *colJ = X + (size_t)jj * n;
        for (int kk = lane; kk < jj; kk += 32) {
            double v[4];
            tri_vals(a, colI[kk], colJ[kk], v);
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (PASS == 1) vmax = fmax(vmax, v[t]);
                if (!(v[t] > thr)) continue;
                unsigned long long rel = (unsigned long long)__double_as_longlong(v[t]) - base;
                int bin = (int)min(rel >> kShift1, (unsigned long long)(kHistBins - 1));
                unsigned int pack = ((unsigned)t << 30) | ((unsigned)ii << 20) | ((unsigned)jj << 10) | (unsigned)kk;
                if (PASS == 1) {
                    atomicAdd(&hist[bin], 1);
                } else if (PASS == 2) {
                    if (take_all || bin > b1) {
                        int at = atomicAdd(&T.n_out, 1);
                        if (at < cap_out) { outp[at] = pack; outvp[at] = v[t]; }
                    } else if (bin == b1) {
                        int sub = (int)((rel >> (kShift1 - 11)) & (kHistBins - 1));
                        atomicAdd(&hist[sub], 1);
                    }
                } else {
                    if (bin == b1) {
                        int sub = (int)((rel >> (kShift1 - 11)) & (kHistBins - 1));
                        if (sub > b2) {
                            int at = atomicAdd(&T.n_out, 1);
                            if (at < cap_out) { outp[at] = pack; outvp[at] = v[t]; }
                        } else if (sub == b2) {
                            int at = atomicAdd(&T.n_bnd, 1);
                            if (at < cap_bnd) { bndp[at] = pack; bndvp[at] = v[t]; }
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (PASS == 1) {
        double m = block_max(vmax, red);
        if (threadIdx.x == 0) atomicMax(&T.maxkey, ord_key(m));
    }
    if (PASS != 3) {
        int *gh = PASS == 1 ? T.hist1 : T.hist2;
        for (int q = threadIdx.x; q < kHistBins; q += blockDim.x)
            if (hist[q]) atomicAdd(&gh[q], hist[q]);
    }
}

__global__ void k_tri_reset(Slot *slots, TriSel *sel) {
    TriSel &T = sel[blockIdx.x];
    for (int q = threadIdx.x; q < kHistBins; q += blockDim.x) {
        T.hist1[q] = 0;
        T.hist2[q] = 0;
    }
    if (threadIdx.x == 0) {
        T.maxkey = ord_key(-kBig);
        T.b1 = T.b2 = 0;
        T.need1 = T.need2 = 0;
        T.take_all = 0;
        T.total = 0;
        T.n_out = T.n_bnd = 0;
    }
}

// level 1 (level = 1) or level 2 (level = 2) bin selection, one thread per slot
__global__ void k_tri_select(Slot *slots, TriSel *sel, int Kdefault, int level) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    TriSel &T = sel[b];
    if (!slots[b].active) return;
    const int K = slots[b].tri_k > 0 ? slots[b].tri_k : Kdefault;  // the slot's own problem's budget
    if (level == 1) {
        int total = 0;
        for (int q = 0; q < kHistBins; ++q) total += T.hist1[q];
        T.total = total;
        if (total <= K) {
            T.take_all = 1;
            return;
        }
        int above = 0, q = kHistBins - 1;
        for (; q >= 0; --q) {
            if (above + T.hist1[q] >= K) break;
            above += T.hist1[q];
        }
        T.b1 = q;
        T.need1 = K - above;
    } else {
        if (T.take_all || T.total == 0) return;
        int above = 0, q = kHistBins - 1;
        for (; q >= 0; --q) {
            if (above + T.hist2[q] >= T.need1) break;
            above += T.hist2[q];
        }
        T.b2 = q;
        T.need2 = T.need1 - above;
    }
}

// ---------------------------------------------------------------------------
// SA: per slot, `runs` runs of the k-gonal annealer.  Run r: type = r % ntypes + 1,
// trial = r / ntypes, stream key = key2(key2(key2(node_key, round), k), trial*8+type).
struct SaJob {
    int slot;        // slot index
    int k;           // 5 or 7
    int runs;
    int ntypes;
    uint64_t key;    // key2(key2(node_key, round), k)
    int out_off;     // first output row of this job
    double sumX;     // filled by k_sa_sumx
};

__global__ void k_sa_sumx(Slot *slots, SaJob *jobs, int njobs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    SaJob &J = jobs[j];
    const Slot &s = slots[J.slot];
    const int n = s.n;
    const double *X = s.X;
    double sumX = 0;
    for (int i = 0; i < n; ++i) {
        sumX += X[i + (size_t)i * n];
        for (int jj = i + 1; jj < n; ++jj) sumX += 2 * fabs(X[jj + (size_t)i * n]);
    }
    J.sumX = sumX;
}

// The SA of one run.  The first K entries of the permutation (the k-set under
// test) and the signs live in registers, selected by unrolled loops rather than
// dynamic indexing (which would put them in local memory); the remaining
// positions stay in the run's global scratch.  Terms are summed in the same
// order as qap_simulated_annealing.c, so the results match the oracle exactly.
template <int K>
__device__ void sa_run(const Slot &s, const SaJob &J, int r, int *perm, int *out, double *out_val) {
    const int n = s.n;
    const double *X = s.X;
    const int type = r % J.ntypes + 1, trial = r / J.ntypes;
    int e[K];
#pragma unroll
    for (int a = 0; a < K; ++a) e[a] = a < type - 1 ? -1 : 1;
    Stream st;
    st.key = key2(J.key, (uint64_t)(trial * 8 + type));
    st.ctr = 0;
    double t = K * K;
    t *= J.sumX;
    t /= (n * (n - 1));
    double cost = kBig;
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int i = n - 1; i > 0; --i) {
        int rr = st.next_int() % i;
        int tmp = perm[i];
        perm[i] = perm[rr];
        perm[rr] = tmp;
    }
    int pk[K], best[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
        pk[i] = perm[i];
        best[i] = pk[i];
    }
    double t1 = t;
    int m1 = n;
    double sol = 0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        sol += X[pk[i] + (size_t)pk[i] * n];
#pragma unroll
        for (int j = i + 1; j < K; ++j) sol += 2 * (e[j] * e[i]) * X[pk[j] + (size_t)pk[i] * n];
    }
    int not_done = 1, sweeps = 0;
    while (not_done > 0) {
        not_done = 0;
        // bound the run time: after 80 sweeps the temperature is 0.6^80 ~ 2e-18 of
        // its start and m1 has grown 2000-fold; real runs stop long before
        if (++sweeps > kSaMaxSweeps) break;
        for (int it = 0; it < m1; ++it) {
            int i1 = st.next_int() % K;
            int i2 = st.next_int() % n;
            if (i2 < i1) { int tmp = i1; i1 = i2; i2 = tmp; }
            // i1 < K always; i2 may lie beyond the prefix
            int p1 = 0, e1 = 0, p2 = 0, e2 = 0;
#pragma unroll
            for (int a = 0; a < K; ++a) {
                if (a == i1) { p1 = pk[a]; e1 = e[a]; }
                if (a == i2) { p2 = pk[a]; e2 = e[a]; }
            }
            if (i2 >= K) p2 = perm[i2];
            double delta = 0.0;
#pragma unroll
            for (int i = 0; i < K; ++i) delta += (e[i] * e1) * (X[pk[i] + (size_t)n * p2] - X[pk[i] + (size_t)n * p1]);
            if (i2 < K)
#pragma unroll
                for (int i = 0; i < K; ++i)
                    delta += (e[i] * e2) * (X[pk[i] + (size_t)n * p1] - X[pk[i] + (size_t)n * p2]);
            delta *= 2.0;
            double tv1 = X[p1 + (size_t)n * p1] + X[p2 + (size_t)n * p2] - 2.0 * X[p2 + (size_t)n * p1];
            double tv2 = 1.0;
            if (i2 < K) tv2 += -2 * (e1 * e2) + 1.0;
            delta += tv1 * tv2;
            if (fabs(delta) < kSaZero) delta = 0.0;
            double sol_temp = sol + delta;
            int accept;
            if (delta > 0) {
                double dt1 = delta / t1;
                if (dt1 > 5) accept = 0;
                else accept = st.next_unit() < exp(-dt1);
            } else {
                accept = 1;
            }
            if (accept) {
                if (fabs(delta) > 0.0001) not_done = 1;
#pragma unroll
                for (int a = 0; a < K; ++a) {
                    if (a == i1) pk[a] = p2;
                    if (a == i2) pk[a] = p1;
                }
                if (i2 >= K) perm[i2] = p1;
                sol = sol_temp;
                if (sol < cost) {
                    cost = sol;
#pragma unroll
                    for (int i = 0; i < K; ++i) best[i] = pk[i];
                }
            }
        }
        t1 *= 0.6;
        m1 = (int)round(m1 * 1.1);
    }
    *out_val = cost;
#pragma unroll
    for (int a = 0; a < K; ++a) out[a] = best[a];
}

__global__ void __launch_bounds__(128) k_sa(Slot *slots, const SaJob *jobs, int njobs, int *perm_scratch,
                                            int nmax, int *out_ineq, double *out_val, int total_runs) {
    int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total_runs) return;
    // locate the job (few jobs: linear scan)
    int jb = 0;
    while (jb + 1 < njobs && jobs[jb + 1].out_off <= gid) ++jb;
    const SaJob &J = jobs[jb];
    const int r = gid - J.out_off;
    const Slot &s = slots[J.slot];
    const int n = s.n, k = J.k;
    int *out = out_ineq + (size_t)gid * 8;
    if (n < k) {
        out_val[gid] = kBig;
        for (int a = 0; a < k; ++a) out[a] = 0;
        return;
    }
    int *perm = perm_scratch + (size_t)gid * nmax;
    if (k == 5) sa_run<5>(s, J, r, perm, out, out_val + gid);
    else sa_run<7>(s, J, r, perm, out, out_val + gid);
}

// ---------------------------------------------------------------------------
size_t trisel_bytes() { return sizeof(TriSel); }
size_t sajob_bytes() { return sizeof(SaJob); }

void launch_tri_separation(Slot *d, int ns, int nmax, void *sel, double thr, int K, unsigned int *out,
                           double *outv, unsigned int *bnd, double *bndv, int cap_out, int cap_bnd,
                           cudaStream_t st) {
    TriSel *T = (TriSel *)sel;
    k_tri_reset<<<ns, 256, 0, st>>>(d, T);
    dim3 g(nmax, ns);
    k_tri_pass<1><<<g, 256, 0, st>>>(d, T, thr, out, outv, bnd, bndv, cap_out, cap_bnd);
    k_tri_select<<<ns, 1, 0, st>>>(d, T, K, 1);
    k_tri_pass<2><<<g, 256, 0, st>>>(d, T, thr, out, outv, bnd, bndv, cap_out, cap_bnd);
    k_tri_select<<<ns, 1, 0, st>>>(d, T, K, 2);
    k_tri_pass<3><<<g, 256, 0, st>>>(d, T, thr, out, outv, bnd, bndv, cap_out, cap_bnd);
}

// host view of the per-slot result header (same leading layout as TriSel)
void tri_sel_readback(const void *sel_host, int slot, double *maxviol, int *take_all, int *need2, int *n_out,
                      int *n_bnd) {
    const TriSel &T = ((const TriSel *)sel_host)[slot];
    unsigned long long k = T.maxkey;
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    memcpy(&v, &b, 8);
    *maxviol = v;
    *take_all = T.take_all;
    *need2 = T.need2;
    *n_out = T.n_out;
    *n_bnd = T.n_bnd;
}

void launch_sa(Slot *d, void *jobs, int njobs, int *perm_scratch, int nmax, int *out_ineq, double *out_val,
               int total_runs, cudaStream_t st) {
    SaJob *J = (SaJob *)jobs;
    k_sa_sumx<<<(njobs + 31) / 32, 32, 0, st>>>(d, J, njobs);
    k_sa<<<(total_runs + 127) / 128, 128, 0, st>>>(d, J, njobs, perm_scratch, nmax, out_ineq, out_val, total_runs);
}

void sajob_fill(void *jobs_host, int idx, int slot, int k, int runs, int ntypes, uint64_t key, int out_off) {
    SaJob &J = ((SaJob *)jobs_host)[idx];
    J.slot = slot;
    J.k = k;
    J.runs = runs;
    J.ntypes = ntypes;
    J.key = key;
    J.out_off = out_off;
    J.sumX = 0;
}

}  // namespace mcb
