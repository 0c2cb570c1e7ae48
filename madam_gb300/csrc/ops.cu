// ops.cu -- operator-level entry points of mcbound.h: one node's worth of device
// memory per call, the same kernels as the batched bound, host pointers in/out.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/mcbound.h"
#include "host_cuts.h"
#include "kernels.h"
#include "mcb_dev.cuh"
#include "ns.h"
#include "tc.h"

using namespace mcb;

namespace {

struct OneSlot {
    Slot h{};
    Slot *d = nullptr;
    std::vector<void *> allocs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T *alloc(size_t count) {
        void *p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (p) allocs.push_back(p);
        return (T *)p;
    }
    explicit OneSlot(int n, int m = 0) {
        size_t NN = (size_t)n * n;
        double *mats = alloc<double>(8 * NN);
        double *vecs = alloc<double>(8 * (size_t)n);
        if (err == cudaSuccess) err = cudaMemset(mats, 0, 8 * NN * sizeof(double));
        h.n = n;
        h.m = m;
        h.active = 1;
        h.L = mats; h.X = mats + NN; h.Q = mats + 2 * NN; h.W = mats + 3 * NN;
        h.A = mats + 4 * NN; h.V = mats + 5 * NN; h.T1 = mats + 6 * NN; h.T2 = mats + 7 * NN;
        h.y = vecs; h.d = vecs + n; h.e = vecs + 2 * n; h.tau = vecs + 3 * n;
        h.ev = vecs + 4 * n; h.vtmp = vecs + 5 * n; h.dy = vecs + 6 * n; h.dy1 = vecs + 7 * n;
        h.acc = alloc<double>(kAcc);
        h.dwork = alloc<double>(eig_dwork_doubles(n));
        d = alloc<Slot>(1);
    }
    cudaError_t push() {
        if (err == cudaSuccess) err = cudaMemcpy(d, &h, sizeof(Slot), cudaMemcpyHostToDevice);
        return err;
    }
    cudaError_t pull() {
        if (err == cudaSuccess) err = cudaMemcpy(&h, d, sizeof(Slot), cudaMemcpyDeviceToHost);
        return err;
    }
    ~OneSlot() {
        for (void *p : allocs) cudaFree(p);
    }
};

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? MCB_OK : MCB_ERR_CUDA; }

int check_dev() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MCB_ERR_NODEV;
    return MCB_OK;
}

CutLists make_lists(int ntri, const int *tri, int npent, const int *pent, int nhept, const int *hept) {
    CutLists c;
    if (ntri) c.tri.assign(tri, tri + 4 * (size_t)ntri);
    if (npent) c.pent.assign(pent, pent + 6 * (size_t)npent);
    if (nhept) c.hept.assign(hept, hept + 8 * (size_t)nhept);
    return c;
}

bool valid_cuts(int n, const CutLists &c) {
    for (size_t a = 0; a < c.tri.size() / 4; ++a) {
        const int *t = &c.tri[4 * a];
        if (!(t[0] > t[1] && t[1] > t[2] && t[2] >= 0 && t[0] < n && t[3] >= 1 && t[3] <= 4)) return false;
    }
    for (size_t a = 0; a < c.pent.size() / 6; ++a) {
        const int *p = &c.pent[6 * a];
        if (p[0] < 1 || p[0] > 3) return false;
        for (int b = 1; b < 6; ++b)
            if (p[b] < 0 || p[b] >= n) return false;
    }
    for (size_t a = 0; a < c.hept.size() / 8; ++a) {
        const int *p = &c.hept[8 * a];
        if (p[0] < 1 || p[0] > 4) return false;
        for (int b = 1; b < 8; ++b)
            if (p[b] < 0 || p[b] >= n) return false;
    }
    return true;
}

// upload a cut system into a OneSlot (cp, B^T incidence)
int upload_one(OneSlot &S, const HostCuts &H) {
    int m = (int)(H.cp.size() / 8);
    S.h.m = m;
    S.h.ne = (int)H.e_idx.size();
    S.h.cp = S.alloc<int>(H.cp.size());
    S.h.e_idx = S.alloc<int>(H.e_idx.size());
    S.h.e_rp = S.alloc<int>(H.e_rp.size());
    S.h.e_cut = S.alloc<int>(H.e_cut.size());
    S.h.e_coef = S.alloc<double>(H.e_coef.size());
    if (S.err) return MCB_ERR_CUDA;
    if (m) {
        cudaMemcpy(S.h.cp, H.cp.data(), H.cp.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(S.h.e_idx, H.e_idx.data(), H.e_idx.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(S.h.e_cut, H.e_cut.data(), H.e_cut.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(S.h.e_coef, H.e_coef.data(), H.e_coef.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(S.h.e_rp, H.e_rp.data(), H.e_rp.size() * sizeof(int), cudaMemcpyHostToDevice);
    return cuda_rc(S.push());
}

// Newton-Schulz form of the projection on one matrix (Xp full, Q lower, M)
int project_ns(OneSlot &S, int n, int proj) {
    NsProj P;
    int rc = P.init(proj & 0xf, n, 1, 0);
    if (rc == MCB_OK && (proj >> 4)) rc = P.configure(((proj >> 4) & 0xf) - 1, P.l0);
    if (rc == MCB_OK) {
        const int npad = P.pad(n);
        rc = P.set_live({0}, {n}, npad, 0);
        if (rc == MCB_OK) launch_ns_prep(S.d, 1, npad, P.stride, P.S, P.Wd, P.d_alpha, 0, 0);
        if (rc == MCB_OK && P.tc()) P.split_inputs(0);
        if (rc == MCB_OK) rc = P.sign(S.d, 1, 0, 0);
        if (rc == MCB_OK) rc = P.product(0);
        if (rc == MCB_OK) launch_ns_post0(S.d, 1, n, P.Gd, npad, P.stride, 0);
        if (rc == MCB_OK && cudaDeviceSynchronize() != cudaSuccess) rc = MCB_ERR_CUDA;
        if (rc == MCB_OK) rc = P.check_error(0);
    }
    P.destroy();
    return rc;
}

}  // namespace

extern "C" {

int mcb_op_B(int n, const double *X, int ntri, const int *tri, int npent, const int *pent, int nhept, const int *hept,
             double *y) {
    if (n < 1 || n > MCB_NMAX || !X || !y || ntri < 0 || npent < 0 || nhept < 0) return MCB_ERR_ARG;
    if ((ntri && !tri) || (npent && !pent) || (nhept && !hept)) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    CutLists cl = make_lists(ntri, tri, npent, pent, nhept, hept);
    if (!valid_cuts(n, cl)) return MCB_ERR_ARG;
    HostCuts H;
    build_host_cuts(cl, n, H);
    OneSlot S(n);
    if (int rc = upload_one(S, H)) return rc;
    int m = cl.m();
    double *dX = S.h.W, *dy = S.alloc<double>(m);
    if (S.err) return MCB_ERR_CUDA;
    cudaMemcpy(dX, X, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    if (m) cudaMemcpy(dy, y, m * sizeof(double), cudaMemcpyHostToDevice);
    launch_op_B(S.d, m, dX, dy, 0);
    if (m) cudaMemcpy(y, dy, m * sizeof(double), cudaMemcpyDeviceToHost);
    return cuda_rc(cudaDeviceSynchronize());
}

int mcb_op_Bt(int n, double *X, int ntri, const int *tri, int npent, const int *pent, int nhept, const int *hept,
              const double *t) {
    if (n < 1 || n > MCB_NMAX || !X || !t || ntri < 0 || npent < 0 || nhept < 0) return MCB_ERR_ARG;
    if ((ntri && !tri) || (npent && !pent) || (nhept && !hept)) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    CutLists cl = make_lists(ntri, tri, npent, pent, nhept, hept);
    if (!valid_cuts(n, cl)) return MCB_ERR_ARG;
    HostCuts H;
    build_host_cuts(cl, n, H);
    OneSlot S(n);
    if (int rc = upload_one(S, H)) return rc;
    int m = cl.m();
    double *dX = S.h.W, *dt = S.alloc<double>(m);
    if (S.err) return MCB_ERR_CUDA;
    cudaMemcpy(dX, X, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    if (m) cudaMemcpy(dt, t, m * sizeof(double), cudaMemcpyHostToDevice);
    launch_op_Bt(S.d, S.h.ne, dX, dt, 0);
    cudaMemcpy(X, dX, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
    return cuda_rc(cudaDeviceSynchronize());
}

int mcb_project_psd(int n, const double *W, int proj, double *Xp, double *Q, double *Z, double *evals, int *M) {
    if (n < 1 || n > MCB_NMAX || !W || !M) return MCB_ERR_ARG;
    const int form = proj & 0xf;
    if (proj & ~0xff) return MCB_ERR_ARG;
    if (form != MCB_PROJ_FP64 && form != MCB_PROJ_NS_BF16 && form != MCB_PROJ_NS_TF32) return MCB_ERR_ARG;
    if (form == MCB_PROJ_FP64 && proj != form) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    OneSlot S(n);
    if (S.push()) return MCB_ERR_CUDA;
    cudaMemcpy(S.h.W, W, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    if (form != MCB_PROJ_FP64) {
        // no eigenvectors in this form: Z and evals are left untouched
        if (int rc = project_ns(S, n, proj)) return rc;
        if (S.pull()) return MCB_ERR_CUDA;
        *M = S.h.M;
        if (Xp) cudaMemcpy(Xp, S.h.X, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
        if (Q) cudaMemcpy(Q, S.h.Q, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
        return cuda_rc(cudaDeviceSynchronize());
    }
    launch_sym_copy(S.d, 1, n, 0, 0, 0);
    launch_tridiag(S.d, 1, n, 0, 0);
    launch_bisect(S.d, 1, n, 1e-8, 0, 0, 0);
    launch_invit(S.d, 1, n, 0, 0);
    launch_backtrans(S.d, 1, n, 0, 0);
    launch_canon_scale(S.d, 1, n, 0, 0);
    launch_syrk_post(S.d, 1, n, 0, nullptr, 0);
    if (cudaDeviceSynchronize() != cudaSuccess || S.pull()) return MCB_ERR_CUDA;
    *M = S.h.M;
    if (Xp) cudaMemcpy(Xp, S.h.X, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (Q) cudaMemcpy(Q, S.h.Q, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (Z && S.h.M > 0) cudaMemcpy(Z, S.h.V, (size_t)n * S.h.M * sizeof(double), cudaMemcpyDeviceToHost);
    if (evals && S.h.M > 0) cudaMemcpy(evals, S.h.ev, S.h.M * sizeof(double), cudaMemcpyDeviceToHost);
    if (S.h.status) return S.h.status;
    return cuda_rc(cudaDeviceSynchronize());
}

int mcb_lambda_max(int n, const double *A, double *lmax, double *lmax_upper) {
    if (n < 1 || n > MCB_NMAX || !A || !lmax) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    OneSlot S(n);
    if (S.push()) return MCB_ERR_CUDA;
    cudaMemcpy(S.h.W, A, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    launch_sym_copy(S.d, 1, n, 0, 0, 0);
    launch_safe_norm(S.d, 1, 0);
    launch_tridiag(S.d, 1, n, 0, 0);
    launch_bisect(S.d, 1, n, 0.0, 1, 0, 0);
    if (cudaDeviceSynchronize() != cudaSuccess || S.pull()) return MCB_ERR_CUDA;
    double acc[kAcc];
    cudaMemcpy(acc, S.h.acc, sizeof(acc), cudaMemcpyDeviceToHost);
    *lmax = S.h.lmax;
    if (lmax_upper) *lmax_upper = acc[ACC_LMAX_HI] + 8.0 * n * 2.220446049250313e-16 * acc[ACC_FNORM];
    return S.h.status ? S.h.status : MCB_OK;
}

int mcb_ipm(int n, const double *L, double *X, double *y, double *Z, double *phi, int *iters) {
    if (n < 1 || n > MCB_NMAX || !L) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    OneSlot S(n);
    if (S.push()) return MCB_ERR_CUDA;
    cudaMemcpy(S.h.L, L, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    launch_ipm_init(S.d, 1, 0);
    double acc[kAcc];
    for (int round = 0; round < 600; ++round) {
        launch_ipm_iteration(S.d, 1, n, 0);
        cudaMemcpy(acc, S.h.acc, sizeof(acc), cudaMemcpyDeviceToHost);
        if (acc[ACC_IPM_DONE] != 0.0) break;
    }
    if (cudaDeviceSynchronize() != cudaSuccess || S.pull()) return MCB_ERR_CUDA;
    if (X) cudaMemcpy(X, S.h.X, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (Z) cudaMemcpy(Z, S.h.Q, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (y) cudaMemcpy(y, S.h.y, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (phi) *phi = acc[ACC_PHI];
    if (iters) *iters = (int)acc[ACC_IPM_IT];
    return S.h.status ? S.h.status : MCB_OK;
}

int mcb_separate_triangles(int n, const double *X, int K, double thr, int *out, double *vals, int *count,
                           double *max_violation) {
    if (n < 1 || n > MCB_NMAX || !X || K < 1 || !out || !count) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    OneSlot S(n);
    const int cap_out = K + 16, cap_bnd = 1 << 16;
    void *sel = S.alloc<unsigned char>(trisel_bytes());
    unsigned int *dout = S.alloc<unsigned int>(cap_out), *dbnd = S.alloc<unsigned int>(cap_bnd);
    double *doutv = S.alloc<double>(cap_out), *dbndv = S.alloc<double>(cap_bnd);
    if (S.err || S.push()) return MCB_ERR_CUDA;
    cudaMemcpy(S.h.W, X, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    launch_sym_copy(S.d, 1, n, 0, 0, 0);
    cudaMemcpy(S.h.X, S.h.A, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToDevice);
    launch_tri_separation(S.d, 1, n, sel, thr, K, dout, doutv, dbnd, dbndv, cap_out, cap_bnd, 0);
    std::vector<unsigned char> hsel(trisel_bytes());
    if (cudaMemcpy(hsel.data(), sel, trisel_bytes(), cudaMemcpyDeviceToHost) != cudaSuccess) return MCB_ERR_CUDA;
    double mv;
    int take_all, need2, n_out, n_bnd;
    tri_sel_readback(hsel.data(), 0, &mv, &take_all, &need2, &n_out, &n_bnd);
    if (n_out > cap_out || n_bnd > cap_bnd) return MCB_ERR_CAPACITY;
    std::vector<unsigned int> pk(n_out + n_bnd);
    std::vector<double> pv(n_out + n_bnd);
    cudaMemcpy(pk.data(), dout, n_out * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(pv.data(), doutv, n_out * 8, cudaMemcpyDeviceToHost);
    std::vector<std::pair<unsigned int, double>> sel_list;
    for (int a = 0; a < n_out; ++a) sel_list.push_back({pk[a], pv[a]});
    if (!take_all && n_bnd) {
        cudaMemcpy(pk.data() + n_out, dbnd, n_bnd * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(pv.data() + n_out, dbndv, n_bnd * 8, cudaMemcpyDeviceToHost);
        std::vector<std::pair<unsigned int, double>> b;
        for (int a = 0; a < n_bnd; ++a) b.push_back({pk[n_out + a], pv[n_out + a]});
        std::sort(b.begin(), b.end(), [](const std::pair<unsigned, double> &x, const std::pair<unsigned, double> &y) {
            if (x.second != y.second) return x.second > y.second;
            return x.first < y.first;
        });
        for (int a = 0; a < need2 && a < n_bnd; ++a) sel_list.push_back(b[a]);
    }
    std::sort(sel_list.begin(), sel_list.end());
    int cnt = (int)sel_list.size();
    for (int a = 0; a < cnt; ++a) {
        unsigned p = sel_list[a].first;
        out[4 * a] = (p >> 20) & 1023;
        out[4 * a + 1] = (p >> 10) & 1023;
        out[4 * a + 2] = p & 1023;
        out[4 * a + 3] = (int)(p >> 30) + 1;
        if (vals) vals[a] = sel_list[a].second;
    }
    *count = cnt;
    if (max_violation) *max_violation = mv;
    return cuda_rc(cudaDeviceSynchronize());
}

int mcb_qap_sa_batch(int n, const double *X, int k, int trials, uint64_t key, int *ineq, double *values) {
    if (n < 2 || n > MCB_NMAX || !X || (k != 5 && k != 7) || trials < 1 || !ineq || !values) return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    OneSlot S(n);
    int ntypes = k == 5 ? 3 : 4, runs = trials * ntypes;
    int *perm = S.alloc<int>((size_t)runs * n), *dout = S.alloc<int>((size_t)runs * 8);
    double *dval = S.alloc<double>(runs);
    void *jobs = S.alloc<unsigned char>(sajob_bytes());
    if (S.err || S.push()) return MCB_ERR_CUDA;
    cudaMemcpy(S.h.X, X, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice);
    std::vector<unsigned char> hj(sajob_bytes());
    sajob_fill(hj.data(), 0, 0, k, runs, ntypes, key, 0);
    cudaMemcpy(jobs, hj.data(), hj.size(), cudaMemcpyHostToDevice);
    launch_sa(S.d, jobs, 1, perm, n, dout, dval, runs, 0);
    std::vector<int> o((size_t)runs * 8);
    cudaMemcpy(o.data(), dout, o.size() * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(values, dval, runs * sizeof(double), cudaMemcpyDeviceToHost);
    for (int r = 0; r < runs; ++r)
        for (int a = 0; a < k; ++a) ineq[(size_t)r * k + a] = o[(size_t)r * 8 + a];
    return cuda_rc(cudaDeviceSynchronize());
}

int mcb_split_gemm(int npad, int batch, const float *A, const float *B, float alpha, float diag, int sym, int variant,
                   float *C) {
    if (npad < kTcTile || npad % kTcTile || npad > 1024 || batch < 1 || batch > 4096 || !A || !B || !C ||
        variant < 0 || variant >= kTcVariants)
        return MCB_ERR_ARG;
    if (int rc = check_dev()) return rc;
    const size_t nn = (size_t)npad * npad, tot = nn * batch;
    std::vector<void *> al;
    cudaError_t e = cudaSuccess;
    auto mk = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&p, bytes);
        if (p) al.push_back(p);
        return p;
    };
    float *dA = (float *)mk(tot * 4), *dB = (float *)mk(tot * 4), *dC = (float *)mk(tot * 4);
    __nv_bfloat16 *pa = (__nv_bfloat16 *)mk(kTcPieces * tot * 2), *pb = (__nv_bfloat16 *)mk(kTcPieces * tot * 2);
    int *live = (int *)mk(batch * sizeof(int)), *nl = (int *)mk(batch * sizeof(int)), *err = (int *)mk(sizeof(int));
    void *maps = mk(6 * tc_map_bytes() + 64);
    int rc = e == cudaSuccess ? MCB_OK : MCB_ERR_NOMEM;
    if (rc == MCB_OK) {
        std::vector<int> l(batch), nv(batch, npad);
        for (int k = 0; k < batch; ++k) l[k] = k;
        cudaMemcpy(dA, A, tot * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, tot * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(live, l.data(), batch * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(nl, nv.data(), batch * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemset(err, 0, sizeof(int));
        // each operand's scale sigma: the smallest power of two >= twice its largest
        // |entry| (the leading digits are then <= 64, and the exact digit-sum groups
        // of the product stay below 2^24 for K <= 1024)
        auto pow2_scale = [&](const float *X) {
            float mx = 0.0f;
            for (size_t i = 0; i < tot; ++i) mx = fmaxf(mx, fabsf(X[i]));
            int e = 0;
            if (mx > 0.0f) frexpf(mx, &e);  // mx = f 2^e with f in [0.5, 1)
            return mx > 0.0f ? ldexpf(1.0f, e + 1) : 1.0f;
        };
        const float sa = pow2_scale(A), sb = pow2_scale(B);
        TcOut oa{nullptr, nullptr, {}, nn, nullptr, 128.0f / sa, nullptr};
        TcOut ob{nullptr, nullptr, {}, nn, nullptr, 128.0f / sb, nullptr};
        for (int p = 0; p < kTcPieces; ++p) {
            oa.p[p] = pa + p * tot;
            ob.p[p] = pb + p * tot;
        }
        tc_split_f32(dA, nn, oa, npad, batch, live, 0);
        tc_split_f32(dB, nn, ob, npad, batch, live, 0);
        // host-side maps (64-byte aligned), passed by value to the kernel
        alignas(64) unsigned char hm[2 * kTcPieces][128];
        for (int p = 0; p < kTcPieces && rc == MCB_OK; ++p) {
            rc = tc_make_map(hm[p], oa.p[p], npad, nn, batch);
            if (rc == MCB_OK) rc = tc_make_map(hm[kTcPieces + p], ob.p[p], npad, nn, batch);
        }
        TcOut oc{dC, nullptr, {}, nn, err, 1.0f, nullptr};
        const float unit = sa * sb / 16384.0f;  // sigma_A sigma_B 2^-14
        if (rc == MCB_OK)
            rc = tc_gemm(hm[0], hm[kTcPieces], oc, npad, batch, live, nl, alpha, diag, unit, 0, sym, variant);
        if (rc == MCB_OK && cudaDeviceSynchronize() != cudaSuccess) rc = MCB_ERR_CUDA;
        int herr = 0;
        if (rc == MCB_OK) cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
        if (rc == MCB_OK && herr) rc = herr;
        if (rc == MCB_OK) cudaMemcpy(C, dC, tot * 4, cudaMemcpyDeviceToHost);
    }
    for (void *p : al) cudaFree(p);
    return rc;
}

}  // extern "C"
