// engine.cu -- host orchestration of the GPU node bound and the C ABI (mcbound.h).
//
// A context holds the original problem (SP->L) resident on the device and a
// fixed number of node slots.  mcb_bound_batch runs MADAM's SDPbound
// (bounding.c:25-250) for up to batch_max nodes in lockstep: every phase (IPM,
// separation, ADMM iterations, safe bound) is one batched launch over the
// slots that are still live; the host keeps the control flow of bounding.c,
// the cut lists (purge / dedup / append of cutting_planes.c) and the GW + 1-opt
// heuristic (heuristic.c), which runs on host threads on the GPU's factor.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/mcbound.h"
#include "host_cuts.h"
#include "kernels.h"
#include "mcb_dev.cuh"
#include "ns.h"
#include "tc.h"
#include "learn.h"
#include "mlp.h"

using namespace mcb;

namespace {

const char *kClassNames[] = {"subproblem", "ipm",   "admm_rhs", "cg",        "admm_su", "build_W",
                             "sym_copy",   "tridiag", "bisect", "invit",     "backtrans", "canon_scale",
                             "syrk_post",  "admm_bx", "admm_finish", "safe_bound", "tri_sep", "sa",
                             "ns_prep",    "ns_gemm", "ns_fp64", "heur_gpu", "learned"};
// unit of mcb_ctx::work per class: 1 = FP64 flops, 2 = bytes, 3 = tensor-core GEMM
// flops (the Newton-Schulz steps, low-precision and FP32-accurate), 0 = not counted
const int kWorkUnit[] = {0, 0, 2, 0, 0, 2, 2, 1, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 2, 3, 1, 0, 0};
enum KClass { K_SUB, K_IPM, K_RHS, K_CG, K_SU, K_W, K_SYMC, K_TRID, K_BIS, K_INV, K_BACK, K_CANON, K_SYRK,
              K_BX, K_FIN, K_SAFE, K_TRI, K_SA, K_NSPREP, K_NSGEMM, K_NSREF, K_HEUR, K_LEARN, K_NCLASS };

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct SlotMem {
    // fixed-size
    double *mats = nullptr;  // 8 * Nmax^2
    double *vecs = nullptr;  // 8 * Nmax
    double *acc = nullptr;
    double *dwork = nullptr;
    // growable
    size_t mcap = 0, gcap = 0, ecap = 0, eicap = 0;
    int *cp = nullptr;
    double *cutd = nullptr;  // 8 * mcap: t s u v rhs cgr cgp cgq
    int *g_rp = nullptr, *g_ci = nullptr;
    double *g_v = nullptr;
    float *g_v32 = nullptr;
    size_t g32cap = 0;
    int *e_idx = nullptr, *e_rp = nullptr, *e_cut = nullptr;
    double *e_coef = nullptr;
};

// A node's cuts at the end of its bound, in global vertex ids (original
// variables; N - 1 for the subproblem's last vertex), with the features of the
// learned models taken at the node's final X and the cut's final dual.
struct NodeRecord {
    std::vector<int> k, type, verts;   // verts: 7 per cut
    std::vector<float> feats;          // kCutFeatures per cut
    std::vector<double> dual;          // final dual s_c
    std::vector<double> pred;          // warm-start dual predicted for the children (learned form)
    size_t size() const { return k.size(); }
};

// the warm start handed to a child: the parent's record and the branching variable
struct WarmIn {
    std::shared_ptr<NodeRecord> rec;
    int ic = -1;
};

// One problem of the context (MADAM's SP and the globals SDPbound reads and writes
// for it): SP->L, the incumbent (Bab_LBGet / Bab_LBUpd, heap.c:15,185), diff
// (bounding.c:241-243) and the k-gonal trial counts (bounding.c:184-187).
struct Problem {
    int N = 0, pb = 0;
    std::vector<double> SL;  // host copy, N x N column-major
    double *d_SL = nullptr;  // device copy
    double LB = 0.0;
    std::vector<int> best_sol;
    double diff = 0.0;
    int pent_trials = 0, hepta_trials = 0;
    int tri_ineq = 0;  // TriIneq (10 N under adjust_TriIneq, process_input.c:122-123)
};

struct NodeRun : CutLists {
    Problem *P = nullptr;  // the node's problem
    mcb_bab_node *node = nullptr;
    int n = 0;
    double fixedvalue = 0, f = 0, basic_bound = 0, bound = 0, oldf = 0, sigma = 0, tol = 0;
    double viol3 = 0, viol5 = 0;
    uint64_t key = 0;
    int count = 0, nbit = 0, nbit_total = 0, ipm_iters = 0;
    int done = 0, prune = 0, giveup = 0, sep_round = 0, heur_calls = 0, M = 0, status = 0;
    std::vector<double> tri_y, pent_y, hept_y;
    std::vector<double> Lsub;          // n x n subproblem matrix (host copy for the heuristic)
    std::vector<double> Zf;            // n x M factor of the last projection (times sqrt(sigma))
    std::vector<unsigned char> signs;  // Newton-Schulz form: hyperplane signs (n x N, 1 = negative)
    bool heur_gpu = false;             // this round's heuristic already ran on the GPU (x, hval set)
    std::vector<int> U;                // subproblem vertex -> original variable (n - 1 entries)
    std::vector<float> pend_F;         // logged cut-scorer features of the last separated triangles
    std::vector<int> pend_pos;         // ... and their positions in tri
    std::vector<int> x;                // heuristic result (BabPbSize)
    double hval = -kBig;
};

}  // namespace

struct mcb_ctx {
    mcb_params prm;
    int N = 0, batch_max = 0, flags = 0;  // N: the order the slots hold (problem 0's)
    // the problems: 0 from mcb_create, more from mcb_add_problem (order <= N)
    std::vector<Problem> probs;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::mutex lb_mu;
    // slots
    std::vector<Slot> hs;
    Slot *d_slots = nullptr;
    std::vector<SlotMem> mem;
    // shared device buffers
    double *d_partials = nullptr;
    int *d_lists = nullptr;
    int list_stride = 0;
    double *d_fixed = nullptr;
    void *d_trisel = nullptr;
    std::vector<unsigned char> h_trisel;
    unsigned int *d_tout = nullptr, *d_tbnd = nullptr;
    double *d_toutv = nullptr, *d_tbndv = nullptr;
    int tcap_out = 0, tcap_bnd = 0;
    void *d_sajobs = nullptr;
    std::vector<unsigned char> h_sajobs;
    int *d_perm = nullptr, *d_saout = nullptr;
    double *d_saval = nullptr;
    size_t sa_cap = 0;
    // Newton-Schulz projection (chosen form)
    int proj = MCB_PROJ_FP64;
    NsProj ns;
    int *d_hlist = nullptr;
    unsigned long long *d_hkeys = nullptr;
    unsigned char *d_hsign = nullptr;
    double *d_hval = nullptr;
    // learned models (not owned) and the training logs
    mcb_mlp *scorer = nullptr, *warm = nullptr;
    std::vector<float> log_x[2], log_y[2];
    std::map<const mcb_bab_node *, WarmIn> warm_in;           // set by the B&B driver
    std::vector<std::shared_ptr<NodeRecord>> last_records;    // per node of the last bound_batch
    int *d_fslot = nullptr, *d_fcp = nullptr;
    double *d_fextra = nullptr;
    float *d_F = nullptr, *d_pred = nullptr;
    size_t fcap = 0;
    // CUDA graph of one ADMM chunk (replayed while its launch configuration holds)
    cudaGraphExec_t gexec = nullptr;
    std::vector<int> gkey;
    long long g_dl[64] = {};
    double g_dw[64] = {};
    long long graph_launches = 0, graph_captures = 0;
    // host-side wall time per phase of bound_batch (seconds)
    double host_s[8] = {};
    // mcb_bab: wall-time limit (0 = none) and, after a run the node or time limit
    // stopped, the largest bound among the open nodes and their count
    int cg_max_iters = 2000;       // CG iterations per solve of (B B^T + I) t = rhs
    double bab_time_limit = 0.0;
    double bab_open_bound = -1e308;
    int bab_open_nodes = 0;
    // instrumentation
    long long h2d = 0, d2h = 0;        // host<->device bytes moved by the bound calls
    long long lib_launches = 0;        // cuBLAS launches (not counted as own kernels)
    double work[K_NCLASS] = {};        // algorithmic work per class (flops or bytes, see kWorkUnit)
    long long launches[K_NCLASS] = {};
    double ms[K_NCLASS] = {};
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> ev_pool;
    std::string err;
};

namespace {

const char *kHostNames[] = {"ipm", "cut_upload", "admm", "safe_bound", "heuristic", "separation", "records", "other"};
enum HostPhase { H_IPM, H_CUTS, H_ADMM, H_SAFE, H_HEUR, H_SEP, H_REC, H_OTHER, H_N };
struct HostTimer {
    double *acc;
    std::chrono::steady_clock::time_point t0;
    explicit HostTimer(double *a) : acc(a), t0(std::chrono::steady_clock::now()) {}
    ~HostTimer() { *acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

// host -> device copy on the context's stream (the source must outlive the copy)
cudaError_t h2d(mcb_ctx *c, void *dst, const void *src, size_t bytes) {
    c->h2d += (long long)bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->st);
}
// device -> host copy on the context's stream, complete when this returns
cudaError_t d2h(mcb_ctx *c, void *dst, const void *src, size_t bytes) {
    c->d2h += (long long)bytes;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(c->st);
}

int set_err(mcb_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

#define CUDA_TRY(c, expr)                                                                         \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return set_err((c), MCB_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_)); \
    } while (0)

// --- instrumentation -------------------------------------------------------
cudaEvent_t get_event(mcb_ctx *c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

struct Prof {
    mcb_ctx *c;
    int cls;
    cudaEvent_t a = nullptr, b = nullptr;
    Prof(mcb_ctx *c_, int cls_, int nkernels) : c(c_), cls(cls_) {
        c->launches[cls] += nkernels;
        if (c->flags & MCB_FLAG_PROFILE) {
            a = get_event(c);
            b = get_event(c);
            cudaEventRecord(a, c->st);
        }
    }
    ~Prof() {
        if (a) {
            cudaEventRecord(b, c->st);
            c->pending.push_back({cls, {a, b}});
        }
    }
};

void flush_prof(mcb_ctx *c) {
    if (c->pending.empty()) return;
    cudaStreamSynchronize(c->st);
    for (auto &p : c->pending) {
        float t = 0;
        cudaEventElapsedTime(&t, p.second.first, p.second.second);
        c->ms[p.first] += t;
        c->ev_pool.push_back(p.second.first);
        c->ev_pool.push_back(p.second.second);
    }
    c->pending.clear();
}

// --- device memory ----------------------------------------------------------
int alloc_slot(mcb_ctx *c, int si) {
    SlotMem &M = c->mem[si];
    Slot &s = c->hs[si];
    const size_t NN = (size_t)c->N * c->N, N = c->N;
    CUDA_TRY(c, cudaMalloc(&M.mats, 8 * NN * sizeof(double)));
    CUDA_TRY(c, cudaMalloc(&M.vecs, 8 * N * sizeof(double)));
    CUDA_TRY(c, cudaMalloc(&M.acc, kAcc * sizeof(double)));
    CUDA_TRY(c, cudaMalloc(&M.dwork, eig_dwork_doubles(c->N) * sizeof(double)));
    CUDA_TRY(c, cudaMemset(M.mats, 0, 8 * NN * sizeof(double)));
    memset(&s, 0, sizeof(Slot));
    s.L = M.mats; s.X = M.mats + NN; s.Q = M.mats + 2 * NN; s.W = M.mats + 3 * NN;
    s.A = M.mats + 4 * NN; s.V = M.mats + 5 * NN; s.T1 = M.mats + 6 * NN; s.T2 = M.mats + 7 * NN;
    s.y = M.vecs; s.d = M.vecs + N; s.e = M.vecs + 2 * N; s.tau = M.vecs + 3 * N;
    s.ev = M.vecs + 4 * N; s.vtmp = M.vecs + 5 * N; s.dy = M.vecs + 6 * N; s.dy1 = M.vecs + 7 * N;
    s.acc = M.acc;
    s.dwork = M.dwork;
    return MCB_OK;
}

// (re)allocate a pair of device arrays with a common capacity when `need` exceeds it
template <typename A, typename B>
int grow2(mcb_ctx *c, A *&a, B *&b, size_t &cap, size_t need, size_t extra_b = 0) {
    if (need <= cap && a && b) return MCB_OK;
    size_t nc = std::max<size_t>({need, cap * 2, 1024});
    if (a) cudaFree(a);
    if (b) cudaFree(b);
    a = nullptr;
    b = nullptr;
    CUDA_TRY(c, cudaMalloc(&a, nc * sizeof(A)));
    CUDA_TRY(c, cudaMalloc(&b, (nc + extra_b) * sizeof(B)));
    cap = nc;
    return MCB_OK;
}

int ensure_cut_capacity(mcb_ctx *c, int si, int m, size_t nnz_g, size_t ne, size_t nnz_e) {
    SlotMem &M = c->mem[si];
    Slot &s = c->hs[si];
    int rc;
    if ((size_t)m > M.mcap || !M.cp) {
        size_t nc = std::max<size_t>({(size_t)m, M.mcap * 2, 4096});
        if (M.cp) cudaFree(M.cp);
        if (M.cutd) cudaFree(M.cutd);
        if (M.g_rp) cudaFree(M.g_rp);
        M.cp = nullptr;
        M.cutd = nullptr;
        M.g_rp = nullptr;
        CUDA_TRY(c, cudaMalloc(&M.cp, nc * 8 * sizeof(int)));
        CUDA_TRY(c, cudaMalloc(&M.cutd, nc * 8 * sizeof(double)));
        CUDA_TRY(c, cudaMalloc(&M.g_rp, (nc + 1) * sizeof(int)));
        M.mcap = nc;
    }
    if ((rc = grow2(c, M.g_ci, M.g_v, M.gcap, nnz_g))) return rc;
    if (nnz_g > M.g32cap || !M.g_v32) {
        if (M.g_v32) cudaFree(M.g_v32);
        M.g_v32 = nullptr;
        CUDA_TRY(c, cudaMalloc(&M.g_v32, M.gcap * sizeof(float)));
        M.g32cap = M.gcap;
    }
    if ((rc = grow2(c, M.e_idx, M.e_rp, M.eicap, ne + 1, 1))) return rc;
    if ((rc = grow2(c, M.e_cut, M.e_coef, M.ecap, nnz_e + 1))) return rc;
    size_t mc = M.mcap;
    s.cp = M.cp;
    s.t = M.cutd; s.s = M.cutd + mc; s.u = M.cutd + 2 * mc; s.v = M.cutd + 3 * mc;
    s.rhs = M.cutd + 4 * mc; s.cgr = M.cutd + 5 * mc; s.cgp = M.cutd + 6 * mc; s.cgq = M.cutd + 7 * mc;
    s.g_rp = M.g_rp; s.g_ci = M.g_ci; s.g_v = M.g_v; s.g_v32 = M.g_v32;
    s.e_idx = M.e_idx; s.e_rp = M.e_rp; s.e_cut = M.e_cut; s.e_coef = M.e_coef;
    return MCB_OK;
}

void free_slot(SlotMem &M) {
    void *ps[] = {M.mats, M.vecs, M.acc, M.dwork, M.cp, M.cutd, M.g_rp, M.g_ci, M.g_v, M.g_v32, M.e_idx, M.e_rp, M.e_cut,
                  M.e_coef};
    for (void *p : ps)
        if (p) cudaFree(p);
    M = SlotMem();
}

int upload_slots(mcb_ctx *c, int ns) {
    CUDA_TRY(c, h2d(c, c->d_slots, c->hs.data(), ns * sizeof(Slot)));
    return MCB_OK;
}
int download_slots(mcb_ctx *c, int ns) {
    CUDA_TRY(c, d2h(c, c->hs.data(), c->d_slots, ns * sizeof(Slot)));
    CUDA_TRY(c, cudaStreamSynchronize(c->st));
    return MCB_OK;
}

// upload one slot's cut system and reset its ADMM state (admm.c:78-95)
// every vertex index of every cut inside [0, n), triangles ordered i > j > k
bool cuts_valid(const NodeRun &r) {
    const int n = r.n;
    for (size_t a = 0; a < r.tri.size(); a += 4) {
        const int *t = &r.tri[a];
        if (!(t[0] < n && t[0] > t[1] && t[1] > t[2] && t[2] >= 0 && t[3] >= 1 && t[3] <= 4)) return false;
    }
    for (size_t a = 0; a < r.pent.size(); a += 6)
        for (int b = 1; b < 6; ++b)
            if (r.pent[a + b] < 0 || r.pent[a + b] >= n || r.pent[a] < 1 || r.pent[a] > 3) return false;
    for (size_t a = 0; a < r.hept.size(); a += 8)
        for (int b = 1; b < 8; ++b)
            if (r.hept[a + b] < 0 || r.hept[a + b] >= n || r.hept[a] < 1 || r.hept[a] > 4) return false;
    return true;
}

int upload_cuts(mcb_ctx *c, int si, NodeRun &r, const HostCuts &H) {
    int m = r.m();
    int rc = ensure_cut_capacity(c, si, m, H.g_ci.size() + 1, H.e_idx.size(), H.e_cut.size());
    if (rc != MCB_OK) return rc;
    Slot &s = c->hs[si];
    s.m = m;
    s.ne = (int)H.e_idx.size();
    std::vector<double> y0;
    y0.reserve(m);
    y0.insert(y0.end(), r.tri_y.begin(), r.tri_y.end());
    y0.insert(y0.end(), r.pent_y.begin(), r.pent_y.end());
    y0.insert(y0.end(), r.hept_y.begin(), r.hept_y.end());
    cudaStream_t st = c->st;
    if (m > 0) {
        CUDA_TRY(c, h2d(c, s.cp, H.cp.data(), H.cp.size() * sizeof(int)));
        CUDA_TRY(c, h2d(c, s.t, y0.data(), m * sizeof(double)));
        CUDA_TRY(c, h2d(c, s.s, y0.data(), m * sizeof(double)));
        CUDA_TRY(c, cudaMemsetAsync(s.u, 0, m * sizeof(double), st));
        CUDA_TRY(c, h2d(c, s.g_ci, H.g_ci.data(), H.g_ci.size() * sizeof(int)));
        CUDA_TRY(c, h2d(c, s.g_v, H.g_v.data(), H.g_v.size() * sizeof(double)));
        CUDA_TRY(c, h2d(c, s.e_cut, H.e_cut.data(), H.e_cut.size() * sizeof(int)));
        CUDA_TRY(c, h2d(c, s.e_coef, H.e_coef.data(), H.e_coef.size() * sizeof(double)));
        CUDA_TRY(c, h2d(c, s.e_idx, H.e_idx.data(), H.e_idx.size() * sizeof(int)));
    }
    CUDA_TRY(c, h2d(c, s.g_rp, H.g_rp.data(), H.g_rp.size() * sizeof(int)));
    CUDA_TRY(c, h2d(c, s.e_rp, H.e_rp.data(), H.e_rp.size() * sizeof(int)));
    // keep the host vectors alive until the copies finish
    CUDA_TRY(c, cudaStreamSynchronize(st));
    return MCB_OK;
}

// --- projection + one ADMM iteration -----------------------------------------
void launch_projection(mcb_ctx *c, int ns, int gate) {
    Slot *d = c->d_slots;
    int N = c->N;
    { Prof p(c, K_SYMC, 1); launch_sym_copy(d, ns, N, 0, gate, c->st); }
    { Prof p(c, K_TRID, 1); launch_tridiag(d, ns, N, gate, c->st); }
    { Prof p(c, K_BIS, 1); launch_bisect(d, ns, N, 1e-8, 0, gate, c->st); }
    { Prof p(c, K_INV, 1); launch_invit(d, ns, N, gate, c->st); }
    { Prof p(c, K_BACK, 1); launch_backtrans(d, ns, N, gate, c->st); }
    { Prof p(c, K_CANON, 1); launch_canon_scale(d, ns, N, gate, c->st); }
}

// the Newton-Schulz projection of every live slot, X+ into the ADMM epilogue
int launch_ns_projection(mcb_ctx *c, int ns) {
    Slot *d = c->d_slots;
    NsProj &P = c->ns;
    {
        Prof p(c, K_NSPREP, P.tc() ? 3 : 2);
        launch_ns_prep(d, ns, P.npad, P.stride, P.S, P.Wd, P.d_alpha, 1, c->st);
        if (P.tc()) P.split_inputs(c->st);
    }
    double lo = P.flops_lo, hi = P.flops_hi, f64 = P.flops_fp64;
    int rc;
    {
        // tcgen05 path: two own GEMM kernels per step and the closing trace; cuBLAS
        // paths: one diagonal update per step and the closing conversion, the GEMMs
        // are cuBLAS launches, counted apart
        Prof p(c, K_NSGEMM, (P.tc() ? 2 : 1) * (int)P.steps.size() + 1);
        rc = P.sign(d, ns, 1, c->st);
        if (!P.tc()) c->lib_launches += 2 * (long long)P.steps.size();
    }
    if (rc) return set_err(c, rc, "cuBLAS GEMM of the Newton-Schulz step failed");
    {
        Prof p(c, K_NSREF, P.tc() ? 1 : 0);
        rc = P.product(c->st);
        if (!P.tc()) c->lib_launches += 1;
    }
    if (rc) return set_err(c, rc, "cuBLAS FP64 GEMM of the projection failed");
    c->work[K_NSGEMM] += (P.flops_lo - lo) + (P.flops_hi - hi);
    c->work[K_NSREF] += P.flops_fp64 - f64;
    c->work[K_NSPREP] += 8.0 * (double)P.live * P.npad * P.npad * 2.5;
    { Prof p(c, K_SYRK, 2); launch_ns_post(d, ns, c->N, c->d_partials, P.Gd, P.npad, P.stride, c->st); }
    return MCB_OK;
}

int launch_admm_iteration(mcb_ctx *c, int ns, int mmax, int emax) {
    Slot *d = c->d_slots;
    int N = c->N;
    { Prof p(c, K_RHS, 1); launch_admm_rhs(d, ns, N, mmax, c->st); }
    {
        // the plain form solves to 1e-13 (the reference's direct factorisation agrees
        // to rounding); the Newton-Schulz forms carry projection errors of ~5e-9 of
        // ||W||, so a 1e-10 solve stays below them
        Prof p(c, K_CG, 1);
        launch_cg(d, ns, mmax, c->cg_max_iters, c->proj == MCB_PROJ_FP64 ? 1e-13 : 1e-10, c->st);
    }
    { Prof p(c, K_SU, 1); launch_admm_su(d, ns, mmax, c->st); }
    { Prof p(c, K_W, 2); launch_build_W(d, ns, N, emax, 0, c->st); }
    if (c->proj == MCB_PROJ_FP64) {
        launch_projection(c, ns, 1);
        { Prof p(c, K_SYRK, 2); launch_syrk_post(d, ns, N, 1, c->d_partials, c->st); }
    } else {
        int rc = launch_ns_projection(c, ns);
        if (rc) return rc;
    }
    { Prof p(c, K_BX, 1); launch_admm_bx(d, ns, mmax, c->st); }
    { Prof p(c, K_FIN, 1); launch_admm_finish(d, ns, c->prm.scaleSigma, c->prm.ADMM_itermax, c->st); }
    return MCB_OK;
}

// `chunk` ADMM iterations.  Without profiling, the launch sequence is captured
// once into a CUDA graph per launch configuration (batch size, cut and edge
// counts, padded order and live slots of the tensor-core path) and replayed:
// every kernel reads the slot state from device memory, so a replay is the same
// work as the launches.  cuBLAS operand modes launch directly.
int run_chunk(mcb_ctx *c, int ns, int mmax, int emax, int chunk) {
    const bool graph = !(c->flags & MCB_FLAG_PROFILE) &&
                       (c->proj == MCB_PROJ_FP64 || c->ns.tc());
    if (!graph) {
        for (int k = 0; k < chunk; ++k)
            if (int rc = launch_admm_iteration(c, ns, mmax, emax)) return rc;
        return MCB_OK;
    }
    std::vector<int> key{ns, mmax, emax, chunk, c->proj, c->ns.npad, c->ns.live, c->ns.variant, c->ns.version,
                         c->cg_max_iters, tc_test_expiry()};
    if (!c->gexec || key != c->gkey) {
        long long l0[K_NCLASS];
        double w0[K_NCLASS];
        memcpy(l0, c->launches, sizeof(l0));
        memcpy(w0, c->work, sizeof(w0));
        cudaGraph_t g = nullptr;
        CUDA_TRY(c, cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        int rc = MCB_OK;
        for (int k = 0; k < chunk && rc == MCB_OK; ++k) rc = launch_admm_iteration(c, ns, mmax, emax);
        cudaError_t e = cudaStreamEndCapture(c->st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return set_err(c, MCB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        if (c->gexec) cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return set_err(c, MCB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        for (int i = 0; i < K_NCLASS; ++i) {
            c->g_dl[i] = c->launches[i] - l0[i];
            c->g_dw[i] = c->work[i] - w0[i];
        }
        c->gkey = key;
        c->graph_captures++;
    } else {
        // the counts of a replay are those recorded at capture
        for (int i = 0; i < K_NCLASS; ++i) {
            c->launches[i] += c->g_dl[i];
            c->work[i] += c->g_dw[i];
        }
    }
    CUDA_TRY(c, cudaGraphLaunch(c->gexec, c->st));
    c->graph_launches++;
    return MCB_OK;
}

// --- heuristic (heuristic.c), counter streams --------------------------------
double eval_solution(const Problem &P, const int *sol) {
    double v = 0.0;
    const int N = P.N, pb = P.pb;
    for (int i = 0; i < pb; ++i)
        for (int j = 0; j < pb; ++j) v += P.SL[j + (size_t)i * N] * sol[i] * sol[j];
    return v;
}

void mc_1opt(int *x, const double *L, int N, std::vector<double> &Lx, std::vector<double> &d,
             std::vector<double> &delta, std::vector<int> &I) {
    for (int i = 0; i < N; ++i) {
        double a = 0.0;
        for (int j = 0; j < N; ++j) a += L[j + (size_t)i * N] * x[j];
        Lx[i] = a;
    }
    for (int i = 0; i < N; ++i) {
        d[i] = L[i + (size_t)i * N];
        delta[i] = d[i] - x[i] * Lx[i];
    }
    double best = -kBig;
    int index = 0;
    for (int i = 0; i < N; ++i)
        if (delta[i] > best) { best = delta[i]; index = i; }
    while (best > 0.001) {
        int nI = 0;
        for (int j = 0; j < N; ++j)
            if (fabs(L[index + (size_t)N * j]) > 0.001) I[nI++] = j;
        if (x[index] > 0)
            for (int q = 0; q < nI; ++q) Lx[I[q]] -= 2 * L[index + (size_t)I[q] * N];
        else
            for (int q = 0; q < nI; ++q) Lx[I[q]] += 2 * L[index + (size_t)I[q] * N];
        x[index] *= -1;
        for (int i = 0; i < N; ++i) delta[i] = d[i] - x[i] * Lx[i];
        best = -kBig;
        index = 0;
        for (int i = 0; i < N; ++i)
            if (delta[i] > best) { best = delta[i]; index = i; }
    }
}

// GW_heuristic with P0->n hyperplanes (heuristic.c:24-91); result into r.x / r.hval
void run_heuristic(const mcb_ctx *c, NodeRun &r) {
    (void)c;
    const int N = r.n, M = r.M, num = r.P->N, pb = r.P->pb;
    std::vector<int> tx(N), sol(pb);
    std::vector<double> v(M > 0 ? M : 1), Lx(N), d(N), delta(N);
    std::vector<int> I(N);
    double best = -kBig;
    r.x.assign(pb, 0);
    for (int i = 0; i < pb; ++i) r.x[i] = r.node->xfixed[i] ? r.node->sol[i] : 0;
    for (int count = 0; count < num; ++count) {
        Stream st;
        st.key = key2(key2(r.key, 0x48455552ull + (uint64_t)r.heur_calls), (uint64_t)count);
        st.ctr = 0;
        if (!r.signs.empty()) {
            // Newton-Schulz form: signs of X v computed on the GPU
            const unsigned char *sg = &r.signs[(size_t)count * N];
            for (int i = 0; i < N; ++i) tx[i] = sg[i] ? -1 : 1;
        } else {
            for (int i = 0; i < M; ++i) v[i] = st.next_unit() - 0.5;
            for (int i = 0; i < N; ++i) {
                double sca = 0.0;
                for (int j = 0; j < M; ++j) sca += v[j] * r.Zf[(size_t)j * N + i];
                tx[i] = sca < 0 ? -1 : 1;
            }
        }
        mc_1opt(tx.data(), r.Lsub.data(), N, Lx, d, delta, I);
        int index = 0;
        for (int i = 0; i < pb; ++i) {
            if (r.node->xfixed[i]) sol[i] = r.node->sol[i];
            else sol[i] = (tx[index++] + 1) / 2;
        }
        double hv = eval_solution(*r.P, sol.data());
        if (best < hv) {
            r.x = sol;
            best = hv;
        }
        if (M == 0) {
            // every hyperplane gives the same all-ones start: the remaining
            // num-1 repetitions cannot change the result
            break;
        }
    }
    r.hval = best;
    r.heur_calls++;
}

void run_heuristics(mcb_ctx *c, std::vector<NodeRun *> &all) {
    if (all.empty()) return;
    std::vector<NodeRun *> rs;
    for (auto *r : all)
        if (!r->heur_gpu) rs.push_back(r);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    unsigned nt = std::min<unsigned>(hw, (unsigned)rs.size());
    if (nt <= 1) {
        for (auto *r : rs) run_heuristic(c, *r);
    } else {
        std::atomic<size_t> next{0};
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&] {
                size_t i;
                while ((i = next.fetch_add(1)) < rs.size()) run_heuristic(c, *rs[i]);
            });
        for (auto &t : th) t.join();
    }
    // updateSolution in slot order (bab_functions.c:114-134)
    for (auto *r : all) {
        r->heur_gpu = false;
        if (r->hval > r->P->LB) {
            r->P->LB = r->hval;
            r->P->best_sol = r->x;
        }
    }
}

// --- learned models: features on the GPU, optional prediction ------------------
// F (host, ncut x kCutFeatures) for cuts cps (8 ints each) of slots slot_of, and
// pred = model(F) when a model is given
int cut_features(mcb_ctx *c, const std::vector<int> &slot_of, const std::vector<int> &cps,
                 const std::vector<double> *extra, mcb_mlp *model, std::vector<float> *F, std::vector<float> *pred) {
    const size_t nc = slot_of.size();
    if (F) F->clear();
    if (pred) pred->clear();
    if (nc == 0) return MCB_OK;
    if (nc > c->fcap) {
        void *ps[] = {c->d_fslot, c->d_fcp, c->d_fextra, c->d_F, c->d_pred};
        for (void *q : ps)
            if (q) cudaFree(q);
        size_t cap = std::max<size_t>(nc, 2 * c->fcap);
        CUDA_TRY(c, cudaMalloc(&c->d_fslot, cap * sizeof(int)));
        CUDA_TRY(c, cudaMalloc(&c->d_fcp, cap * 8 * sizeof(int)));
        CUDA_TRY(c, cudaMalloc(&c->d_fextra, cap * sizeof(double)));
        CUDA_TRY(c, cudaMalloc(&c->d_F, cap * kCutFeatures * sizeof(float)));
        CUDA_TRY(c, cudaMalloc(&c->d_pred, cap * sizeof(float)));
        c->fcap = cap;
    }
    CUDA_TRY(c, h2d(c, c->d_fslot, slot_of.data(), nc * sizeof(int)));
    CUDA_TRY(c, h2d(c, c->d_fcp, cps.data(), nc * 8 * sizeof(int)));
    if (extra) CUDA_TRY(c, h2d(c, c->d_fextra, extra->data(), nc * sizeof(double)));
    {
        Prof p(c, K_LEARN, model ? 2 : 1);
        launch_cut_features(c->d_slots, c->d_fslot, c->d_fcp, (int)nc, extra ? c->d_fextra : nullptr, c->d_F,
                            c->st);
        if (model) mlp_forward_device(mlp_impl(model), c->d_F, (int)nc, c->d_pred, c->st);
    }
    if (F) {
        F->resize(nc * kCutFeatures);
        CUDA_TRY(c, d2h(c, F->data(), c->d_F, F->size() * sizeof(float)));
    }
    if (pred && model) {
        pred->resize(nc);
        CUDA_TRY(c, d2h(c, pred->data(), c->d_pred, nc * sizeof(float)));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->st));
    return MCB_OK;
}

void tri_key_to_cp(unsigned int key, int *cp) {
    int t[4] = {(int)((key >> 20) & 1023), (int)((key >> 10) & 1023), (int)(key & 1023), (int)(key >> 30) + 1};
    encode_cut(3, t, cp);
}

// --- separation --------------------------------------------------------------
int separate_triangles(mcb_ctx *c, int ns, std::vector<NodeRun *> &runs, std::vector<int> &want) {
    // learned ranking: the 2K most violated candidates, ranked by the scorer; K is
    // the budget of each node's own problem
    const bool learned = (c->flags & MCB_FLAG_LEARNED) && c->scorer;
    int Kc = 0;
    for (int si = 0; si < ns; ++si) {
        c->hs[si].active = want[si];
        c->hs[si].tri_k = (learned ? 2 : 1) * runs[si]->P->tri_ineq;
        Kc = std::max(Kc, c->hs[si].tri_k);
    }
    int rc = upload_slots(c, ns);
    if (rc) return rc;
    {
        Prof p(c, K_TRI, 6);
        launch_tri_separation(c->d_slots, ns, c->N, c->d_trisel, c->prm.violated_TriIneq, Kc, c->d_tout, c->d_toutv,
                              c->d_tbnd, c->d_tbndv, c->tcap_out, c->tcap_bnd, c->st);
    }
    CUDA_TRY(c, d2h(c, c->h_trisel.data(), c->d_trisel, ns * trisel_bytes()));
    CUDA_TRY(c, cudaStreamSynchronize(c->st));
    std::vector<unsigned int> pk;
    std::vector<double> pv;
    for (int si = 0; si < ns; ++si) {
        if (!want[si]) continue;
        NodeRun &r = *runs[si];
        const int K = r.P->tri_ineq;
        double maxv;
        int take_all, need2, n_out, n_bnd;
        tri_sel_readback(c->h_trisel.data(), si, &maxv, &take_all, &need2, &n_out, &n_bnd);
        if (n_out > c->tcap_out || n_bnd > c->tcap_bnd)
            return set_err(c, MCB_ERR_CAPACITY, "triangle candidate buffer overflow");
        pk.resize(n_out + n_bnd);
        pv.resize(n_out + n_bnd);
        if (n_out) {
            CUDA_TRY(c, d2h(c, pk.data(), c->d_tout + (size_t)si * c->tcap_out, n_out * 4));
            CUDA_TRY(c, d2h(c, pv.data(), c->d_toutv + (size_t)si * c->tcap_out, n_out * 8));
        }
        std::vector<std::pair<unsigned int, double>> sel;
        sel.reserve(Kc);
        for (int a = 0; a < n_out; ++a) sel.push_back({pk[a], pv[a]});
        if (!take_all && n_bnd) {
            std::vector<std::pair<unsigned int, double>> b(n_bnd);
            std::vector<unsigned int> bk(n_bnd);
            std::vector<double> bv(n_bnd);
            CUDA_TRY(c, d2h(c, bk.data(), c->d_tbnd + (size_t)si * c->tcap_bnd, n_bnd * 4));
            CUDA_TRY(c, d2h(c, bv.data(), c->d_tbndv + (size_t)si * c->tcap_bnd, n_bnd * 8));
            for (int a = 0; a < n_bnd; ++a) b[a] = {bk[a], bv[a]};
            std::sort(b.begin(), b.end(), [](const std::pair<unsigned, double> &x, const std::pair<unsigned, double> &y) {
                if (x.second != y.second) return x.second > y.second;
                return x.first < y.first;
            });
            for (int a = 0; a < need2 && a < n_bnd; ++a) sel.push_back(b[a]);
        }
        if (learned && (int)sel.size() > K) {
            std::vector<int> so(sel.size(), si), cps(sel.size() * 8);
            for (size_t a = 0; a < sel.size(); ++a) tri_key_to_cp(sel[a].first, &cps[8 * a]);
            std::vector<float> pred;
            int rc2 = cut_features(c, so, cps, nullptr, c->scorer, nullptr, &pred);
            if (rc2) return rc2;
            std::vector<int> ord(sel.size());
            for (size_t a = 0; a < ord.size(); ++a) ord[a] = (int)a;
            std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
                if (pred[x] != pred[y]) return pred[x] > pred[y];
                if (sel[x].second != sel[y].second) return sel[x].second > sel[y].second;
                return sel[x].first < sel[y].first;
            });
            std::vector<std::pair<unsigned int, double>> top;
            for (int a = 0; a < K; ++a) top.push_back(sel[ord[a]]);
            sel.swap(top);
        }
        std::sort(sel.begin(), sel.end());
        // updateTriangleInequalities, cutting_planes.c:132-214 (purge already done by the caller)
        std::unordered_set<uint64_t> have;
        have.reserve(r.tri.size() / 4 * 2 + 16);
        for (size_t a = 0; a < r.tri.size() / 4; ++a) {
            const int *t = &r.tri[4 * a];
            have.insert(((uint64_t)(t[3] - 1) << 30) | ((uint64_t)t[0] << 20) | ((uint64_t)t[1] << 10) | (uint64_t)t[2]);
        }
        size_t next = r.tri.size() / 4;
        const size_t first_new = next;
        std::vector<int> so, cps;
        for (auto &e : sel) {
            if (next == MCB_MAX_TRI) break;
            if (have.count(e.first)) continue;
            int type = (int)(e.first >> 30) + 1, i = (e.first >> 20) & 1023, j = (e.first >> 10) & 1023, k = e.first & 1023;
            r.tri.insert(r.tri.end(), {i, j, k, type});
            r.tri_y.push_back(0.0);
            if (c->flags & MCB_FLAG_LOG) {
                so.push_back(si);
                cps.resize(cps.size() + 8);
                tri_key_to_cp(e.first, &cps[cps.size() - 8]);
            }
            ++next;
        }
        if ((c->flags & MCB_FLAG_LOG) && !so.empty()) {
            // features at separation time; the targets are the duals after the next ADMM call
            std::vector<float> F;
            int rc2 = cut_features(c, so, cps, nullptr, nullptr, &F, nullptr);
            if (rc2) return rc2;
            r.pend_F = F;
            r.pend_pos.clear();
            for (size_t a = 0; a < so.size(); ++a) r.pend_pos.push_back((int)(first_new + a));
        }
        r.viol3 = maxv;
    }
    return MCB_OK;
}

// k-gonal separation for the slots in want5 / want7 (cutting_planes.c:224-409, 419-605)
int separate_kgonal(mcb_ctx *c, int ns, std::vector<NodeRun *> &runs, std::vector<int> &want5,
                    std::vector<int> &want7, const std::vector<int> &yoff5, const std::vector<int> &yoff7) {
    (void)yoff5;
    (void)yoff7;
    struct Job { int slot, k, runs, off; };
    std::vector<Job> jobs;
    int total = 0;
    for (int si = 0; si < ns; ++si) {
        if (want5[si] && runs[si]->n >= 5) {
            int rr = runs[si]->P->pent_trials * 3;
            jobs.push_back({si, 5, rr, total});
            total += rr;
        }
        if (want7[si] && runs[si]->n >= 7) {
            int rr = runs[si]->P->hepta_trials * 4;
            jobs.push_back({si, 7, rr, total});
            total += rr;
        }
    }
    if (total > 0) {
        if ((size_t)total > c->sa_cap) {
            if (c->d_perm) cudaFree(c->d_perm);
            if (c->d_saout) cudaFree(c->d_saout);
            if (c->d_saval) cudaFree(c->d_saval);
            c->d_perm = nullptr; c->d_saout = nullptr; c->d_saval = nullptr;
            size_t cap = std::max<size_t>(total, 2 * c->sa_cap);
            CUDA_TRY(c, cudaMalloc(&c->d_perm, cap * c->N * sizeof(int)));
            CUDA_TRY(c, cudaMalloc(&c->d_saout, cap * 8 * sizeof(int)));
            CUDA_TRY(c, cudaMalloc(&c->d_saval, cap * sizeof(double)));
            c->sa_cap = cap;
        }
        c->h_sajobs.resize(jobs.size() * sajob_bytes());
        for (size_t a = 0; a < jobs.size(); ++a) {
            NodeRun &r = *runs[jobs[a].slot];
            uint64_t key = key2(key2(r.key, (uint64_t)r.sep_round), (uint64_t)jobs[a].k);
            sajob_fill(c->h_sajobs.data(), (int)a, jobs[a].slot, jobs[a].k, jobs[a].runs, jobs[a].k == 5 ? 3 : 4, key,
                       jobs[a].off);
        }
        if (c->d_sajobs) cudaFree(c->d_sajobs);
        c->d_sajobs = nullptr;
        CUDA_TRY(c, cudaMalloc(&c->d_sajobs, c->h_sajobs.size()));
        CUDA_TRY(c, h2d(c, c->d_sajobs, c->h_sajobs.data(), c->h_sajobs.size()));
        {
            Prof p(c, K_SA, 2);
            launch_sa(c->d_slots, c->d_sajobs, (int)jobs.size(), c->d_perm, c->N, c->d_saout, c->d_saval, total, c->st);
        }
    }
    std::vector<int> ineq((size_t)total * 8);
    std::vector<double> val(total);
    if (total > 0) {
        CUDA_TRY(c, d2h(c, ineq.data(), c->d_saout, (size_t)total * 8 * sizeof(int)));
        CUDA_TRY(c, d2h(c, val.data(), c->d_saval, (size_t)total * sizeof(double)));
        CUDA_TRY(c, cudaStreamSynchronize(c->st));
    }
    for (int si = 0; si < ns; ++si) {
        for (int k : {5, 7}) {
            bool want = k == 5 ? want5[si] : want7[si];
            if (!want) continue;
            NodeRun &r = *runs[si];
            std::vector<int> &cuts = k == 5 ? r.pent : r.hept;
            std::vector<double> &cy = k == 5 ? r.pent_y : r.hept_y;
            int stride = k + 1, cap = k == 5 ? c->prm.PentIneq : c->prm.HeptaIneq;
            int maxcuts = k == 5 ? MCB_MAX_PENT : MCB_MAX_HEPT;
            double minAll = kBig;
            std::vector<int> list;
            std::vector<double> lv;
            int least = 0;
            double leastv = -kBig;
            const Job *jb = nullptr;
            for (auto &j : jobs)
                if (j.slot == si && j.k == k) jb = &j;
            if (jb) {
                for (int rr = 0; rr < jb->runs; ++rr) {
                    int g = jb->off + rr;
                    double v = val[g];
                    int type = rr % (k == 5 ? 3 : 4) + 1;
                    minAll = v < minAll ? v : minAll;
                    if (!(v < 1.0)) continue;
                    int size = (int)lv.size();
                    if (size < cap) {
                        list.push_back(type);
                        for (int a = 0; a < k; ++a) list.push_back(ineq[(size_t)g * 8 + a]);
                        lv.push_back(v);
                        if (size == 0 || v > leastv) { leastv = v; least = size; }
                    } else if (v < leastv) {
                        list[(size_t)stride * least] = type;
                        for (int a = 0; a < k; ++a) list[(size_t)stride * least + 1 + a] = ineq[(size_t)g * 8 + a];
                        lv[least] = v;
                        leastv = kBig;
                        for (int q = 0; q < size; ++q)
                            if (lv[q] > leastv) { leastv = lv[q]; least = q; }
                    }
                }
            }
            // dedup against the kept cuts only (as the reference), append with y = 0
            size_t kept = cuts.size() / stride, next = kept;
            for (size_t l = 0; l < lv.size(); ++l) {
                if (next == (size_t)maxcuts) break;
                const int *cand = &list[stride * l];
                bool found = false;
                for (size_t q = 0; q < kept && !found; ++q)
                    found = memcmp(&cuts[stride * q], cand, stride * sizeof(int)) == 0;
                if (!found) {
                    cuts.insert(cuts.end(), cand, cand + stride);
                    cy.push_back(0.0);
                    ++next;
                }
            }
            if (k == 5) r.viol5 = minAll;
        }
    }
    return MCB_OK;
}

// training pairs of the cut scorer: features at separation -> log(1 + dual after the ADMM call)
void log_scorer_targets(mcb_ctx *c, NodeRun &r, const std::vector<double> &s) {
    if (!(c->flags & MCB_FLAG_LOG)) return;
    for (size_t a = 0; a < r.pend_pos.size(); ++a) {
        size_t pos = (size_t)r.pend_pos[a];
        if (pos >= s.size()) continue;
        c->log_x[0].insert(c->log_x[0].end(), r.pend_F.begin() + a * kCutFeatures,
                           r.pend_F.begin() + (a + 1) * kCutFeatures);
        c->log_y[0].push_back((float)log1p(std::max(s[pos], 0.0)));
    }
    r.pend_F.clear();
    r.pend_pos.clear();
}

// purge cuts whose dual s is below 1e-5 (cutting_planes.c:144-166 and analogues)
void purge(NodeRun &r, const std::vector<double> &s) {
    size_t nt = r.tri.size() / 4, np = r.pent.size() / 6, nh = r.hept.size() / 8;
    auto fam = [&](std::vector<int> &cuts, std::vector<double> &cy, size_t cnt, int stride, size_t off) {
        size_t next = 0;
        for (size_t q = 0; q < cnt; ++q) {
            double yq = s[off + q];
            if (yq < 1e-5) continue;
            if (next != q) memmove(&cuts[stride * next], &cuts[stride * q], stride * sizeof(int));
            cy[next] = yq;
            ++next;
        }
        cuts.resize(stride * next);
        cy.resize(next);
    };
    fam(r.tri, r.tri_y, nt, 4, 0);
    fam(r.pent, r.pent_y, np, 6, nt);
    fam(r.hept, r.hept_y, nh, 8, nt + np);
}

void store_fracsol(const mcb_ctx *c, NodeRun &r, const std::vector<double> &lastrow) {
    (void)c;
    int index = 0;
    for (int i = 0; i < r.P->pb; ++i) {
        if (r.node->xfixed[i]) r.node->fracsol[i] = (double)r.node->sol[i];
        else r.node->fracsol[i] = 0.5 * (lastrow[index++] + 1.0);
    }
}

int fetch_lastrow(mcb_ctx *c, int si, int n, std::vector<double> &row) {
    row.resize(n);
    // last row of X: X[(n-1) + i n]
    c->d2h += (long long)n * sizeof(double);
    CUDA_TRY(c, cudaMemcpy2DAsync(row.data(), sizeof(double), c->hs[si].X + (n - 1), (size_t)n * sizeof(double),
                                  sizeof(double), n, cudaMemcpyDeviceToHost, c->st));
    CUDA_TRY(c, cudaStreamSynchronize(c->st));
    return MCB_OK;
}

uint64_t node_key(const int *xfixed, const int *sol, int pb) {
    uint64_t h = 0x4D414441u;
    for (int i = 0; i < pb; ++i)
        if (xfixed[i]) h = key2(h, (uint64_t)(2 * i + (sol[i] ? 1 : 0)));
    return h;
}

// Newton-Schulz form: the heuristic's hyperplane signs sign(X v) for every node in
// hrun, computed on the GPU (the library's tcgen05 GEMM) and copied to r.signs
int ns_hyperplanes(mcb_ctx *c, std::vector<NodeRun *> &runs, std::vector<NodeRun *> &hrun) {
    std::vector<int> list;
    std::vector<unsigned long long> keys;
    int nm = 1, nh = 1;
    for (size_t q = 0; q < hrun.size(); ++q) {
        NodeRun *r = hrun[q];
        int si = -1;
        for (size_t k = 0; k < runs.size(); ++k)
            if (runs[k] == r) si = (int)k;
        if (r->M == 0) { r->signs.clear(); continue; }  // X+ = 0: all-ones start, as the plain form
        list.push_back(si);
        keys.push_back(key2(r->key, 0x48455552ull + (uint64_t)r->heur_calls));
        nm = std::max(nm, r->n);
        nh = std::max(nh, r->P->N);
    }
    if (list.empty()) return MCB_OK;
    // as many hyperplanes as the largest listed problem's order; each node keeps its own N
    const int count = nh, k = (int)list.size();
    const size_t ostride = (size_t)c->N * c->N;
    CUDA_TRY(c, h2d(c, c->d_hlist, list.data(), k * sizeof(int)));
    CUDA_TRY(c, h2d(c, c->d_hkeys, keys.data(), k * sizeof(unsigned long long)));
    int rc;
    {
        // tcgen05 path: X, the normals, their planes, the product and the signs;
        // the cuBLAS operand modes take a cuBLAS GEMM (counted apart) instead
        Prof p(c, K_HEUR, c->ns.tc() ? 6 : 3);
        if (!c->ns.tc()) c->lib_launches += 1;
        rc = c->ns.hyperplanes(c->d_slots, list, c->d_hlist, c->d_hkeys, count, (nm + 15) / 16 * 16, c->d_hsign,
                               ostride, c->st);
    }
    if (rc) return set_err(c, rc, "hyperplane GEMM failed");
    // the 1-opt of every hyperplane and the cut values, on the GPU; the host keeps
    // the first best hyperplane (heuristic.c's strict comparison) per node
    {
        Prof p(c, K_HEUR, 1);
        launch_heur_1opt(c->d_slots, c->d_hlist, k, count, c->d_lists, c->list_stride, c->d_hsign, ostride, c->d_hval,
                         c->st);
    }
    std::vector<double> hv((size_t)k * count);
    CUDA_TRY(c, d2h(c, hv.data(), c->d_hval, hv.size() * sizeof(double)));
    std::vector<unsigned char> best;
    for (int q = 0; q < k; ++q) {
        NodeRun &r = *runs[list[q]];
        int bi = 0;
        for (int h = 1; h < r.P->N; ++h)
            if (hv[(size_t)q * count + h] > hv[(size_t)q * count + bi]) bi = h;
        best.resize(r.n);
        CUDA_TRY(c, d2h(c, best.data(), c->d_hsign + (size_t)q * ostride + (size_t)bi * r.n, r.n));
        r.x.assign(r.P->pb, 0);
        int idx = 0;
        for (int i = 0; i < r.P->pb; ++i) {
            if (r.node->xfixed[i]) r.x[i] = r.node->sol[i];
            else r.x[i] = best[idx++] ? 0 : 1;
        }
        r.hval = hv[(size_t)q * count + bi];
        r.heur_calls++;
        r.heur_gpu = true;
        r.signs.clear();
    }
    return MCB_OK;
}

// the parent's final cuts mapped into the child's subproblem (cuts through the
// branching variable dropped), with the warm model's predicted duals as y0
void apply_warm_start(mcb_ctx *c, NodeRun &r) {
    auto it = c->warm_in.find(r.node);
    if (it == c->warm_in.end() || !it->second.rec) return;
    const NodeRecord &P = *it->second.rec;
    if (P.pred.size() != P.size()) return;
    std::vector<int> loc(r.P->N, -1);
    for (size_t v = 0; v < r.U.size(); ++v) loc[r.U[v]] = (int)v;
    loc[r.P->N - 1] = r.n - 1;
    for (size_t q = 0; q < P.size(); ++q) {
        const int k = P.k[q];
        int v[7];
        bool ok = true;
        for (int a = 0; a < k && ok; ++a) {
            v[a] = loc[P.verts[7 * q + a]];
            ok = v[a] >= 0;
        }
        double y0 = expm1(std::max((double)P.pred[q], 0.0));
        if (!ok || y0 < 1e-5) continue;
        if (k == 3) {
            if ((int)(r.tri.size() / 4) >= MCB_MAX_TRI) continue;
            r.tri.insert(r.tri.end(), {v[0], v[1], v[2], P.type[q]});
            r.tri_y.push_back(y0);
        } else if (k == 5) {
            if ((int)(r.pent.size() / 6) >= MCB_MAX_PENT) continue;
            r.pent.push_back(P.type[q]);
            r.pent.insert(r.pent.end(), v, v + 5);
            r.pent_y.push_back(y0);
        } else {
            if ((int)(r.hept.size() / 8) >= MCB_MAX_HEPT) continue;
            r.hept.push_back(P.type[q]);
            r.hept.insert(r.hept.end(), v, v + 7);
            r.hept_y.push_back(y0);
        }
    }
}

// the node's final record (cuts with dual >= 1e-5 of its last ADMM call, features
// at its final X, the warm model's predictions when loaded)
int make_record(mcb_ctx *c, int si, NodeRun &r, std::shared_ptr<NodeRecord> &out) {
    out = std::make_shared<NodeRecord>();
    const int m = r.m();
    if (m == 0 || r.count == 0) return MCB_OK;
    std::vector<double> sv(m);
    CUDA_TRY(c, d2h(c, sv.data(), c->hs[si].s, m * sizeof(double)));
    log_scorer_targets(c, r, sv);
    NodeRecord &R = *out;
    std::vector<int> so, cps;
    std::vector<double> ex;
    auto glob = [&](int v) { return v == r.n - 1 ? r.P->N - 1 : r.U[v]; };
    auto add = [&](int k, int type, const int *v, double dual) {
        R.k.push_back(k);
        R.type.push_back(type);
        for (int a = 0; a < 7; ++a) R.verts.push_back(a < k ? glob(v[a]) : 0);
        R.dual.push_back(dual);
        int cp[8], raw[8];
        if (k == 3) { raw[0] = v[0]; raw[1] = v[1]; raw[2] = v[2]; raw[3] = type; }
        else { raw[0] = type; for (int a = 0; a < k; ++a) raw[1 + a] = v[a]; }
        encode_cut(k, raw, cp);
        so.push_back(si);
        cps.insert(cps.end(), cp, cp + 8);
        ex.push_back(dual);
    };
    size_t q = 0;
    for (size_t a = 0; a < r.tri.size() / 4; ++a, ++q)
        if (sv[q] >= 1e-5) add(3, r.tri[4 * a + 3], &r.tri[4 * a], sv[q]);
    for (size_t a = 0; a < r.pent.size() / 6; ++a, ++q)
        if (sv[q] >= 1e-5) add(5, r.pent[6 * a], &r.pent[6 * a + 1], sv[q]);
    for (size_t a = 0; a < r.hept.size() / 8; ++a, ++q)
        if (sv[q] >= 1e-5) add(7, r.hept[8 * a], &r.hept[8 * a + 1], sv[q]);
    std::vector<float> pred;
    mcb_mlp *model = (c->flags & MCB_FLAG_LEARNED) ? c->warm : nullptr;
    int rc = cut_features(c, so, cps, &ex, model, &R.feats, model ? &pred : nullptr);
    if (rc) return rc;
    if (model) R.pred.assign(pred.begin(), pred.end());
    return MCB_OK;
}

// --- the batched SDPbound ----------------------------------------------------
int bound_batch(mcb_ctx *c, mcb_bab_node *const *nodes, const int *probs, int count, int rank, double *bounds,
                mcb_node_stats *stats) {
    auto t0 = std::chrono::steady_clock::now();
    auto t_last = t0;
    // wall time since the previous tick goes to `phase`
    auto tick = [&](int phase) {
        auto t = std::chrono::steady_clock::now();
        c->host_s[phase] += std::chrono::duration<double>(t - t_last).count();
        t_last = t;
    };
    const int N = c->N;
    const mcb_params &P = c->prm;
    int rc;
    std::vector<NodeRun> R(count);
    std::vector<NodeRun *> runs(count);
    std::vector<int> lists((size_t)count * c->list_stride, 0);
    for (int si = 0; si < count; ++si) {
        NodeRun &r = R[si];
        runs[si] = &r;
        r.node = nodes[si];
        r.P = &c->probs[probs ? probs[si] : 0];
        const int pb = r.P->pb;
        int *ls = &lists[(size_t)si * c->list_stride];
        std::vector<int> U, F1, FX, FS;
        for (int i = 0; i < pb; ++i) {
            if (!r.node->xfixed[i]) U.push_back(i);
            else {
                if (r.node->sol[i] == 1) F1.push_back(i);
                FX.push_back(i);
                FS.push_back(r.node->sol[i]);
            }
        }
        ls[0] = (int)U.size(); ls[1] = (int)F1.size(); ls[2] = (int)FX.size();
        int *p = ls + 3;
        for (int v : U) *p++ = v;
        for (int v : F1) *p++ = v;
        for (int v : FX) *p++ = v;
        for (int v : FS) *p++ = v;
        r.n = (int)U.size() + 1;
        r.U = U;
        r.key = node_key(r.node->xfixed, r.node->sol, pb);
        r.sigma = P.sigma0;
        r.tol = P.tol0;
        Slot &s = c->hs[si];
        s.SL = r.P->d_SL; s.N = r.P->N;
        s.n = r.n; s.m = 0; s.ne = 0; s.active = 1; s.M = 0; s.sigma = r.sigma; s.tol = r.tol;
        s.nbit = 0; s.stop = 0; s.status = 0;
    }
    // the k-gonal trial growth of give-ups (bounding.c:184-187), per problem, applied after the batch
    std::map<Problem *, std::pair<int, int>> pend;
    const int ns = count;
    CUDA_TRY(c, h2d(c, c->d_lists, lists.data(), lists.size() * sizeof(int)));
    if ((rc = upload_slots(c, ns))) return rc;
    { Prof p(c, K_SUB, 1); launch_subproblem(c->d_slots, ns, c->d_lists, c->list_stride, c->d_fixed, c->st); }
    std::vector<double> fixedv(ns);
    CUDA_TRY(c, d2h(c, fixedv.data(), c->d_fixed, ns * sizeof(double)));
    // IPM (ipm_mc_pk.c), batched until every slot has converged
    { Prof p(c, K_IPM, 1); launch_ipm_init(c->d_slots, ns, c->st); }
    std::vector<double> acc((size_t)ns * kAcc);
    for (int round = 0; round < 200; ++round) {
        for (int k = 0; k < 3; ++k) { Prof p(c, K_IPM, 6); launch_ipm_iteration(c->d_slots, ns, N, c->st); }
        bool all = true;
        for (int si = 0; si < ns; ++si)
            CUDA_TRY(c, d2h(c, &acc[(size_t)si * kAcc], c->hs[si].acc, kAcc * sizeof(double)));
        CUDA_TRY(c, cudaStreamSynchronize(c->st));
        for (int si = 0; si < ns; ++si) all = all && acc[(size_t)si * kAcc + ACC_IPM_DONE] != 0.0;
        if (all) break;
    }
    if ((rc = download_slots(c, ns))) return rc;
    for (int si = 0; si < ns; ++si) {
        NodeRun &r = R[si];
        r.fixedvalue = fixedv[si];
        r.f = acc[(size_t)si * kAcc + ACC_PHI];
        r.ipm_iters = (int)acc[(size_t)si * kAcc + ACC_IPM_IT];
        if (c->hs[si].status) r.status = c->hs[si].status;
        r.basic_bound = r.f + r.fixedvalue;
        r.Lsub.resize((size_t)r.n * r.n);
        CUDA_TRY(c, d2h(c, r.Lsub.data(), c->hs[si].L, r.Lsub.size() * sizeof(double)));
    }
    std::vector<double> row;
    for (int si = 0; si < ns; ++si) {
        if ((rc = fetch_lastrow(c, si, R[si].n, row))) return rc;
        store_fracsol(c, R[si], row);
    }
    tick(H_IPM);
    // first heuristic: empty factor (M = 0), then prune / give-up tests (bounding.c:88-114)
    run_heuristics(c, runs);
    tick(H_HEUR);
    std::vector<int> want(ns, 0);
    for (int si = 0; si < ns; ++si) {
        NodeRun &r = R[si];
        r.bound = r.f + r.fixedvalue;
        if (r.status) { r.done = 1; continue; }
        if (r.bound < r.P->LB + 1.0) { r.prune = 1; r.done = 1; continue; }
        if (P.use_diff && rank != 0 && r.bound > r.P->LB + r.P->diff + 1.0) { r.giveup = 1; r.done = 1; continue; }
        want[si] = 1;
    }
    if ((c->flags & MCB_FLAG_LEARNED) && c->warm)
        for (int si = 0; si < ns; ++si)
            if (want[si]) apply_warm_start(c, R[si]);
    if ((rc = separate_triangles(c, ns, runs, want))) return rc;
    for (int si = 0; si < ns; ++si)
        if (want[si]) R[si].sep_round++;
    tick(H_SEP);
    // outer loop (bounding.c:121-236), in lockstep
    std::vector<double> sbuf;
    while (true) {
        std::vector<int> live(ns, 0);
        int nlive = 0;
        for (int si = 0; si < ns; ++si) live[si] = !R[si].done, nlive += live[si];
        if (!nlive) break;
        int mmax = 0, emax = 0;
        // the per-node sparse structures (B^T incidence, B B^T + I) on host threads
        std::vector<HostCuts> HC(ns);
        {
            std::vector<int> todo;
            for (int si = 0; si < ns; ++si)
                if (live[si]) {
                    if (!cuts_valid(R[si])) return set_err(c, MCB_ERR_NUMERIC, "cut list holds an out-of-range vertex index");
                    todo.push_back(si);
                }
            std::atomic<size_t> next{0};
            auto work = [&] {
                size_t q;
                while ((q = next.fetch_add(1)) < todo.size()) build_host_cuts(R[todo[q]], R[todo[q]].n, HC[todo[q]]);
            };
            unsigned nt = std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)todo.size());
            std::vector<std::thread> th;
            for (unsigned t = 1; t < nt; ++t) th.emplace_back(work);
            work();
            for (auto &t : th) t.join();
        }
        for (int si = 0; si < ns; ++si) {
            Slot &s = c->hs[si];
            s.active = live[si];
            if (!live[si]) continue;
            NodeRun &r = R[si];
            r.count++;
            r.oldf = r.f;
            if ((rc = upload_cuts(c, si, r, HC[si]))) return rc;
            s.sigma = r.sigma;
            s.tol = r.tol;
            s.nbit = 0;
            s.stop = 0;
            mmax = std::max(mmax, s.m);
            emax = std::max(emax, s.ne);
        }
        if ((rc = upload_slots(c, ns))) return rc;
        launch_cg_values(c->d_slots, ns, c->st);  // FP32 copy of B B^T + I for the inner CG
        tick(H_CUTS);
        // ADMM_solver (admm.c:49-771): chunks of iterations until every live slot stopped
        for (int it = 0; it < P.ADMM_itermax + 8;) {
            const int chunk = 8;
            std::vector<int> nb0(ns);
            for (int si = 0; si < ns; ++si) nb0[si] = c->hs[si].nbit;
            if (c->proj != MCB_PROJ_FP64) {
                std::vector<int> lv, ln;
                int nm = 1;
                for (int si = 0; si < ns; ++si)
                    if (live[si] && !c->hs[si].stop) {
                        lv.push_back(si);
                        ln.push_back(c->hs[si].n);
                        nm = std::max(nm, c->hs[si].n);
                    }
                if ((rc = c->ns.set_live(lv, ln, c->ns.pad(nm), c->st)))
                    return set_err(c, rc, "live-slot upload or TMA descriptors");
            }
            if ((rc = run_chunk(c, ns, mmax, emax, chunk))) return rc;
            it += chunk;
            if ((rc = download_slots(c, ns))) return rc;
            if (c->proj != MCB_PROJ_FP64 && (rc = c->ns.check_error(c->st)))
                return set_err(c, rc, "a tensor-core wait expired");
            for (int si = 0; si < ns; ++si) {
                if (!live[si]) continue;
                const Slot &s2 = c->hs[si];
                double iters = s2.nbit - nb0[si], n3 = (double)s2.n, Mx = (double)s2.M;
                c->work[K_TRID] += iters * 4.0 / 3.0 * n3 * n3 * n3;
                c->work[K_BACK] += iters * 2.0 * n3 * n3 * Mx;
                c->work[K_SYRK] += iters * n3 * (n3 + 1.0) * Mx;
                c->work[K_W] += iters * (24.0 * n3 * (n3 + 1.0) / 2.0 + 20.0 * s2.ne);
                c->work[K_SYMC] += iters * (8.0 * n3 * (n3 + 1.0) / 2.0 + 8.0 * n3 * n3);
                c->work[K_RHS] += iters * (8.0 * n3 * 4.0 + 32.0 * s2.m + 3.0 * 8.0 * 10.0 * s2.m);
            }
            bool all = true;
            for (int si = 0; si < ns; ++si)
                if (live[si] && !c->hs[si].stop) all = false;
            if (all) break;
        }
        tick(H_ADMM);
        // safe bound
        {
            Prof p(c, K_SAFE, 6);
            launch_build_W(c->d_slots, ns, N, emax, 1, c->st);
            launch_safe_norm(c->d_slots, ns, c->st);
            launch_tridiag(c->d_slots, ns, N, 0, c->st);
            launch_bisect(c->d_slots, ns, N, 0.0, 1, 0, c->st);
            launch_safe_finish(c->d_slots, ns, c->st);
        }
        if ((rc = download_slots(c, ns))) return rc;
        for (int si = 0; si < ns; ++si) {
            if (!live[si]) continue;
            CUDA_TRY(c, d2h(c, &acc[(size_t)si * kAcc], c->hs[si].acc, kAcc * sizeof(double)));
        }
        CUDA_TRY(c, cudaStreamSynchronize(c->st));
        tick(H_SAFE);
        std::vector<NodeRun *> hrun;
        for (int si = 0; si < ns; ++si) {
            if (!live[si]) continue;
            NodeRun &r = R[si];
            Slot &s = c->hs[si];
            if (s.status) { r.status = s.status; r.done = 1; continue; }
            r.nbit = s.nbit;
            r.nbit_total += s.nbit;
            r.sigma = s.sigma;
            r.f = s.f;
            r.M = s.M;
            r.tol = r.tol * P.scaleTol;
            if (r.tol < P.minTol) r.tol = P.minTol;
            r.bound = r.f + r.fixedvalue;
            r.prune = r.bound < r.P->LB + 1.0;
            if (!r.prune) {
                if (c->proj == MCB_PROJ_FP64) {
                    double sg = acc[(size_t)si * kAcc + ACC_SIGMA_LAST];
                    r.Zf.resize((size_t)r.n * r.M);
                    if (r.M > 0) {
                        CUDA_TRY(c, d2h(c, r.Zf.data(), s.V, r.Zf.size() * sizeof(double)));
                        double sca = sqrt(sg);
                        for (auto &z : r.Zf) z *= sca;
                    }
                }
                hrun.push_back(&r);
            }
        }
        if (c->proj != MCB_PROJ_FP64 && !hrun.empty())
            if ((rc = ns_hyperplanes(c, runs, hrun))) return rc;
        run_heuristics(c, hrun);
        tick(H_HEUR);
        std::vector<int> want3(ns, 0), want5(ns, 0), want7(ns, 0), yo5(ns, 0), yo7(ns, 0);
        for (int si = 0; si < ns; ++si) {
            if (!live[si]) continue;
            NodeRun &r = R[si];
            if (r.status) continue;
            if (!r.prune) r.prune = r.bound < r.P->LB + 1.0;
            double gap = r.bound - r.P->LB;
            if (r.count == P.triag_iter + P.pent_iter + P.hept_iter)
                if (gap - 1.0 > (r.oldf - r.f) * (P.max_outer_iter - r.count)) r.giveup = 1;
            if (r.count == P.max_outer_iter)
                if (gap - 1.0 > (r.oldf - r.f) * P.extra_iter) r.giveup = 1;
            if (r.count == P.max_outer_iter + P.extra_iter) r.giveup = 1;
            if (rank != 0 && r.giveup && !r.prune) {
                pend[r.P].first += 60;
                pend[r.P].second += 50;
            }
            if (!r.prune && !r.giveup) want3[si] = 1;
        }
        // purge with the new duals, then separate
        for (int si = 0; si < ns; ++si) {
            if (!want3[si]) continue;
            NodeRun &r = R[si];
            sbuf.resize(r.m());
            if (!sbuf.empty())
                CUDA_TRY(c, d2h(c, sbuf.data(), c->hs[si].s, sbuf.size() * sizeof(double)));
            log_scorer_targets(c, r, sbuf);
            purge(r, sbuf);
        }
        if (std::any_of(want3.begin(), want3.end(), [](int v) { return v; }))
            if ((rc = separate_triangles(c, ns, runs, want3))) return rc;
        for (int si = 0; si < ns; ++si) {
            if (!want3[si]) continue;
            NodeRun &r = R[si];
            if (P.include_Pent && (r.count >= P.triag_iter || r.viol3 < 0.2)) want5[si] = 1;
        }
        // heptagonal test uses viol5 of this round: run the pentagonal SA first
        std::vector<int> none(ns, 0);
        if (std::any_of(want5.begin(), want5.end(), [](int v) { return v; }))
            if ((rc = separate_kgonal(c, ns, runs, want5, none, yo5, yo7))) return rc;
        for (int si = 0; si < ns; ++si) {
            if (!want3[si]) continue;
            NodeRun &r = R[si];
            if (P.include_Hepta && ((r.count >= P.triag_iter + P.pent_iter) || (r.viol3 < 0.2 && (1 - r.viol5 < 0.4))))
                want7[si] = 1;
        }
        if (std::any_of(want7.begin(), want7.end(), [](int v) { return v; }))
            if ((rc = separate_kgonal(c, ns, runs, none, want7, yo5, yo7))) return rc;
        tick(H_SEP);
        for (int si = 0; si < ns; ++si) {
            if (!live[si]) continue;
            NodeRun &r = R[si];
            if (want3[si]) r.sep_round++;
            r.done = r.prune || r.giveup || r.status || (r.nbit >= P.ADMM_itermax);
            if ((rc = fetch_lastrow(c, si, r.n, row))) return rc;
            store_fracsol(c, r, row);
        }
        tick(H_OTHER);
    }
    tick(H_OTHER);
    const bool want_records = (c->flags & MCB_FLAG_LOG) || ((c->flags & MCB_FLAG_LEARNED) && c->warm);
    c->last_records.assign(ns, nullptr);
    if (want_records)
        for (int si = 0; si < ns; ++si)
            if (!R[si].status && !R[si].prune)
                if ((rc = make_record(c, si, R[si], c->last_records[si]))) return rc;
    flush_prof(c);
    tick(H_REC);
    int ret = MCB_OK;
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int si = 0; si < ns; ++si) {
        NodeRun &r = R[si];
        r.bound = r.f + r.fixedvalue;
        if (rank == 0 && r.count > 0 && !r.status) r.P->diff = r.basic_bound - r.bound;  // bounding.c:241-243
        if (bounds) bounds[si] = r.bound;
        if (r.status && ret == MCB_OK) ret = r.status;
        if (stats) {
            mcb_node_stats &S = stats[si];
            S.bound = r.bound;
            S.basic_bound = r.basic_bound;
            S.n_sub = r.n;
            S.outer_iters = r.count;
            S.admm_iters = r.nbit_total;
            S.ipm_iters = r.ipm_iters;
            S.n_tri = (int)r.tri.size() / 4;
            S.n_pent = (int)r.pent.size() / 6;
            S.n_hept = (int)r.hept.size() / 8;
            S.pruned = r.prune;
            S.gaveup = r.giveup;
            S.seconds = secs;
        }
    }
    for (auto &kv : pend) {
        kv.first->pent_trials += kv.second.first;
        kv.first->hepta_trials += kv.second.second;
    }
    if (ret != MCB_OK && c->err.empty()) c->err = "a device iteration cap or factorisation failed";
    return ret;
}

// a new problem of the context (its SP->L on the host and the device); its id or -1
int add_problem(mcb_ctx *c, int N, const double *SL) {
    Problem P;
    P.N = N;
    P.pb = N - 1;
    P.SL.assign(SL, SL + (size_t)N * N);
    P.best_sol.assign(P.pb, 0);
    P.pent_trials = c->prm.Pent_Trials;
    P.hepta_trials = c->prm.Hepta_Trials;
    P.tri_ineq = c->prm.adjust_TriIneq ? 10 * N : c->prm.TriIneq;
    if (cudaMalloc(&P.d_SL, (size_t)N * N * sizeof(double)) != cudaSuccess) return -1;
    if (cudaMemcpy(P.d_SL, SL, (size_t)N * N * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(P.d_SL);
        return -1;
    }
    c->probs.push_back(std::move(P));
    return (int)c->probs.size() - 1;
}

}  // namespace

// =============================================================================
// C ABI
extern "C" {

int mcb_version(void) { return 10000; }

const char *mcb_strerror(int s) {
    switch (s) {
    case MCB_OK: return "ok";
    case MCB_ERR_ARG: return "invalid argument";
    case MCB_ERR_CUDA: return "CUDA error";
    case MCB_ERR_NOMEM: return "out of memory";
    case MCB_ERR_NUMERIC: return "numerical failure";
    case MCB_ERR_CAPACITY: return "capacity exceeded";
    case MCB_ERR_ITER: return "iteration cap reached";
    case MCB_ERR_NODEV: return "no CUDA device";
    default: return "unknown error";
    }
}

const char *mcb_last_error(const mcb_ctx *c) { return c ? c->err.c_str() : ""; }

mcb_ctx *mcb_create(const mcb_params *params, int N, const double *SL, int batch_max, int flags, void *stream,
                    int *status) {
    auto fail = [&](int code) -> mcb_ctx * {
        if (status) *status = code;
        return nullptr;
    };
    if (!params || !SL || N < 2 || N > MCB_NMAX || batch_max < 1 || batch_max > 4096) return fail(MCB_ERR_ARG);
    const int proj = flags & 0xff;
    if (proj != MCB_PROJ_FP64 && proj != MCB_PROJ_NS_BF16 && proj != MCB_PROJ_NS_TF32) return fail(MCB_ERR_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MCB_ERR_NODEV);
    mcb_ctx *c = new mcb_ctx();
    c->prm = *params;
    if (c->prm.adjust_TriIneq) c->prm.TriIneq = N * 10;  // process_input.c:122-123
    c->N = N;
    c->batch_max = batch_max;
    c->flags = flags;
    if (stream) c->st = (cudaStream_t)stream;
    else { cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking); c->own_stream = true; }
    int rc = add_problem(c, N, SL) == 0 ? MCB_OK : MCB_ERR_CUDA;
    auto chk = [&](cudaError_t e) { if (e != cudaSuccess && rc == MCB_OK) { rc = MCB_ERR_CUDA; c->err = cudaGetErrorString(e); } };
    c->hs.assign(batch_max, Slot());
    c->mem.assign(batch_max, SlotMem());
    for (int i = 0; i < batch_max && rc == MCB_OK; ++i) rc = alloc_slot(c, i);
    for (int i = 0; i < batch_max && rc == MCB_OK; ++i) rc = ensure_cut_capacity(c, i, 4096, 4096 * 16, 4096 * 8, 4096 * 24);
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_slots, batch_max * sizeof(Slot)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_partials, (size_t)batch_max * syrk_tiles(N) * 3 * sizeof(double)));
    c->list_stride = 3 + 3 * N;
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_lists, (size_t)batch_max * c->list_stride * sizeof(int)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_fixed, batch_max * sizeof(double)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_trisel, batch_max * trisel_bytes()));
    c->h_trisel.resize(batch_max * trisel_bytes());
    c->tcap_out = 2 * c->prm.TriIneq + 16;  // the learned ranking reads 2K candidates
    c->tcap_bnd = 1 << 16;
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_tout, (size_t)batch_max * c->tcap_out * sizeof(unsigned int)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_toutv, (size_t)batch_max * c->tcap_out * sizeof(double)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_tbnd, (size_t)batch_max * c->tcap_bnd * sizeof(unsigned int)));
    if (rc == MCB_OK) chk(cudaMalloc(&c->d_tbndv, (size_t)batch_max * c->tcap_bnd * sizeof(double)));
    c->proj = proj;
    if (rc == MCB_OK && cg_prepare()) {
        rc = MCB_ERR_CUDA;
        c->err = "CG kernel attributes";
    }
    if (rc == MCB_OK && proj != MCB_PROJ_FP64) {
        rc = c->ns.init(proj, N, batch_max, c->st);
        if (rc != MCB_OK) c->err = "Newton-Schulz buffers or cuBLAS handle";
        if (rc == MCB_OK) chk(cudaMalloc(&c->d_hlist, batch_max * sizeof(int)));
        if (rc == MCB_OK) chk(cudaMalloc(&c->d_hkeys, batch_max * sizeof(unsigned long long)));
        if (rc == MCB_OK) chk(cudaMalloc(&c->d_hsign, (size_t)batch_max * N * N));
        if (rc == MCB_OK) chk(cudaMalloc(&c->d_hval, (size_t)batch_max * N * sizeof(double)));
    }
    if (rc != MCB_OK) {
        if (status) *status = rc;
        mcb_destroy(c);
        return nullptr;
    }
    if (status) *status = MCB_OK;
    return c;
}

void mcb_destroy(mcb_ctx *c) {
    if (!c) return;
    if (c->st) cudaStreamSynchronize(c->st);
    for (auto &m : c->mem) free_slot(m);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->ns.destroy();
    for (auto &P : c->probs)
        if (P.d_SL) cudaFree(P.d_SL);
    void *ps[] = {c->d_slots, c->d_partials, c->d_lists, c->d_fixed, c->d_trisel, c->d_tout, c->d_toutv,
                  c->d_tbnd, c->d_tbndv, c->d_sajobs, c->d_perm, c->d_saout, c->d_saval,
                  c->d_hlist, c->d_hkeys, c->d_hsign, c->d_hval, c->d_fslot, c->d_fcp, c->d_fextra, c->d_F, c->d_pred};
    for (void *p : ps)
        if (p) cudaFree(p);
    for (auto &p : c->pending) { cudaEventDestroy(p.second.first); cudaEventDestroy(p.second.second); }
    for (auto e : c->ev_pool) cudaEventDestroy(e);
    if (c->own_stream && c->st) cudaStreamDestroy(c->st);
    delete c;
}

void mcb_set_lb(mcb_ctx *c, double lb, const int *sol) { mcb_set_problem_lb(c, 0, lb, sol); }
double mcb_get_lb(const mcb_ctx *c, int *sol) { return mcb_get_problem_lb(c, 0, sol); }
int mcb_set_problem_lb(mcb_ctx *c, int problem, double lb, const int *sol) {
    if (!c || problem < 0 || problem >= (int)c->probs.size()) return MCB_ERR_ARG;
    Problem &P = c->probs[problem];
    P.LB = lb;
    if (sol) P.best_sol.assign(sol, sol + P.pb);
    return MCB_OK;
}
double mcb_get_problem_lb(const mcb_ctx *c, int problem, int *sol) {
    if (!c || problem < 0 || problem >= (int)c->probs.size()) return 0.0;
    const Problem &P = c->probs[problem];
    if (sol) memcpy(sol, P.best_sol.data(), P.pb * sizeof(int));
    return P.LB;
}
void mcb_set_diff(mcb_ctx *c, double d) {
    if (c) c->probs[0].diff = d;
}
double mcb_get_diff(const mcb_ctx *c) { return c ? c->probs[0].diff : 0.0; }
int mcb_add_problem(mcb_ctx *c, int N, const double *SL) {
    if (!c || !SL || N < 2 || N > c->N) return MCB_ERR_ARG;
    const int id = add_problem(c, N, SL);
    return id < 0 ? MCB_ERR_CUDA : id;
}
int mcb_problem_count(const mcb_ctx *c) { return c ? (int)c->probs.size() : 0; }
int mcb_set_models(mcb_ctx *c, mcb_mlp *scorer, mcb_mlp *warm) {
    if (!c) return MCB_ERR_ARG;
    if ((scorer && mcb_mlp_num_params(scorer) <= 0) || (warm && mcb_mlp_num_params(warm) <= 0)) return MCB_ERR_ARG;
    if ((scorer && mlp_inputs(scorer) != kCutFeatures) || (warm && mlp_inputs(warm) != kCutFeatures))
        return MCB_ERR_ARG;
    c->scorer = scorer;
    c->warm = warm;
    return MCB_OK;
}
int mcb_log_count(const mcb_ctx *c, int which) {
    if (!c || which < 0 || which > 1) return 0;
    return (int)c->log_y[which].size();
}
int mcb_log_fetch(const mcb_ctx *c, int which, int cap, float *X, float *y) {
    if (!c || which < 0 || which > 1) return MCB_ERR_ARG;
    int k = std::min(cap, (int)c->log_y[which].size());
    if (X) memcpy(X, c->log_x[which].data(), (size_t)k * kCutFeatures * sizeof(float));
    if (y) memcpy(y, c->log_y[which].data(), (size_t)k * sizeof(float));
    return k;
}
void mcb_log_clear(mcb_ctx *c) {
    if (!c) return;
    for (int w = 0; w < 2; ++w) { c->log_x[w].clear(); c->log_y[w].clear(); }
}
int mcb_autotune_table(const mcb_ctx *c, int cap, int *npad, int *bucket, int *variant, float *us0, float *us1) {
    if (!c || c->proj == MCB_PROJ_FP64) return 0;
    int k = 0;
    for (const auto &e : c->ns.tuned) {
        if (k < cap) {
            if (npad) npad[k] = e.first.first;
            if (bucket) bucket[k] = e.first.second;
            if (variant) variant[k] = e.second.variant;
            if (us0) us0[k] = e.second.us[0];
            if (us1) us1[k] = e.second.us[1];
        }
        ++k;
    }
    return k;
}
int mcb_autotune_save(const mcb_ctx *c, const char *path) {
    if (!c || !path || c->proj == MCB_PROJ_FP64) return MCB_ERR_ARG;
    FILE *f = fopen(path, "w");
    if (!f) return MCB_ERR_ARG;
    fprintf(f, "{\"tc_gemm\": [");
    bool first = true;
    for (const auto &e : c->ns.tuned) {
        fprintf(f, "%s\n  {\"npad\": %d, \"bucket\": %d, \"variant\": %d, \"us\": [%.3f, %.3f]}", first ? "" : ",",
                e.first.first, e.first.second, e.second.variant, e.second.us[0], e.second.us[1]);
        first = false;
    }
    fprintf(f, "\n]}\n");
    fclose(f);
    return MCB_OK;
}
int mcb_autotune_load(mcb_ctx *c, const char *path) {
    if (!c || !path || c->proj == MCB_PROJ_FP64) return MCB_ERR_ARG;
    FILE *f = fopen(path, "r");
    if (!f) return MCB_ERR_ARG;
    std::string txt;
    char buf[4096];
    size_t r;
    while ((r = fread(buf, 1, sizeof(buf), f)) > 0) txt.append(buf, r);
    fclose(f);
    size_t pos = 0;
    int loaded = 0;
    while ((pos = txt.find("\"npad\"", pos)) != std::string::npos) {
        int np = 0, b = 0, v = 0;
        float u0 = 0, u1 = 0;
        if (sscanf(txt.c_str() + pos, "\"npad\": %d, \"bucket\": %d, \"variant\": %d, \"us\": [%f, %f]", &np, &b, &v,
                   &u0, &u1) == 5 &&
            np > 0 && np % 128 == 0 && b > 0 && v >= 0 && v < 2) {
            c->ns.tuned[{np, b}] = NsProj::Tuned{v, {u0, u1}};
            ++loaded;
        }
        pos += 6;
    }
    return loaded > 0 ? MCB_OK : MCB_ERR_ARG;
}
int mcb_ns_options(mcb_ctx *c, int operands, double l0) {
    if (!c || c->proj == MCB_PROJ_FP64) return MCB_ERR_ARG;
    return c->ns.configure(operands, l0);
}
int mcb_ns_schedule(const mcb_ctx *c, int cap, float *a, float *b, int *accurate) {
    if (!c || c->proj == MCB_PROJ_FP64) return 0;
    int k = 0;
    for (const NsStep &s : c->ns.steps) {
        if (k >= cap) break;
        if (a) a[k] = s.a;
        if (b) b[k] = s.b;
        if (accurate) accurate[k] = s.accurate;
        ++k;
    }
    return (int)c->ns.steps.size();
}
void mcb_set_trials(mcb_ctx *c, int p, int h) {
    if (!c) return;
    c->probs[0].pent_trials = p;
    c->probs[0].hepta_trials = h;
}
void mcb_get_trials(const mcb_ctx *c, int *p, int *h) {
    if (p) *p = c ? c->probs[0].pent_trials : 0;
    if (h) *h = c ? c->probs[0].hepta_trials : 0;
}

int mcb_bound_batch_multi(mcb_ctx *c, mcb_bab_node *const *nodes, const int *problems, int count, int rank,
                          double *bounds, mcb_node_stats *stats) {
    if (!c || !nodes || count < 1) return MCB_ERR_ARG;
    for (int i = 0; i < count; ++i)
        if (!nodes[i] || (problems && (problems[i] < 0 || problems[i] >= (int)c->probs.size()))) return MCB_ERR_ARG;
    c->err.clear();
    int rc = MCB_OK;
    if (!problems || count <= c->batch_max) {
        for (int off = 0; off < count && rc == MCB_OK; off += c->batch_max) {
            int k = std::min(c->batch_max, count - off);
            rc = bound_batch(c, nodes + off, problems ? problems + off : nullptr, k, rank,
                             bounds ? bounds + off : nullptr, stats ? stats + off : nullptr);
        }
        return rc;
    }
    // more nodes than slots: chunks of nodes with similar subproblem orders (the
    // tensor-core path pads a chunk to its largest order), in decreasing order
    std::vector<int> ord(count), nsub(count);
    for (int i = 0; i < count; ++i) {
        const Problem &P = c->probs[problems[i]];
        int fixed = 0;
        for (int v = 0; v < P.pb; ++v) fixed += nodes[i]->xfixed[v] != 0;
        nsub[i] = P.pb - fixed + 1;
        ord[i] = i;
    }
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return nsub[a] > nsub[b]; });
    std::vector<mcb_bab_node *> nd(count);
    std::vector<int> pr(count);
    for (int i = 0; i < count; ++i) {
        nd[i] = nodes[ord[i]];
        pr[i] = problems[ord[i]];
    }
    std::vector<double> bo(count);
    std::vector<mcb_node_stats> so(count);
    for (int off = 0; off < count && rc == MCB_OK; off += c->batch_max) {
        int k = std::min(c->batch_max, count - off);
        rc = bound_batch(c, nd.data() + off, pr.data() + off, k, rank, bo.data() + off, so.data() + off);
    }
    for (int i = 0; i < count; ++i) {
        if (bounds) bounds[ord[i]] = bo[i];
        if (stats) stats[ord[i]] = so[i];
    }
    return rc;
}

int mcb_bound_batch(mcb_ctx *c, mcb_bab_node *const *nodes, int count, int rank, double *bounds, mcb_node_stats *stats) {
    return mcb_bound_batch_multi(c, nodes, nullptr, count, rank, bounds, stats);
}

int mcb_evaluate(mcb_ctx *c, mcb_bab_node *node, int rank, double *bound, mcb_node_stats *st) {
    mcb_bab_node *arr[1] = {node};
    return mcb_bound_batch(c, arr, 1, rank, bound, st);
}

// ---- branch and bound -----------------------------------------------------
namespace {
struct Heap {
    std::vector<mcb_bab_node *> d;
    static int cmp(const mcb_bab_node *a, const mcb_bab_node *b) { return a->upper_bound > b->upper_bound ? 1 : -1; }
    void down(int cur) {
        int used = (int)d.size(), child = 2 * cur + 1;
        if (child + 1 < used && cmp(d[child + 1], d[child]) > 0) child++;
        while (child < used && cmp(d[cur], d[child]) < 0) {
            std::swap(d[cur], d[child]);
            cur = child;
            child = 2 * cur + 1;
            if (child + 1 < used && cmp(d[child + 1], d[child]) > 0) child++;
        }
    }
    void up(int cur) {
        int parent = (cur - 1) / 2;
        while (cur > 0 && cmp(d[parent], d[cur]) < 0) {
            std::swap(d[cur], d[parent]);
            cur = parent;
            parent = (cur - 1) / 2;
        }
    }
    mcb_bab_node *pop() {
        mcb_bab_node *n = d[0];
        d[0] = d.back();
        d.pop_back();
        if (!d.empty()) down(0);
        return n;
    }
    void push(mcb_bab_node *n) {
        d.push_back(n);
        up((int)d.size() - 1);
    }
};

mcb_bab_node *child_of(const mcb_bab_node *p, int pb, int ic, int xic) {
    mcb_bab_node *n = (mcb_bab_node *)malloc(sizeof(mcb_bab_node));
    for (int i = 0; i < pb; ++i) {
        n->xfixed[i] = p->xfixed[i];
        n->sol[i] = p->xfixed[i] ? p->sol[i] : 0;
    }
    n->xfixed[ic] = 1;
    n->sol[ic] = xic;
    n->level = p->level + 1;
    n->upper_bound = p->upper_bound;
    return n;
}

// training pairs of the warm-start model: the parent's cut features (with its dual)
// -> log(1 + the same cut's dual at the end of the child's cold-started bound)
void log_warm_pairs(mcb_ctx *c, const WarmIn &w, const std::shared_ptr<NodeRecord> &child) {
    if (!w.rec || !child || child->size() == 0) return;
    std::map<std::vector<int>, double> cd;
    for (size_t q = 0; q < child->size(); ++q) {
        std::vector<int> key{child->k[q], child->type[q]};
        key.insert(key.end(), child->verts.begin() + 7 * q, child->verts.begin() + 7 * q + child->k[q]);
        cd[key] = child->dual[q];
    }
    const NodeRecord &P = *w.rec;
    for (size_t q = 0; q < P.size(); ++q) {
        bool through = false;
        for (int a = 0; a < P.k[q]; ++a) through = through || P.verts[7 * q + a] == w.ic;
        if (through) continue;
        std::vector<int> key{P.k[q], P.type[q]};
        key.insert(key.end(), P.verts.begin() + 7 * q, P.verts.begin() + 7 * q + P.k[q]);
        auto it = cd.find(key);
        double t = it == cd.end() ? 0.0 : it->second;
        c->log_x[1].insert(c->log_x[1].end(), P.feats.begin() + q * kCutFeatures, P.feats.begin() + (q + 1) * kCutFeatures);
        c->log_y[1].push_back((float)log1p(std::max(t, 0.0)));
    }
}

int branching_var(const mcb_ctx *c, const mcb_bab_node *node) {
    int ic = -1;
    if (c->prm.branchingStrategy == 0) {
        double mx = -kBig;
        for (int i = 0; i < c->probs[0].pb; ++i)
            if (!node->xfixed[i] && fabs(0.5 - node->fracsol[i]) > mx) { ic = i; mx = fabs(0.5 - node->fracsol[ic]); }
    } else {
        double mn = kBig;
        for (int i = 0; i < c->probs[0].pb; ++i)
            if (!node->xfixed[i] && fabs(0.5 - node->fracsol[i]) < mn) { ic = i; mn = fabs(0.5 - node->fracsol[ic]); }
    }
    return ic;
}
}  // namespace

int mcb_bab(mcb_ctx *c, int batch, int max_nodes, double *opt, int *sol, double *root_bound, int *nodes_out,
            mcb_node_stats *log, int log_cap, int *log_count) {
    if (!c || batch < 1) return MCB_ERR_ARG;
    batch = std::min(batch, c->batch_max);
    const auto t_start = std::chrono::steady_clock::now();
    c->bab_open_bound = -1e308;
    c->bab_open_nodes = 0;
    int lc = 0, nodes = 1, evaluated = 0, rc = MCB_OK;
    Heap h;
    mcb_bab_node *root = (mcb_bab_node *)calloc(1, sizeof(mcb_bab_node));
    mcb_node_stats st;
    double rb = 0;
    rc = mcb_evaluate(c, root, 0, &rb, &st);
    evaluated++;
    if (log && lc < log_cap) log[lc++] = st;
    if (root_bound) *root_bound = rb;
    root->upper_bound = rb;
    if (rc == MCB_OK && c->probs[0].LB + 1.0 < rb && !c->prm.root) {
        int ic = branching_var(c, root);
        std::shared_ptr<NodeRecord> rec = c->last_records.empty() ? nullptr : c->last_records[0];
        for (int xic = 0; xic <= 1 && ic >= 0; ++xic) {
            mcb_bab_node *ch = child_of(root, c->probs[0].pb, ic, xic);
            if (rec && rec->size()) c->warm_in[ch] = WarmIn{rec, ic};
            h.push(ch);
            nodes++;
        }
    }
    free(root);
    std::vector<mcb_bab_node *> cur;
    std::vector<double> b;
    std::vector<mcb_node_stats> sts;
    while (rc == MCB_OK && !h.d.empty()) {
        if (max_nodes > 0 && evaluated >= max_nodes) { rc = MCB_ERR_CAPACITY; c->err = "node limit reached"; break; }
        if (c->bab_time_limit > 0.0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() >= c->bab_time_limit) {
            rc = MCB_ERR_CAPACITY;
            c->err = "time limit reached";
            break;
        }
        cur.clear();
        while (!h.d.empty() && (int)cur.size() < batch) cur.push_back(h.pop());
        b.assign(cur.size(), 0);
        sts.assign(cur.size(), mcb_node_stats());
        rc = mcb_bound_batch(c, cur.data(), (int)cur.size(), 1, b.data(), sts.data());
        evaluated += (int)cur.size();
        for (size_t a = 0; a < cur.size(); ++a) {
            if (log && lc < log_cap) log[lc++] = sts[a];
            cur[a]->upper_bound = b[a];
            std::shared_ptr<NodeRecord> rec = a < c->last_records.size() ? c->last_records[a] : nullptr;
            auto it = c->warm_in.find(cur[a]);
            if (it != c->warm_in.end()) {
                if (c->flags & MCB_FLAG_LOG) log_warm_pairs(c, it->second, rec);
                c->warm_in.erase(it);
            }
            if (rc == MCB_OK && c->probs[0].LB + 1.0 < b[a]) {
                int ic = branching_var(c, cur[a]);
                if (ic >= 0) {
                    for (int xic = 0; xic <= 1; ++xic) {
                        mcb_bab_node *ch = child_of(cur[a], c->probs[0].pb, ic, xic);
                        if (rec && rec->size()) c->warm_in[ch] = WarmIn{rec, ic};
                        h.push(ch);
                    }
                    nodes += 2;
                }
            }
            free(cur[a]);
        }
    }
    // the open nodes' bounds (their parents' bounds) bound every cut still unexplored
    for (auto *n : h.d) {
        if (c->probs[0].LB + 1.0 < n->upper_bound) {
            c->bab_open_bound = std::max(c->bab_open_bound, n->upper_bound);
            c->bab_open_nodes++;
        }
        free(n);
    }
    c->warm_in.clear();
    if (opt) *opt = c->probs[0].LB;
    if (sol) memcpy(sol, c->probs[0].best_sol.data(), c->probs[0].pb * sizeof(int));
    if (nodes_out) *nodes_out = nodes;
    if (log_count) *log_count = lc;
    return rc;
}

// ---- instrumentation ------------------------------------------------------
int mcb_kernel_stats(const mcb_ctx *c, int cap, char (*names)[32], long long *launches, double *ms) {
    int k = 0;
    for (int i = 0; i < K_NCLASS && k < cap; ++i, ++k) {
        if (names) snprintf(names[k], 32, "%s", kClassNames[i]);
        if (launches) launches[k] = c ? c->launches[i] : 0;
        if (ms) ms[k] = c ? c->ms[i] : 0.0;
    }
    return k;
}
void mcb_reset_kernel_stats(mcb_ctx *c) {
    if (!c) return;
    for (int i = 0; i < K_NCLASS; ++i) { c->launches[i] = 0; c->ms[i] = 0; c->work[i] = 0; }
    c->h2d = c->d2h = 0;
    c->lib_launches = 0;
    for (double &h : c->host_s) h = 0.0;
}
long long mcb_library_launch_count(const mcb_ctx *c) { return c ? c->lib_launches : 0; }
int mcb_host_stats(const mcb_ctx *c, int cap, char (*names)[32], double *seconds) {
    int k = 0;
    for (int i = 0; i < H_N && k < cap; ++i, ++k) {
        if (names) snprintf(names[k], 32, "%s", kHostNames[i]);
        if (seconds) seconds[k] = c ? c->host_s[i] : 0.0;
    }
    return k;
}
void mcb_graph_stats(const mcb_ctx *c, long long *captures, long long *replays) {
    if (captures) *captures = c ? c->graph_captures : 0;
    if (replays) *replays = c ? c->graph_launches : 0;
}
int mcb_set_cg_limit(mcb_ctx *c, int max_iters) {
    if (!c || max_iters < 1) return MCB_ERR_ARG;
    c->cg_max_iters = max_iters;
    return MCB_OK;
}
void mcb_set_time_limit(mcb_ctx *c, double seconds) {
    if (c) c->bab_time_limit = seconds > 0.0 ? seconds : 0.0;
}
double mcb_bab_open_bound(const mcb_ctx *c, int *open_nodes) {
    if (open_nodes) *open_nodes = c ? c->bab_open_nodes : 0;
    return c ? c->bab_open_bound : -1e308;
}
void mcb_set_profile(mcb_ctx *c, int on) {
    if (!c) return;
    if (on) c->flags |= MCB_FLAG_PROFILE;
    else {
        flush_prof(c);
        c->flags &= ~MCB_FLAG_PROFILE;
    }
}
void mcb_transfer_stats(const mcb_ctx *c, long long *h2d_bytes, long long *d2h_bytes) {
    if (h2d_bytes) *h2d_bytes = c ? c->h2d : 0;
    if (d2h_bytes) *d2h_bytes = c ? c->d2h : 0;
}
int mcb_kernel_work(const mcb_ctx *c, int cap, double *work, int *unit) {
    int k = 0;
    for (int i = 0; i < K_NCLASS && k < cap; ++i, ++k) {
        if (work) work[k] = c ? c->work[i] : 0.0;
        if (unit) unit[k] = kWorkUnit[i];
    }
    return k;
}
long long mcb_launch_count(const mcb_ctx *c) {
    if (!c) return 0;
    long long t = 0;
    for (int i = 0; i < K_NCLASS; ++i) t += c->launches[i];
    return t;
}

}  // extern "C"
