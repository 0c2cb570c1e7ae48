/*
 * mcbound.h -- C ABI of the GB300 (sm_103a) node-bound library for the MADAM
 * exact Max-Cut branch-and-bound.
 *
 * The library replaces MADAM's bound call:
 *     double Evaluate(BabNode *node, Problem *SP, Problem *PP, int rank)
 * (admm.h:246, evaluate.c:12-21) and everything below it: createSubproblem
 * (evaluate.c:39-116), SDPbound (bounding.c:25-250), the basic-SDP IPM
 * (ipm_mc_pk.c), ADMM with the safe bound (admm.c:49-771), the cut operators and
 * PSD projection (operators.c) and the triangle / pentagonal / heptagonal
 * separation (cutting_planes.c, qap_simulated_annealing.c).  The GW + 1-opt
 * heuristic that SDPbound calls (heuristic.c) runs on the host inside the
 * library on the GPU's eigen factor.
 *
 * Conventions: plain pointers and sizes, host memory in and out; device memory
 * is owned by the context; every entry point returns a status code (MCB_OK = 0
 * or a negative MCB_ERR_*), never exits and never traps the GPU.  One context
 * per host thread; a context is not re-entrant.  Matrices are column-major.
 */
#ifndef MCBOUND_H
#define MCBOUND_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCB_NMAX 1024     /* admm.h:131 NMAX */
#define MCB_MAX_TRI 50000 /* admm.h:34 */
#define MCB_MAX_PENT 50000
#define MCB_MAX_HEPT 50000

enum mcb_status {
    MCB_OK = 0,
    MCB_ERR_ARG = -1,      /* invalid argument or size beyond the stated limit   */
    MCB_ERR_CUDA = -2,     /* CUDA runtime error (message in mcb_last_error)     */
    MCB_ERR_NOMEM = -3,    /* device or host allocation failed                   */
    MCB_ERR_NUMERIC = -4,  /* factorisation failed / non-finite values           */
    MCB_ERR_CAPACITY = -5, /* a cut or candidate buffer would overflow           */
    MCB_ERR_ITER = -6,     /* a device iteration cap was reached (CG, bisection) */
    MCB_ERR_NODEV = -7     /* no CUDA device                                     */
};
/* A NULL context is an argument error everywhere: calls that return a status return
 * MCB_ERR_ARG, setters do nothing, getters return 0 (counters they write are 0). */

/* Projection forms (mcb_create flags, low byte) */
#define MCB_PROJ_FP64 0x0      /* plain: FP64 tridiagonal eigensolver (dsyevr's method) */
#define MCB_PROJ_NS_BF16 0x1   /* chosen: Newton-Schulz sign iteration on the tensor cores (tcgen05, operands
                                  as five BF16 digit planes: ~5e-10 per product), FP64 assembly and safe bound */
#define MCB_PROJ_NS_TF32 0x2   /* chosen: as MCB_PROJ_NS_BF16; with MCB_NS_OPERANDS_NATIVE its one-pass
                                  steps use TF32 operands (cuBLAS) instead of BF16 */
/* Other flags */
#define MCB_FLAG_PROFILE 0x100 /* time every kernel class with CUDA events */
/* operands of the Newton-Schulz growth steps (mcb_ns_options) */
#define MCB_NS_OPERANDS_NATIVE 0 /* one pass of the form's type (BF16 / TF32): rounding floor ~1e-3 */
#define MCB_NS_OPERANDS_SPLIT 1  /* five BF16 digit planes per operand, exact digit-sum groups, own tcgen05
                                    kernel (default) */
#define MCB_NS_OPERANDS_FP32 2   /* FP32 FMA through cuBLAS, no tensor cores (reference point) */
#define MCB_NS_OPERANDS_CUBLAS_SPLIT 3 /* cuBLAS's BF16x9 emulation of FP32 (reference point) */
#define MCB_FLAG_LEARNED 0x200 /* learned cut ranking + dual warm start (models set by mcb_set_models) */
#define MCB_FLAG_LOG 0x400     /* log the learned models' training pairs (mcb_log_fetch) */

/* Same fields, order and meaning as MADAM's Parameters (admm.h:57-89). */
typedef struct mcb_params {
    double sigma0;
    double scaleSigma;
    int ADMM_itermax;
    double tol0;
    double scaleTol;
    double minTol;
    int triag_iter;
    int pent_iter;
    int hept_iter;
    int max_outer_iter;
    int extra_iter;
    double violated_TriIneq;
    int TriIneq;
    int adjust_TriIneq;
    int PentIneq;
    int HeptaIneq;
    int Pent_Trials;
    int Hepta_Trials;
    int include_Pent;
    int include_Hepta;
    int root;
    int use_diff;
    int branchingStrategy;
} mcb_params;

/* Same layout as MADAM's BabNode (admm.h:147-155), so a BabNode* can be passed. */
typedef struct mcb_bab_node {
    int xfixed[MCB_NMAX];
    int sol[MCB_NMAX];
    double fracsol[MCB_NMAX];
    int level;
    double upper_bound;
} mcb_bab_node;

/* Per-node counters returned by the bound calls. */
typedef struct mcb_node_stats {
    double bound;       /* f + fixedvalue (what Evaluate returns)          */
    double basic_bound; /* IPM bound + fixedvalue                          */
    int n_sub;          /* subproblem size                                 */
    int outer_iters;    /* cutting-plane rounds                            */
    int admm_iters;     /* ADMM iterations, all rounds                     */
    int ipm_iters;      /* IPM iterations                                  */
    int n_tri, n_pent, n_hept; /* cuts in the final relaxation             */
    int pruned, gaveup;
    double seconds;     /* wall time of the batch call this node was in    */
} mcb_node_stats;

typedef struct mcb_ctx mcb_ctx;

/* ---- context ----------------------------------------------------------------
 * SL is MADAM's SP->L (N x N extended Laplacian, process_input.c:255-299), N <= 1024.
 * batch_max: most nodes bounded together by mcb_bound_batch.
 * stream: a cudaStream_t to launch on (NULL: the context creates its own). */
mcb_ctx *mcb_create(const mcb_params *params, int N, const double *SL, int batch_max, int flags,
                    void *stream, int *status);
void mcb_destroy(mcb_ctx *ctx);
const char *mcb_strerror(int status);
const char *mcb_last_error(const mcb_ctx *ctx);
int mcb_version(void);

/* Global state SDPbound reads and writes in MADAM: incumbent (Bab_LBGet/Bab_LBUpd,
 * heap.c:15,185), diff (bounding.c:241-243), Pent/Hepta_Trials (bounding.c:184-187). */
void mcb_set_lb(mcb_ctx *ctx, double lb, const int *sol);
double mcb_get_lb(const mcb_ctx *ctx, int *sol);
void mcb_set_diff(mcb_ctx *ctx, double diff);
double mcb_get_diff(const mcb_ctx *ctx);
void mcb_set_trials(mcb_ctx *ctx, int pent_trials, int hepta_trials);
void mcb_get_trials(const mcb_ctx *ctx, int *pent_trials, int *hepta_trials);
/* Newton-Schulz forms only (no counterpart in the reference, whose projection is
 * dsyevr): growth-step operands (MCB_NS_OPERANDS_*) and l0, the smallest
 * |eigenvalue| / ||W||_F the sign iteration resolves (default 1e-6; smaller
 * eigenvalues change X+ by at most l0 ||W||_F / 2 each).  MCB_ERR_ARG on the FP64 form. */
int mcb_ns_options(mcb_ctx *ctx, int operands, double l0);
/* the Newton-Schulz step schedule of the context: count, and per step a, b of
 * S <- a S + b S^3 and whether it is a closing step (l > 0.9, the plain cubic;
 * with MCB_NS_OPERANDS_NATIVE these run on accurate operands) */
int mcb_ns_schedule(const mcb_ctx *ctx, int cap, float *a, float *b, int *accurate);
/* the default schedule (safety 2%, closing within 1e-7 of 1) for a given l0; host
 * arithmetic only, callable without a device.  Returns the step count or MCB_ERR_ARG. */
int mcb_ns_schedule_for(double l0, int cap, float *a, float *b, int *accurate);

/* ---- the bound ---------------------------------------------------------------
 * mcb_evaluate: Evaluate(node, SP, PP, rank) (evaluate.c:12).  Writes
 * node->fracsol, updates the incumbent, returns the bound in *bound.
 * mcb_bound_batch: the same for `count` independent nodes in one batched pass;
 * the incumbent is shared (read at the start, updated as nodes find solutions). */
int mcb_evaluate(mcb_ctx *ctx, mcb_bab_node *node, int rank, double *bound, mcb_node_stats *stats);
int mcb_bound_batch(mcb_ctx *ctx, mcb_bab_node *const *nodes, int count, int rank, double *bounds,
                    mcb_node_stats *stats);

/* ---- several independent problems in one context ---------------------------
 * No counterpart in the reference, which holds one problem per process (SP,
 * process_input.c:182-312).  A context holds problem 0 (mcb_create's SL) and any
 * number added by mcb_add_problem, of order N <= the context's (the slots are
 * sized for it); each problem keeps its own incumbent, diff, Pent/Hepta_Trials
 * and triangle budget (10 N under adjust_TriIneq).  mcb_bound_batch_multi bounds
 * nodes of several problems in one batched pass: node i belongs to problem
 * problems[i] (its xfixed / sol over that problem's N - 1 variables), and is
 * bounded exactly as it would be alone in a context of that problem.  A call with
 * more nodes than the context's batch_max bounds them in chunks of batch_max
 * nodes of similar subproblem order.  The other calls of this header act on
 * problem 0. */
int mcb_add_problem(mcb_ctx *ctx, int N, const double *SL); /* returns the id (>= 1) or MCB_ERR_* */
int mcb_problem_count(const mcb_ctx *ctx);
int mcb_bound_batch_multi(mcb_ctx *ctx, mcb_bab_node *const *nodes, const int *problems, int count, int rank,
                          double *bounds, mcb_node_stats *stats);
int mcb_set_problem_lb(mcb_ctx *ctx, int problem, double lb, const int *sol);
double mcb_get_problem_lb(const mcb_ctx *ctx, int problem, int *sol);

/* Serial-equivalent branch-and-bound driver (the MPI master/worker loop of
 * main.c / bab_functions.c:226-334 as one process): root with rank 0 branched
 * at once, then nodes popped in bound order `batch` at a time.  Returns status;
 * *nodes counts as the reference does (1 + 2 per branching). */
int mcb_bab(mcb_ctx *ctx, int batch, int max_nodes, double *opt, int *sol, double *root_bound,
            int *nodes, mcb_node_stats *log, int log_cap, int *log_count);
/* Iteration cap of the conjugate-gradient solve of (B B^T + I) t = rhs in every ADMM
 * iteration (default 2000).  The reference factorises B B^T + I with CHOLMOD
 * (admm.c:480-487,546) and has no such cap; a solve that reaches it before its
 * tolerance ends that node's bound with MCB_ERR_ITER. */
int mcb_set_cg_limit(mcb_ctx *ctx, int max_iters);
/* Wall-time limit of mcb_bab in seconds (0: none), checked before each batch: the
 * reference's time limit (bab_functions.c:140-147, compiled out there; its report
 * prints "TIME LIMIT REACHED.", bab_functions.c:360-369).  A run that the node or
 * time limit stops returns MCB_ERR_CAPACITY with the incumbent in *opt / sol and
 * mcb_last_error "node limit reached" or "time limit reached". */
void mcb_set_time_limit(mcb_ctx *ctx, double seconds);
/* After an mcb_bab run the node or time limit stopped: the largest bound among the
 * open nodes not pruned by the incumbent (an upper bound on every cut left
 * unexplored) and their count in *open_nodes; -1e308 and 0 when the tree closed. */
double mcb_bab_open_bound(const mcb_ctx *ctx, int *open_nodes);

/* ---- operator-level entry points (host pointers; device memory per call) -----
 * Cut arrays: tri = 4 ints per cut (i, j, k, type) with i > j > k (Triangle_Inequality,
 * admm.h:93-100); pent = 6 ints (type, perm[5]); hept = 8 ints (type, perm[7]). */
/* y += B(X), operators.c:62-150 (X read through its lower triangle) */
int mcb_op_B(int n, const double *X, int ntri, const int *tri, int npent, const int *pent, int nhept,
             const int *hept, double *y);
/* X -= B^T(t), operators.c:171-513 */
int mcb_op_Bt(int n, double *X, int ntri, const int *tri, int npent, const int *pent, int nhept,
              const int *hept, const double *t);
/* PSD projection, operators.c:521-619: W (lower) -> Xp = W_+ (full symmetric),
 * Q = Xp - W (lower), Z = eigenvectors * sqrt(lambda) of the M eigenvalues > 1e-8
 * (ascending), evals.  proj = MCB_PROJ_* form; the Newton-Schulz forms may add
 * MCB_PROJ_OPERANDS(MCB_NS_OPERANDS_*) and write neither Z nor evals (M is the
 * rounded (n + trace sign(W)) / 2). */
#define MCB_PROJ_OPERANDS(op) (((op) + 1) << 4)
int mcb_project_psd(int n, const double *W, int proj, double *Xp, double *Q, double *Z, double *evals,
                    int *M);
/* The same projection for callers that cannot allocate device memory (their
 * memory is handed out by their own pool or capped by their scheduler).  No
 * counterpart in the reference, which projects host arrays.  W, Xp, Q, Z and
 * evals are the caller's DEVICE buffers (n*n, n*n, n*n, n*n, n doubles); the
 * call allocates nothing: its only scratch is a static device array of the
 * library sized for n <= MCB_NOALLOC_MAX_N (about 5.3 MB on every GPU that
 * loads the library, for as long as it stays loaded).  Larger n returns
 * MCB_ERR_ARG.  Runs on `stream` and returns after it completes, with M on the
 * host.  The first call on a device looks up the scratch's device address
 * (cudaGetSymbolAddress).  Calls share the scratch: calls that overlap on the
 * GPU race. */
#define MCB_NOALLOC_MAX_N 512
int mcb_project_psd_noalloc(int n, const double *W, double *Xp, double *Q, double *Z, double *evals, int *M,
                            void *stream);
/* The tensor-core GEMM of the Newton-Schulz form (no counterpart in the
 * reference): C = alpha A B^T + diag I for `batch` row-major npad x npad FP32
 * matrices (host buffers).  Each operand is scaled by a power of two and cut into
 * five signed 7-bit digits, one BF16 plane each; tcgen05.mma sums the nineteen
 * plane products of digit sum <= 5 in four FP32 accumulators, the three leading
 * digit-sum groups exactly, so C is accurate to ~5e-10 of its norm before its
 * rounding to FP32.  npad a multiple of 128, <= 1024.  sym = 1 computes the lower
 * 128 x 128 tiles only and mirrors them (for products known to be symmetric).
 * variant: 0 = two pipeline stages, 1 = one (the autotuner picks per matrix order). */
int mcb_split_gemm(int npad, int batch, const float *A, const float *B, float alpha, float diag, int sym,
                   int variant, float *C);
/* The autotuner's table of a context (Newton-Schulz forms): for every (npad,
 * live-slot bucket) met so far the chosen tcgen05 variant and the microseconds
 * per launch each variant took.  Returns the number of entries. */
int mcb_autotune_table(const mcb_ctx *ctx, int cap, int *npad, int *bucket, int *variant, float *us0, float *us1);
/* Save / load the table as JSON ({"tc_gemm": [{"npad":..,"bucket":..,"variant":..,"us":[..,..]}]});
 * loaded entries are used instead of timing. */
int mcb_autotune_save(const mcb_ctx *ctx, const char *path);
int mcb_autotune_load(mcb_ctx *ctx, const char *path);
/* Test of the tensor-core kernel's bounded waits (no counterpart in the reference).
 * While on (process-wide), the tcgen05 GEMM issues no TMA loads, so nothing is in
 * flight and its first wait on a full pipeline stage runs out after ~a millisecond:
 * every call that launches it reports MCB_ERR_ITER, and calls after it is switched
 * off run normally.  Lets a test drive the expiry path on a GPU without faulting it. */
void mcb_tc_test_expiry(int on);
/* largest eigenvalue (admm.c:731-752) and a rigorous upper bound on it */
int mcb_lambda_max(int n, const double *A, double *lmax, double *lmax_upper);
/* basic SDP relaxation by the predictor-corrector IPM, ipm_mc_pk.c */
int mcb_ipm(int n, const double *L, double *X, double *y, double *Z, double *phi, int *iters);
/* triangle separation, cutting_planes.c:48-127: the K most violated (> thr) in scan order */
int mcb_separate_triangles(int n, const double *X, int K, double thr, int *out, double *vals, int *count,
                           double *max_violation);
/* k-gonal SA (qap_simulated_annealing.c) on X (full symmetric): trials * ntypes
 * independent runs (ntypes = 3 for k = 5, 4 for k = 7), run r with type r % ntypes + 1
 * and counter stream key2(key, (r / ntypes) * 8 + type) -- the runs of one
 * getViolated_Pentagonal/HeptagonalInequalities call (cutting_planes.c:247-250,
 * 444-447).  ineq: k ints per run; values: the SA cost per run. */
int mcb_qap_sa_batch(int n, const double *X, int k, int trials, uint64_t key, int *ineq, double *values);

/* ---- learned cut ranking and dual warm start ----------------------------------
 * No counterpart in the reference.  A small MLP (d inputs, two tanh layers of
 * h1 and h2 units, one linear output; FP32), trained on the GPU by the library's
 * own forward / backward / Adam kernels (mean squared error).  Host buffers in
 * and out; X is row-major n x d.  Parameter vector layout:
 * [W1 (h1 x d, row-major) | b1 | W2 (h2 x h1) | b2 | w3 (h2) | b3]. */
typedef struct mcb_mlp mcb_mlp;
mcb_mlp *mcb_mlp_create(int d_in, int h1, int h2, uint64_t seed, int *status);
void mcb_mlp_destroy(mcb_mlp *mlp);
int mcb_mlp_num_params(const mcb_mlp *mlp);
int mcb_mlp_get_params(const mcb_mlp *mlp, float *params);
int mcb_mlp_set_params(mcb_mlp *mlp, const float *params);  /* also resets Adam's moments */
int mcb_mlp_predict(mcb_mlp *mlp, const float *X, int n, float *out);
/* gradient of mean((f(X) - Y)^2) with respect to the parameters, and the loss */
int mcb_mlp_gradient(mcb_mlp *mlp, const float *X, const float *Y, int n, float *grad, float *loss);
/* `epochs` passes of Adam (beta 0.9 / 0.999) over shuffled minibatches; final_loss
 * = the loss over all n samples after training */
int mcb_mlp_train(mcb_mlp *mlp, const float *X, const float *Y, int n, int epochs, int batch, float lr,
                  uint64_t seed, float *final_loss);

/* Attach the models to a context (not owned; either may be null).  With
 * MCB_FLAG_LEARNED the scorer ranks the 2K most violated triangles of each
 * separation (cutting_planes.c:48-127 keeps the K most violated) and keeps the K
 * best scores; mcb_bab hands each child its parent's final cuts (those through
 * the branching variable dropped) with duals predicted by the warm model as the
 * starting cut set.  Without a model that part is the plain method.  Both models
 * take the 10 features documented in k_learn.cu and predict log(1 + dual). */
int mcb_set_models(mcb_ctx *ctx, mcb_mlp *cut_scorer, mcb_mlp *warm_start);
/* Training pairs logged under MCB_FLAG_LOG: which = 0 cut scorer (features at
 * separation -> log(1 + dual after the next ADMM call)), 1 warm start (parent's
 * final cut features with its dual -> log(1 + the child's final dual of the
 * same cut, 0 if absent)); rows of 10 floats. */
int mcb_log_count(const mcb_ctx *ctx, int which);
int mcb_log_fetch(const mcb_ctx *ctx, int which, int cap, float *X, float *y);
void mcb_log_clear(mcb_ctx *ctx);

/* ---- instrumentation ---------------------------------------------------------
 * Per kernel class: launches and total device time (ms, CUDA events on the
 * context's stream; needs MCB_FLAG_PROFILE).  Returns the number of classes. */
int mcb_kernel_stats(const mcb_ctx *ctx, int cap, char (*names)[32], long long *launches, double *ms);
void mcb_reset_kernel_stats(mcb_ctx *ctx);
/* algorithmic work per kernel class, same order as mcb_kernel_stats: unit[i] = 1 for
 * FP64 flops, 2 for bytes, 0 when the class has no counted work.  Counted from the
 * iterations each node actually executed. */
int mcb_kernel_work(const mcb_ctx *ctx, int cap, double *work, int *unit);
/* host<->device bytes moved by the bound calls since the last reset */
void mcb_transfer_stats(const mcb_ctx *ctx, long long *h2d_bytes, long long *d2h_bytes);
/* FP64 FMA throughput of the current device in GFLOP/s (microbenchmark) */
double mcb_measure_fp64_peak(void);
/* launches of the library's own kernels, and of cuBLAS GEMMs (Newton-Schulz forms) */
long long mcb_launch_count(const mcb_ctx *ctx);
long long mcb_library_launch_count(const mcb_ctx *ctx);
/* wall time of the bound calls per phase (ipm, cut_upload, admm, safe_bound,
 * heuristic, separation, records, other), GPU waits included; returns the count */
int mcb_host_stats(const mcb_ctx *ctx, int cap, char (*names)[32], double *seconds);
/* ADMM chunks run as CUDA graphs when profiling is off: graphs captured, and replays */
void mcb_graph_stats(const mcb_ctx *ctx, long long *captures, long long *replays);
/* switch per-class CUDA-event timing (MCB_FLAG_PROFILE) on or off between calls */
void mcb_set_profile(mcb_ctx *ctx, int on);

#ifdef __cplusplus
}
#endif
#endif
