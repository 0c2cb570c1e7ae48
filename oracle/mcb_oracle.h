/*
 * mcb_oracle.h -- CPU oracle for the MADAM node-bound path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (MADAM: evaluate.c, bounding.c, ipm_mc_pk.c, admm.c, operators.c,
 * cutting_planes.c, qap_simulated_annealing.c, heuristic.c, heap.c,
 * bab_functions.c).  It is used by the tests, by the smoke check and by the
 * CPU-baseline leg of the benchmark, always as the checker.  The product
 * (madam_gb300/libmcbound.so) never links, loads or calls it.
 *
 * Dense LAPACK/BLAS calls (dsyevr, dpotrf, dpotri, dposv, dsymm, dsymv, dsyrk,
 * dlansy) go to the same third-party library the reference links (an OpenBLAS
 * build; here the copy that SciPy ships), resolved at run time with dlopen.
 * The reference's sparse CHOLMOD factorisation of (B B^T + I) (admm.c:480-487,
 * 546) is restated as a conjugate-gradient solve on the explicitly assembled
 * sparse matrix, converged to a relative residual of 1e-14.
 *
 * Two random-number modes:
 *   ORC_RNG_GLIBC    one global glibc TYPE_3 rand() stream seeded with 2020
 *                    (bab_functions.c:82), consumed in the reference's order by
 *                    the GW heuristic (heuristic.c:48) and the k-gonal SA
 *                    (qap_simulated_annealing.c:75,116-117,155).  Used to pin
 *                    the oracle against the reference's own outputs.
 *   ORC_RNG_COUNTER  counter-based streams keyed by (node, call, trial): the
 *                    form the GPU build uses so that nodes can be bounded in
 *                    any order and in parallel.  GPU parity tests use this.
 */
#ifndef MCB_ORACLE_H
#define MCB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NMAX 1024
#define ORC_MAX_TRI 50000   /* admm.h:34 */
#define ORC_MAX_PENT 50000  /* admm.h:35 */
#define ORC_MAX_HEPT 50000  /* admm.h:36 */
#define ORC_SA_ZERO 1e-11   /* |delta| below this is zero in counter mode */
#define ORC_SA_MAX_SWEEPS 80 /* sweep cap of the SA in counter mode */

enum { ORC_RNG_GLIBC = 0, ORC_RNG_COUNTER = 1 };
enum { ORC_TOPK_REFERENCE = 0, ORC_TOPK_CANONICAL = 1 };

/* Same fields, order and defaults as the reference's Parameters (admm.h:57-89). */
typedef struct orc_params {
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
} orc_params;

/* Same layout as the reference's BabNode (admm.h:147-155). */
typedef struct orc_node {
    int xfixed[ORC_NMAX];
    int sol[ORC_NMAX];
    double fracsol[ORC_NMAX];
    int level;
    double upper_bound;
} orc_node;

/* Per-node statistics the oracle records (also the learned model's training log). */
typedef struct orc_node_stats {
    double bound;          /* returned bound (f + fixedvalue)            */
    double basic_bound;    /* IPM bound + fixedvalue                     */
    int n_sub;             /* subproblem size                            */
    int outer_iters;       /* cutting-plane rounds (count)               */
    int admm_iters;        /* total ADMM iterations                      */
    int ipm_iters;         /* IPM iterations                             */
    int n_tri, n_pent, n_hept; /* cuts in the final relaxation           */
    int pruned, gaveup;
    double seconds;
} orc_node_stats;

typedef struct orc_ctx orc_ctx;

/* LAPACK loader: path to a shared library exporting LP64 BLAS/LAPACK symbols
 * (plain "dsyevr_" or SciPy's "scipy_dsyevr_" naming).  Returns 0 on success. */
int orc_lapack_init(const char *path);

/* glibc TYPE_3 random(): restated from its published description.  */
typedef struct orc_glibc { uint32_t r[34]; int pos; } orc_glibc;
void orc_glibc_seed(orc_glibc *g, unsigned int seed);
int orc_glibc_next(orc_glibc *g);

/* counter-based generator (splitmix64 finaliser over key + counter) */
uint64_t orc_mix64(uint64_t z);
uint64_t orc_key2(uint64_t a, uint64_t b);
uint64_t orc_node_key(const int *xfixed, const int *sol, int pb);

/* ---- problem construction ---- */
void orc_default_params(orc_params *p);
/* extended Laplacian of process_input.c:255-299; L is nv*nv column-major */
void orc_build_L(int nv, int ne, const int *ei, const int *ej, const double *w, double *L);
int orc_create_subproblem(int N, const double *SL, const int *xfixed, const int *sol, double *PL);
double orc_fixed_value(int N, const double *SL, const int *xfixed, const int *sol);
double orc_evaluate_solution(int N, const double *SL, const int *sol);

/* ---- kernels of the bound (operator-level entry points for KATs) ---- */
/* cut arrays: tri = 4 ints (i,j,k,type); pent = 6 ints (type,p0..p4); hept = 8 ints (type,p0..p6) */
void orc_op_B(int n, const double *X, int ntri, const int *tri, int npent, const int *pent,
              int nhept, const int *hept, double *y);
void orc_op_Bt(int n, double *X, int ntri, const int *tri, int npent, const int *pent,
               int nhept, const int *hept, const double *t);
/* PSD projection (operators.c:521-619): W (n*n, lower) -> Xp (lower), Q, Z (n*M), evals.
 * Returns M or -1 on LAPACK failure.  canon_sign flips each eigenvector so that its
 * largest-magnitude entry is positive. */
int orc_project(int n, const double *W, double *Xp, double *Q, double *Z, double *evals, int canon_sign);
/* dsyevr ABSTOL used by orc_project / orc_lambda_max (default 1e-8 as the reference) */
void orc_set_abstol(double abstol);
/* Newton-Schulz projection model: with k > 0 steps (p_i(x) = a_i x + b_i x^3), orc_project
 * returns the sign-iteration projection in exact arithmetic instead of the reference's:
 * X_+ = sum_j lambda_j (1 + p_k(...p_1(lambda_j / ||W||_F))) / 2 v_j v_j^T over all eigenpairs
 * (Z and M stay the reference's).  k = 0 restores the reference projection. */
void orc_set_ns_schedule(int k, const double *a, const double *b);
/* relative residual at which the ADMM's linear solve stops (default 1e-15; <= 0 restores it) */
void orc_set_cg_tol(double tol);
/* on != 0: the ADMM's (B B^T + I) solve by a dense Cholesky factor instead of conjugate gradients */
void orc_set_direct_solve(int on);
/* append every matrix W the ADMM projects to the file at path (int n, n x n doubles); NULL closes */
void orc_set_projection_dump(const char *path);
/* largest eigenvalue as admm.c:731-752 computes it */
double orc_lambda_max(int n, const double *A);
/* basic SDP bound by the predictor-corrector IPM (ipm_mc_pk.c); returns iterations or -1 */
int orc_ipm(const double *L, int n, double *X, double *y, double *Z, double *phi);
/* triangle separation (cutting_planes.c:48-127); out = 4 ints per cut, vals per cut */
double orc_sep_triangles(const double *X, int n, int K, double thr, int mode,
                         int *out, double *vals, int *count);
/* k-gonal simulated annealing (qap_simulated_annealing.c); H is k*k, X full n*n symmetric */
double orc_qap_sa(const int *H, int k, const double *X, int n, int rng_mode,
                  orc_glibc *g, uint64_t key, int *ineq);

/* ---- whole-node / whole-tree drivers ---- */
orc_ctx *orc_create(const orc_params *p, int N, const double *SL, int rng_mode, int topk_mode,
                    int canon_sign);
void orc_destroy(orc_ctx *c);
void orc_set_lb(orc_ctx *c, double lb, const int *sol);
double orc_get_lb(orc_ctx *c, int *sol);
void orc_set_diff(orc_ctx *c, double diff);
double orc_get_diff(orc_ctx *c);
void orc_set_trials(orc_ctx *c, int pent_trials, int hepta_trials);
void orc_get_trials(orc_ctx *c, int *pent_trials, int *hepta_trials);
void orc_set_admm_trace(orc_ctx *c, double *buf, int cap);
/* Evaluate (evaluate.c:12) = createSubproblem + SDPbound */
double orc_evaluate(orc_ctx *c, orc_node *node, int rank, orc_node_stats *st);
/* serial branch-and-bound: root via Init_PQ (rank 0), then worker steps (rank 1).
 * Returns number of nodes (reference counting: 1 + 2 per branching) or -1. */
int orc_bab(orc_ctx *c, double *opt, int *sol, double *root_bound, int max_nodes,
            orc_node_stats *log, int log_cap, int *log_count);

#ifdef __cplusplus
}
#endif
#endif
