/* Internal declarations shared by the oracle's translation units.
 * TEST INFRASTRUCTURE ONLY (see mcb_oracle.h). */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

#include <stddef.h>
#include "mcb_oracle.h"

#define ORC_BIG 1e+9 /* BIG_NUMBER, admm.h:31 */

/* LAPACK / BLAS entry points, resolved by orc_lapack_init (Fortran ABI, LP64). */
typedef void (*orc_dsyevr_t)(const char *, const char *, const char *, const int *, double *,
                             const int *, const double *, const double *, const int *,
                             const int *, const double *, int *, double *, double *,
                             const int *, int *, double *, const int *, int *, const int *,
                             int *, size_t, size_t, size_t);
typedef void (*orc_dpotrf_t)(const char *, const int *, double *, const int *, int *, size_t);
typedef void (*orc_dpotri_t)(const char *, const int *, double *, const int *, int *, size_t);
typedef void (*orc_dposv_t)(const char *, const int *, const int *, double *, const int *,
                            double *, const int *, int *, size_t);
typedef void (*orc_dsymm_t)(const char *, const char *, const int *, const int *,
                            const double *, const double *, const int *, const double *,
                            const int *, const double *, double *, const int *, size_t,
                            size_t);
typedef void (*orc_dsymv_t)(const char *, const int *, const double *, const double *,
                            const int *, const double *, const int *, const double *,
                            double *, const int *, size_t);
typedef void (*orc_dsyrk_t)(const char *, const char *, const int *, const int *,
                            const double *, const double *, const int *, const double *,
                            double *, const int *, size_t, size_t);
typedef double (*orc_dlansy_t)(const char *, const char *, const int *, const double *,
                               const int *, double *, size_t, size_t);

typedef void (*orc_dcopy_t)(const int *, const double *, const int *, double *, const int *);
typedef void (*orc_dscal_t)(const int *, const double *, double *, const int *);
typedef void (*orc_daxpy_t)(const int *, const double *, const double *, const int *, double *, const int *);
typedef double (*orc_ddot_t)(const int *, const double *, const int *, const double *, const int *);
typedef double (*orc_dnrm2_t)(const int *, const double *, const int *);

typedef struct orc_lapack {
    orc_dcopy_t dcopy;
    orc_dscal_t dscal;
    orc_daxpy_t daxpy;
    orc_ddot_t ddot;
    orc_dnrm2_t dnrm2;
    orc_dsyevr_t dsyevr;
    orc_dpotrf_t dpotrf;
    orc_dpotri_t dpotri;
    orc_dposv_t dposv;
    orc_dsymm_t dsymm;
    orc_dsymv_t dsymv;
    orc_dsyrk_t dsyrk;
    orc_dlansy_t dlansy;
    int ready;
} orc_lapack;
extern orc_lapack orc_la;

/* One cut expanded into its clique form: <B_c, X> = -scale * sum_{a<b} e_a e_b X[p_a,p_b]. */
typedef struct orc_clique {
    int k;
    int p[7];
    int e[7];
    double scale;
} orc_clique;

void orc_tri_clique(const int *tri, orc_clique *c);   /* tri = (i,j,k,type) */
void orc_pent_clique(const int *pent, orc_clique *c); /* pent = (type,p0..p4) */
void orc_hept_clique(const int *hept, orc_clique *c); /* hept = (type,p0..p6) */

/* Node-independent state of the bound (the reference keeps these as globals,
 * global_var.h:6-51; here they live in the context). */
struct orc_ctx {
    orc_params prm;     /* current parameters (Pent/Hepta_Trials mutate, bounding.c:184-187) */
    int N;              /* SP->n */
    int pb;             /* BabPbSize = N - 1 */
    double *SL;         /* SP->L, N*N */
    int rng_mode, topk_mode, canon_sign;
    orc_glibc g;        /* the global rand() stream in glibc mode */
    uint64_t node_key;  /* key of the node being bounded (counter mode) */
    int heur_calls;     /* heuristic calls within the node (counter mode) */
    int sep_round;      /* separation round within the node (counter mode) */
    double LB;          /* BabLB, heap.c:9 */
    int *best_sol;      /* BabSol */
    double diff;        /* global diff, bounding.c:241-243 */
    /* subproblem and iterates */
    int n;
    double *L, *X, *Q, *y;
    double f;
    /* cuts (AoS restated as flat int arrays) */
    int ntri, npent, nhept;
    int *tri, *pent, *hept;       /* capacity ORC_MAX_* */
    double *tri_y, *pent_y, *hept_y;
    double *t, *s, *u;            /* capacity of all families */
    /* eigen factor for the heuristic (Z = V diag(sqrt(w)) * sqrt(sigma)), M columns */
    double *Z;
    int M;
    /* scratch */
    double *W1, *W2, *W3;
    int *list_i;
    double *list_v;
    double *trace;
    int trace_cap, trace_len;
};

void orc_set_work_n(int N);
/* admm.c:49-771 */
int orc_admm(orc_ctx *c, double *sigma, double tol, int *nbit);
/* cutting_planes.c:132-214, 316-409, 512-605 */
double orc_update_tri(orc_ctx *c, const double *s, int *added, int *subtracted);
double orc_update_pent(orc_ctx *c, const double *s, int *added, int *subtracted, int triag);
double orc_update_hept(orc_ctx *c, const double *s, int *added, int *subtracted, int off);
/* heuristic.c:10-224 */
double orc_run_heuristic(orc_ctx *c, const orc_node *node, int *x);
/* bab_functions.c:114-134 */
int orc_update_solution(orc_ctx *c, const int *x);

/* random draw helpers */
int orc_rand_glibc(orc_ctx *c);
typedef struct orc_stream { uint64_t key; uint64_t ctr; } orc_stream;
uint64_t orc_stream_next(orc_stream *s);

#endif
