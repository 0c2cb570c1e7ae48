/* The subset of the CHOLMOD interface that the reference's admm.c uses
 * (admm.c:98-114, 117, 480-487, 546, 709-714), declared for a small stand-in
 * implementation (cholmod_shim.c) that solves (B B^T + beta I) x = b by
 * conjugate gradients on the explicitly assembled sparse matrix.  Used only to
 * build the reference itself as a CPU oracle (oracle/_ref). */
#ifndef MCB_REF_CHOLMOD_SHIM_H
#define MCB_REF_CHOLMOD_SHIM_H
#include <stddef.h>

#define CHOLMOD_REAL 1
#define CHOLMOD_A 0

typedef struct cholmod_common_struct { int status; } cholmod_common;

typedef struct cholmod_triplet_struct {
    size_t nrow, ncol, nzmax, nnz;
    void *i, *j, *x;
    int stype, itype, xtype, dtype;
} cholmod_triplet;

typedef struct cholmod_sparse_struct {
    size_t nrow, ncol, nzmax;
    int *ri, *ci;
    double *v;
    int xtype;
} cholmod_sparse;

typedef struct cholmod_dense_struct {
    size_t nrow, ncol, nzmax, d;
    void *x;
    int xtype;
} cholmod_dense;

typedef struct cholmod_factor_struct {
    int m;
    int *rp, *ci;
    double *v;
} cholmod_factor;

int cholmod_start(cholmod_common *c);
int cholmod_finish(cholmod_common *c);
cholmod_triplet *cholmod_allocate_triplet(size_t nrow, size_t ncol, size_t nzmax, int stype, int xtype,
                                          cholmod_common *c);
cholmod_sparse *cholmod_triplet_to_sparse(cholmod_triplet *t, size_t nzmax, cholmod_common *c);
cholmod_dense *cholmod_zeros(size_t nrow, size_t ncol, int xtype, cholmod_common *c);
cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *c);
int cholmod_factorize_p(cholmod_sparse *A, double beta[2], int *fset, size_t fsize, cholmod_factor *L,
                        cholmod_common *c);
cholmod_dense *cholmod_solve(int sys, cholmod_factor *L, cholmod_dense *B, cholmod_common *c);
int cholmod_free_dense(cholmod_dense **X, cholmod_common *c);
int cholmod_free_factor(cholmod_factor **L, cholmod_common *c);
int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *c);
int cholmod_free_triplet(cholmod_triplet **T, cholmod_common *c);
#endif
