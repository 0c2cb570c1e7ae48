/* Stand-in for the CHOLMOD calls of the reference's admm.c: the factor object
 * holds G = B B^T + beta I in CSR form and cholmod_solve runs conjugate
 * gradients on it to a relative residual of 1e-15 (shared code: ../orc_gram.c).  Used only to build the
 * reference itself as a CPU oracle (oracle/_ref). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cholmod.h"
#include "../orc_gram.h"

int cholmod_start(cholmod_common *c) { c->status = 0; return 1; }
int cholmod_finish(cholmod_common *c) { (void)c; return 1; }

cholmod_triplet *cholmod_allocate_triplet(size_t nrow, size_t ncol, size_t nzmax, int stype, int xtype,
                                          cholmod_common *c) {
    (void)c;
    cholmod_triplet *t = calloc(1, sizeof(*t));
    t->nrow = nrow; t->ncol = ncol; t->nzmax = nzmax; t->stype = stype; t->xtype = xtype;
    t->i = calloc(nzmax + 1, sizeof(int));
    t->j = calloc(nzmax + 1, sizeof(int));
    t->x = calloc(nzmax + 1, sizeof(double));
    return t;
}

cholmod_sparse *cholmod_triplet_to_sparse(cholmod_triplet *t, size_t nzmax, cholmod_common *c) {
    (void)nzmax; (void)c;
    cholmod_sparse *A = calloc(1, sizeof(*A));
    A->nrow = t->nrow; A->ncol = t->ncol; A->nzmax = t->nnz; A->xtype = t->xtype;
    A->ri = malloc((t->nnz + 1) * sizeof(int));
    A->ci = malloc((t->nnz + 1) * sizeof(int));
    A->v = malloc((t->nnz + 1) * sizeof(double));
    memcpy(A->ri, t->i, t->nnz * sizeof(int));
    memcpy(A->ci, t->j, t->nnz * sizeof(int));
    memcpy(A->v, t->x, t->nnz * sizeof(double));
    return A;
}

cholmod_dense *cholmod_zeros(size_t nrow, size_t ncol, int xtype, cholmod_common *c) {
    (void)c;
    cholmod_dense *d = calloc(1, sizeof(*d));
    d->nrow = nrow; d->ncol = ncol; d->nzmax = nrow * ncol; d->d = nrow; d->xtype = xtype;
    d->x = calloc(nrow * ncol + 1, sizeof(double));
    return d;
}

cholmod_factor *cholmod_analyze(cholmod_sparse *A, cholmod_common *c) {
    (void)c;
    cholmod_factor *L = calloc(1, sizeof(*L));
    L->m = (int)A->nrow;
    return L;
}

int cholmod_factorize_p(cholmod_sparse *A, double beta[2], int *fset, size_t fsize, cholmod_factor *L,
                        cholmod_common *c) {
    (void)fset; (void)fsize; (void)c;
    orc_gram G;
    orc_gram_build((int)A->nrow, A->nzmax, A->ri, A->ci, A->v, beta[0], &G);
    L->m = G.m; L->rp = G.rp; L->ci = G.ci; L->v = G.v;
    return 1;
}

cholmod_dense *cholmod_solve(int sys, cholmod_factor *L, cholmod_dense *B, cholmod_common *c) {
    (void)sys;
    cholmod_dense *X = cholmod_zeros((size_t)L->m, 1, CHOLMOD_REAL, c);
    orc_gram G = {L->m, L->rp, L->ci, L->v};
    orc_gram_solve(&G, B->x, X->x);
    return X;
}

int cholmod_free_dense(cholmod_dense **X, cholmod_common *c) {
    (void)c;
    if (X && *X) { free((*X)->x); free(*X); *X = NULL; }
    return 1;
}
int cholmod_free_factor(cholmod_factor **L, cholmod_common *c) {
    (void)c;
    if (L && *L) { free((*L)->rp); free((*L)->ci); free((*L)->v); free(*L); *L = NULL; }
    return 1;
}
int cholmod_free_sparse(cholmod_sparse **A, cholmod_common *c) {
    (void)c;
    if (A && *A) { free((*A)->ri); free((*A)->ci); free((*A)->v); free(*A); *A = NULL; }
    return 1;
}
int cholmod_free_triplet(cholmod_triplet **T, cholmod_common *c) {
    (void)c;
    if (T && *T) { free((*T)->i); free((*T)->j); free((*T)->x); free(*T); *T = NULL; }
    return 1;
}
