/* (B B^T + beta I) in CSR form and its CG solve (see orc_gram.c).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef ORC_GRAM_H
#define ORC_GRAM_H
#include <stddef.h>
typedef struct orc_gram { int m; int *rp, *ci; double *v; } orc_gram;
/* rows/cols/vals: the triplet of B (m x n^2), entries in the order admm.c:117-477 writes them */
void orc_gram_build(int m, size_t nz, const int *rows, const int *cols, const double *vals, double beta,
                    orc_gram *G);
void orc_gram_free(orc_gram *G);
/* x = G^{-1} b by conjugate gradients from x = 0 to relative residual 1e-15 (orc_set_cg_tol) */
void orc_gram_solve(const orc_gram *G, const double *b, double *x);
void orc_set_cg_tol(double tol);
#endif
