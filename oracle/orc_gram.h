/* (B B^T + beta I) in CSR form and its CG solve (see orc_gram.c).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef ORC_GRAM_H
#define ORC_GRAM_H
#include <stddef.h>
typedef struct orc_gram { int m; int *rp, *ci; double *v; double *L; } orc_gram;
/* rows/cols/vals: the triplet of B (m x n^2), entries in the order admm.c:117-477 writes them */
void orc_gram_build(int m, size_t nz, const int *rows, const int *cols, const double *vals, double beta,
                    orc_gram *G);
void orc_gram_free(orc_gram *G);
/* x = G^{-1} b by conjugate gradients from x = 0 to relative residual 1e-15 (orc_set_cg_tol), or,
 * after orc_set_direct_solve(1), by a dense Cholesky factor of G (made at the first solve and kept
 * with G) -- the arithmetic of the reference's CHOLMOD factor and solve, admm.c:480-487,546, up to
 * ordering and rounding -- so that the conjugate-gradient stand-in can be compared with it */
void orc_gram_solve(orc_gram *G, const double *b, double *x);
void orc_set_cg_tol(double tol);
void orc_set_direct_solve(int on);
#endif
