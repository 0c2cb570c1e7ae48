/*
 * orc_gram.c -- (B B^T + beta I) assembly and conjugate-gradient solve, shared
 * by the oracle's ADMM (orc_core.c) and by the CHOLMOD stand-in used to build
 * the reference itself (ref/cholmod_shim.c), so that both perform the same
 * floating-point operations in the same order.
 * TEST INFRASTRUCTURE ONLY (see mcb_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc_gram.h"

typedef struct { int col, row; double v; } gent;
static int gent_cmp(const void *a, const void *b) {
    const gent *x = a, *y = b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->row < y->row ? -1 : (x->row > y->row);
}
typedef struct { int r, c; double v; } gtrip;
static int gtrip_cmp(const void *a, const void *b) {
    const gtrip *x = a, *y = b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    return x->c < y->c ? -1 : (x->c > y->c);
}

void orc_gram_build(int m, size_t nz, const int *rows, const int *cols, const double *vals, double beta,
                    orc_gram *G) {
    gent *e = malloc((nz + 1) * sizeof(gent));
    for (size_t k = 0; k < nz; ++k) { e[k].col = cols[k]; e[k].row = rows[k]; e[k].v = vals[k]; }
    qsort(e, nz, sizeof(gent), gent_cmp);
    size_t cap = (size_t)m + 16, nt = 0;
    gtrip *tr = malloc(cap * sizeof(gtrip));
    for (int q = 0; q < m; ++q) { tr[nt].r = q; tr[nt].c = q; tr[nt].v = beta; ++nt; }
    for (size_t s = 0; s < nz;) {
        size_t f = s;
        while (f < nz && e[f].col == e[s].col) ++f;
        for (size_t a = s; a < f; ++a)
            for (size_t b = s; b < f; ++b) {
                if (nt == cap) { cap *= 2; tr = realloc(tr, cap * sizeof(gtrip)); }
                tr[nt].r = e[a].row; tr[nt].c = e[b].row; tr[nt].v = e[a].v * e[b].v; ++nt;
            }
        s = f;
    }
    qsort(tr, nt, sizeof(gtrip), gtrip_cmp);
    G->m = m;
    G->L = NULL;
    G->rp = calloc((size_t)m + 1, sizeof(int));
    G->ci = malloc((nt + 1) * sizeof(int));
    G->v = malloc((nt + 1) * sizeof(double));
    size_t k = 0;
    for (size_t a = 0; a < nt;) {
        size_t b = a;
        double acc = 0.0;
        while (b < nt && tr[b].r == tr[a].r && tr[b].c == tr[a].c) acc += tr[b++].v;
        G->ci[k] = tr[a].c; G->v[k] = acc; G->rp[tr[a].r + 1]++; ++k;
        a = b;
    }
    for (int q = 0; q < m; ++q) G->rp[q + 1] += G->rp[q];
    free(e);
    free(tr);
}

void orc_gram_free(orc_gram *G) {
    free(G->rp); free(G->ci); free(G->v); free(G->L);
    G->rp = NULL; G->ci = NULL; G->v = NULL; G->L = NULL;
}

static int gram_direct = 0;
void orc_set_direct_solve(int on) { gram_direct = on != 0; }

/* dense lower Cholesky factor of G (column-major, m x m), left-looking; 0 on success */
static int gram_factor(orc_gram *G) {
    const int m = G->m;
    double *L = calloc((size_t)m * m + 1, sizeof(double));
    for (int i = 0; i < m; ++i)
        for (int k = G->rp[i]; k < G->rp[i + 1]; ++k) L[i + (size_t)G->ci[k] * m] = G->v[k];
    for (int j = 0; j < m; ++j) {
        double *cj = L + (size_t)j * m;
        for (int k = 0; k < j; ++k) {
            const double *ck = L + (size_t)k * m;
            const double ljk = ck[j];
            if (ljk == 0.0) continue;
            for (int i = j; i < m; ++i) cj[i] -= ck[i] * ljk;
        }
        if (!(cj[j] > 0.0)) { free(L); return -1; }
        const double d = sqrt(cj[j]);
        cj[j] = d;
        for (int i = j + 1; i < m; ++i) cj[i] /= d;
        for (int i = 0; i < j; ++i) cj[i] = 0.0;
    }
    G->L = L;
    return 0;
}

/* squared relative residual at which the solve stops (1e-15 by default) */
static double gram_tol2 = 1e-30;
void orc_set_cg_tol(double tol) { gram_tol2 = tol > 0 ? tol * tol : 1e-30; }

void orc_gram_solve(orc_gram *G, const double *b, double *x) {
    int m = G->m;
    if (gram_direct && (G->L || gram_factor(G) == 0)) {
        const double *L = G->L;
        for (int i = 0; i < m; ++i) x[i] = b[i];
        for (int j = 0; j < m; ++j) {  /* L y = b */
            const double *cj = L + (size_t)j * m;
            x[j] /= cj[j];
            for (int i = j + 1; i < m; ++i) x[i] -= cj[i] * x[j];
        }
        for (int j = m - 1; j >= 0; --j) {  /* L^T x = y */
            const double *cj = L + (size_t)j * m;
            double acc = x[j];
            for (int i = j + 1; i < m; ++i) acc -= cj[i] * x[i];
            x[j] = acc / cj[j];
        }
        return;
    }
    double *r = malloc(((size_t)m + 1) * sizeof(double)), *p = malloc(((size_t)m + 1) * sizeof(double));
    double *q = malloc(((size_t)m + 1) * sizeof(double));
    double bb = 0.0;
    for (int i = 0; i < m; ++i) { x[i] = 0.0; r[i] = b[i]; p[i] = b[i]; bb += b[i] * b[i]; }
    double rr = bb;
    for (int it = 0; it < 10000 && bb > 0.0 && rr > gram_tol2 * bb; ++it) {
        double pq = 0.0;
        for (int i = 0; i < m; ++i) {
            double acc = 0.0;
            for (int k = G->rp[i]; k < G->rp[i + 1]; ++k) acc += G->v[k] * p[G->ci[k]];
            q[i] = acc;
            pq += p[i] * acc;
        }
        double al = rr / pq, rr2 = 0.0;
        for (int i = 0; i < m; ++i) { x[i] += al * p[i]; r[i] -= al * q[i]; rr2 += r[i] * r[i]; }
        double be = rr2 / rr;
        for (int i = 0; i < m; ++i) p[i] = r[i] + be * p[i];
        rr = rr2;
    }
    free(r); free(p); free(q);
}
