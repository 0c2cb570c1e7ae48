/*
 * orc_core.c -- oracle: random streams, problem construction, cut operators,
 * PSD projection, basic-SDP IPM and the ADMM solver.
 * TEST INFRASTRUCTURE ONLY (see mcb_oracle.h).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "orc_internal.h"
#include "orc_gram.h"

orc_lapack orc_la;

static void *orc_sym(void *h, const char *name) {
    char buf[64];
    snprintf(buf, sizeof buf, "scipy_%s_", name);
    void *p = dlsym(h, buf);
    if (!p) {
        snprintf(buf, sizeof buf, "%s_", name);
        p = dlsym(h, buf);
    }
    return p;
}

int orc_lapack_init(const char *path) {
    if (orc_la.ready) return 0;
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    orc_la.dcopy = (orc_dcopy_t)orc_sym(h, "dcopy");
    orc_la.dscal = (orc_dscal_t)orc_sym(h, "dscal");
    orc_la.daxpy = (orc_daxpy_t)orc_sym(h, "daxpy");
    orc_la.ddot = (orc_ddot_t)orc_sym(h, "ddot");
    orc_la.dnrm2 = (orc_dnrm2_t)orc_sym(h, "dnrm2");
    orc_la.dsyevr = (orc_dsyevr_t)orc_sym(h, "dsyevr");
    orc_la.dpotrf = (orc_dpotrf_t)orc_sym(h, "dpotrf");
    orc_la.dpotri = (orc_dpotri_t)orc_sym(h, "dpotri");
    orc_la.dposv = (orc_dposv_t)orc_sym(h, "dposv");
    orc_la.dsymm = (orc_dsymm_t)orc_sym(h, "dsymm");
    orc_la.dsymv = (orc_dsymv_t)orc_sym(h, "dsymv");
    orc_la.dsyrk = (orc_dsyrk_t)orc_sym(h, "dsyrk");
    orc_la.dlansy = (orc_dlansy_t)orc_sym(h, "dlansy");
    if (!orc_la.dcopy || !orc_la.dscal || !orc_la.daxpy || !orc_la.ddot || !orc_la.dnrm2 ||
        !orc_la.dsyevr || !orc_la.dpotrf || !orc_la.dpotri || !orc_la.dposv || !orc_la.dsymm ||
        !orc_la.dsymv || !orc_la.dsyrk || !orc_la.dlansy)
        return -2;
    orc_la.ready = 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* glibc random() TYPE_3 (degree 31, separation 3), restated from its published
 * description: r[0] = seed, r[i] = 16807 r[i-1] mod (2^31-1) for i < 31,
 * r[i] = r[i-31] for 31 <= i < 34, r[i] = r[i-31] + r[i-3] (mod 2^32) after
 * that; output k is r[k+344] >> 1.  The reference seeds it with srand(2020)
 * (bab_functions.c:82). */
void orc_glibc_seed(orc_glibc *g, unsigned int seed) {
    int32_t r[34];
    r[0] = (int32_t)(seed == 0 ? 1 : seed);
    for (int i = 1; i < 31; ++i) {
        int32_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
        int32_t word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        r[i] = word;
    }
    for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
    for (int i = 0; i < 34; ++i) g->r[i] = (uint32_t)r[i];
    g->pos = 34; /* index of the next value to generate */
    for (int i = 34; i < 344; ++i) (void)orc_glibc_next(g);
}

int orc_glibc_next(orc_glibc *g) {
    int i = g->pos;
    uint32_t v = g->r[(i - 31) % 34] + g->r[(i - 3) % 34];
    g->r[i % 34] = v;
    g->pos = i + 1;
    if (g->pos >= 34 * 1000000) g->pos -= 34 * 999999; /* keep the index bounded, same residues */
    return (int)(v >> 1);
}

/* splitmix64 finaliser */
uint64_t orc_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t orc_key2(uint64_t a, uint64_t b) { return orc_mix64(a ^ orc_mix64(b + 0x632BE59BD9B4E019ull)); }

uint64_t orc_node_key(const int *xfixed, const int *sol, int pb) {
    uint64_t h = 0x4D414441u; /* arbitrary start value */
    for (int i = 0; i < pb; ++i)
        if (xfixed[i]) h = orc_key2(h, (uint64_t)(2 * i + (sol[i] ? 1 : 0)));
    return h;
}

uint64_t orc_stream_next(orc_stream *s) {
    s->ctr += 1;
    return orc_mix64(s->key + s->ctr * 0x9E3779B97F4A7C15ull);
}

int orc_rand_glibc(orc_ctx *c) { return orc_glibc_next(&c->g); }

/* ------------------------------------------------------------------------- */
void orc_default_params(orc_params *p) {
    /* defaults of admm.h:59-81 */
    p->sigma0 = 1.0;
    p->scaleSigma = 1.001;
    p->ADMM_itermax = 2000;
    p->tol0 = 5e-2;
    p->scaleTol = 0.6;
    p->minTol = 1e-4;
    p->triag_iter = 5;
    p->pent_iter = 5;
    p->hept_iter = 5;
    p->max_outer_iter = 20;
    p->extra_iter = 10;
    p->violated_TriIneq = 1e-3;
    p->TriIneq = 5000;
    p->adjust_TriIneq = 1;
    p->PentIneq = 5000;
    p->HeptaIneq = 5000;
    p->Pent_Trials = 60;
    p->Hepta_Trials = 50;
    p->include_Pent = 1;
    p->include_Hepta = 1;
    p->root = 0;
    p->use_diff = 1;
    p->branchingStrategy = 1;
}

/* Extended Laplacian, process_input.c:255-299:
 * L = [Lap, Lap e; (Lap e)^T, e^T Lap e] where Lap = Diag(A e) - A on the first
 * nv-1 vertices (degrees counted over all nv vertices). */
void orc_build_L(int nv, int ne, const int *ei, const int *ej, const double *w, double *L) {
    double *A = calloc((size_t)nv * nv, sizeof(double));
    double *deg = calloc((size_t)nv, sizeof(double));
    for (int e = 0; e < ne; ++e) {
        int i = ei[e] - 1, j = ej[e] - 1;
        A[(size_t)nv * j + i] = w[e];
        A[(size_t)nv * i + j] = w[e];
    }
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j < nv; ++j) deg[i] += A[j + (size_t)i * nv];
    double sum = 0.0;
    for (int ii = 0; ii < nv; ++ii) {
        double row = 0.0;
        for (int jj = 0; jj < nv; ++jj) {
            size_t at = jj + (size_t)ii * nv;
            if (ii < nv - 1 && jj < nv - 1) {
                L[at] = (ii == jj ? deg[ii] : 0.0) - A[at];
                row += L[at];
            } else if (jj == nv - 1 && ii != nv - 1) {
                L[at] = row;
                sum += row;
            } else if (ii == nv - 1 && jj != nv - 1) {
                L[at] = L[ii + (size_t)jj * nv];
            } else {
                L[at] = sum;
            }
        }
    }
    free(A);
    free(deg);
}

/* createSubproblem, evaluate.c:39-116.  Returns the subproblem size. */
int orc_create_subproblem(int N, const double *SL, const int *xfixed, const int *sol, double *PL) {
    int pb = N - 1, nfix = 0;
    for (int i = 0; i < pb; ++i) nfix += xfixed[i] ? 1 : 0;
    int n = pb + 1 - nfix;
    double *fixedRow = calloc((size_t)(n > 1 ? n - 1 : 1), sizeof(double));
    int index = 0;
    for (int i = 0; i < pb; ++i) {
        double row_sum = 0.0;
        int fixed = 0;
        for (int j = 0; j < pb; ++j) {
            if (!xfixed[i] && !xfixed[j]) {
                PL[index] = SL[j + (size_t)i * N];
                row_sum += PL[index];
                ++index;
            } else if ((xfixed[i] && sol[i] == 1) && !xfixed[j]) {
                fixedRow[fixed] += SL[j + (size_t)i * N];
                ++fixed;
            }
        }
        if (!xfixed[i]) {
            PL[index] = row_sum;
            ++index;
        }
    }
    for (int i = 0; i < n - 1; ++i) PL[i + (size_t)(n - 1) * n] = PL[n - 1 + (size_t)i * n];
    double sum = 0.0;
    for (int i = 0; i < n - 1; ++i) {
        PL[i + (size_t)i * n] += 2 * fixedRow[i];
        PL[n - 1 + (size_t)i * n] += 2 * fixedRow[i];
        PL[i + (size_t)(n - 1) * n] += 2 * fixedRow[i];
        sum += PL[i + (size_t)(n - 1) * n];
    }
    PL[n - 1 + (size_t)(n - 1) * n] = sum;
    for (size_t i = 0; i < (size_t)n * n; ++i) PL[i] *= 0.25;
    free(fixedRow);
    return n;
}

/* getFixedValue, evaluate.c:124-139 */
double orc_fixed_value(int N, const double *SL, const int *xfixed, const int *sol) {
    double v = 0.0;
    for (int i = 0; i < N - 1; ++i)
        for (int j = 0; j < N - 1; ++j)
            if (xfixed[i] && xfixed[j]) v += SL[j + (size_t)i * N] * sol[i] * sol[j];
    return v;
}

/* evaluateSolution, bab_functions.c:96-107 */
double orc_evaluate_solution(int N, const double *SL, const int *sol) {
    double v = 0.0;
    for (int i = 0; i < N - 1; ++i)
        for (int j = 0; j < N - 1; ++j) v += SL[j + (size_t)i * N] * sol[i] * sol[j];
    return v;
}

/* ------------------------------------------------------------------------- */
/* Cut families as signed cliques.  The sign patterns are those of op_B
 * (operators.c:81-148): triangle types 1-4, pentagonal H1-H3
 * (cutting_planes.c:242-244), heptagonal H1-H4 (cutting_planes.c:438-441). */
void orc_tri_clique(const int *tri, orc_clique *c) {
    static const int sg[4][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}};
    int type = tri[3];
    c->k = 3;
    c->p[0] = tri[0];
    c->p[1] = tri[1];
    c->p[2] = tri[2];
    const int *e = sg[(type >= 1 && type <= 4) ? type - 1 : 3];
    for (int a = 0; a < 3; ++a) c->e[a] = e[a];
    c->scale = 1.0;
}

void orc_pent_clique(const int *pent, orc_clique *c) {
    int type = pent[0];
    c->k = 5;
    for (int a = 0; a < 5; ++a) {
        c->p[a] = pent[1 + a];
        c->e[a] = 1;
    }
    if (type == 2) c->e[0] = -1;
    else if (type == 3) c->e[0] = c->e[1] = -1;
    c->scale = 0.5;
}

void orc_hept_clique(const int *hept, orc_clique *c) {
    int type = hept[0];
    c->k = 7;
    for (int a = 0; a < 7; ++a) {
        c->p[a] = hept[1 + a];
        c->e[a] = 1;
    }
    for (int a = 0; a < type - 1 && a < 3; ++a) c->e[a] = -1;
    c->scale = 1.0 / 3.0;
}

static inline double lowr(const double *X, int n, int a, int b) {
    /* the reference reads the lower triangle (row > col) */
    return a > b ? X[a + (size_t)b * n] : X[b + (size_t)a * n];
}

static double clique_apply(const orc_clique *c, const double *X, int n) {
    /* the reference's term order: pairs (a,b), a<b, in row-major order over a */
    double acc = 0.0;
    for (int a = 0; a < c->k; ++a)
        for (int b = a + 1; b < c->k; ++b) acc += (c->e[a] * c->e[b] > 0 ? -1.0 : 1.0) * lowr(X, n, c->p[a], c->p[b]);
    return c->scale * acc;
}

/* op_B, operators.c:62-150: y += B(X), X read through its lower triangle. */
void orc_op_B(int n, const double *X, int ntri, const int *tri, int npent, const int *pent,
              int nhept, const int *hept, double *y) {
    orc_clique c;
    for (int q = 0; q < ntri; ++q) {
        orc_tri_clique(tri + 4 * q, &c);
        y[q] += clique_apply(&c, X, n);
    }
    for (int q = 0; q < npent; ++q) {
        orc_pent_clique(pent + 6 * q, &c);
        y[ntri + q] += clique_apply(&c, X, n);
    }
    for (int q = 0; q < nhept; ++q) {
        orc_hept_clique(hept + 8 * q, &c);
        y[ntri + npent + q] += clique_apply(&c, X, n);
    }
}

static void clique_scatter(const orc_clique *c, double *X, int n, double tval) {
    double temp = 0.5 * c->scale * tval;
    for (int a = 0; a < c->k; ++a)
        for (int b = a + 1; b < c->k; ++b) {
            double v = (c->e[a] * c->e[b] > 0) ? temp : -temp;
            int i = c->p[a], j = c->p[b];
            X[i + (size_t)j * n] += v;
            X[j + (size_t)i * n] += v;
        }
}

/* op_Bt, operators.c:171-513: X -= B^T(t) on both triangles. */
void orc_op_Bt(int n, double *X, int ntri, const int *tri, int npent, const int *pent, int nhept,
               const int *hept, const double *t) {
    orc_clique c;
    for (int q = 0; q < ntri; ++q) {
        orc_tri_clique(tri + 4 * q, &c);
        clique_scatter(&c, X, n, t[q]);
    }
    for (int q = 0; q < npent; ++q) {
        orc_pent_clique(pent + 6 * q, &c);
        clique_scatter(&c, X, n, t[ntri + q]);
    }
    for (int q = 0; q < nhept; ++q) {
        orc_hept_clique(hept + 8 * q, &c);
        clique_scatter(&c, X, n, t[ntri + npent + q]);
    }
}

/* ------------------------------------------------------------------------- */
/* project_SDP, operators.c:521-619.  W is read through its lower triangle and
 * is not modified.  Xp receives X_+ in its lower triangle (upper triangle
 * copied from W, as dsyevr leaves the upper triangle of its input untouched),
 * Q = X_+ - W on the lower triangle and 0 on the strictly upper triangle, as the
 * reference's full-array daxpy produces.  Z receives the M eigenvectors of the
 * positive eigenvalues, each scaled by sqrt(lambda). */
/* LAPACK workspace sizes follow the reference's allocation for the original
 * problem size (allocate_free.c:31-32: 26 N and 10 N); LAPACK chooses blocked or
 * unblocked reductions from LWORK, so the size is part of the arithmetic. */
static int orc_work_n = 0;
void orc_set_work_n(int N) { orc_work_n = N; }
/* dsyevr's ABSTOL: the reference passes 1e-8 (operators.c:574, admm.c:738); the
 * counter (GPU-matching) form asks for full precision (0). */
static double orc_abstol = 1e-8;
void orc_set_abstol(double a) { orc_abstol = a; }
/* Newton-Schulz projection model (mcb_oracle.h); off while ns_k == 0 */
static int ns_k = 0;
static double ns_a[64], ns_b[64];
void orc_set_ns_schedule(int k, const double *a, const double *b) {
    ns_k = k < 0 ? 0 : (k > 64 ? 64 : k);
    for (int i = 0; i < ns_k; ++i) { ns_a[i] = a[i]; ns_b[i] = b[i]; }
}

int orc_project(int n, const double *W, double *Xp, double *Q, double *Z, double *evals,
                int canon_sign) {
    size_t nn = (size_t)n * n;
    double *A = malloc(nn * sizeof(double));
    memcpy(A, W, nn * sizeof(double));
    for (size_t i = 0; i < nn; ++i) Q[i] = -W[i];
    int wn = orc_work_n > n ? orc_work_n : n;
    int lwork = 26 * wn, liwork = 10 * wn; /* allocate_free.c:31-32 */
    double *work = malloc((size_t)lwork * sizeof(double));
    int *iwork = malloc((size_t)liwork * sizeof(int));
    int *isuppz = malloc((size_t)2 * n * sizeof(int));
    double VL = 1e-8, VU;
    double ninf = orc_la.dlansy("I", "L", &n, A, &n, work, 1, 1);
    double nfro = orc_la.dlansy("F", "L", &n, A, &n, work, 1, 1);
    VU = ninf < nfro ? ninf : nfro;
    if (VU < VL) VU = 2.0 * VL;
    int IL = 0, IU = 0, M = 0, info = 0;
    double abstol = orc_abstol;
    orc_la.dsyevr("V", "V", "L", &n, A, &n, &VL, &VU, &IL, &IU, &abstol, &M, evals, Z, &n, isuppz,
                  work, &lwork, iwork, &liwork, &info, 1, 1, 1);
    if (info != 0) { /* operators.c:583-593: retry with VL = 0, ABSTOL = 0 */
        memcpy(A, W, nn * sizeof(double));
        VL = 0.0;
        abstol = 0.0;
        orc_la.dsyevr("V", "V", "L", &n, A, &n, &VL, &VU, &IL, &IU, &abstol, &M, evals, Z, &n,
                      isuppz, work, &lwork, iwork, &liwork, &info, 1, 1, 1);
        if (info != 0) {
            free(A); free(work); free(iwork); free(isuppz);
            return -1;
        }
    }
    for (int j = 0; j < M; ++j) {
        double *col = Z + (size_t)j * n;
        if (canon_sign) {
            int arg = 0;
            double big = -1.0;
            for (int i = 0; i < n; ++i)
                if (fabs(col[i]) > big) { big = fabs(col[i]); arg = i; }
            if (col[arg] < 0)
                for (int i = 0; i < n; ++i) col[i] = -col[i];
        }
        double sc = sqrt(evals[j]);
        for (int i = 0; i < n; ++i) col[i] *= sc;
    }
    /* X_+ = Z Z^T on the lower triangle; the upper triangle keeps W's values */
    memcpy(Xp, W, nn * sizeof(double));
    double one = 1.0, zero = 0.0, mone = -1.0;
    if (ns_k > 0) {
        /* the sign iteration in exact arithmetic: every eigenvalue's step function becomes the
         * composed step polynomials at lambda / ||W||_F; positive and negative weights in two SYRKs */
        double *B = malloc(nn * sizeof(double)), *V = malloc(nn * sizeof(double));
        double *ev = malloc((size_t)n * sizeof(double));
        double *Vp = malloc(nn * sizeof(double)), *Vn = malloc(nn * sizeof(double));
        memcpy(B, W, nn * sizeof(double));
        int Ma = 0, info2 = 0, np_ = 0, nm_ = 0;
        double za = 0.0;
        orc_la.dsyevr("V", "A", "L", &n, B, &n, &VL, &VU, &IL, &IU, &za, &Ma, ev, V, &n, isuppz,
                      work, &lwork, iwork, &liwork, &info2, 1, 1, 1);
        for (int j = 0; j < Ma && info2 == 0; ++j) {
            double x = nfro > 0 ? ev[j] / nfro : 0.0;
            for (int k = 0; k < ns_k; ++k) x = ns_a[k] * x + ns_b[k] * x * x * x;
            double wgt = ev[j] * (1.0 + x) / 2.0;
            double *dst = wgt > 0 ? Vp + (size_t)np_++ * n : (wgt < 0 ? Vn + (size_t)nm_++ * n : NULL);
            if (!dst) continue;
            double sc = sqrt(fabs(wgt));
            for (int i = 0; i < n; ++i) dst[i] = V[i + (size_t)j * n] * sc;
        }
        for (int j = 0; j < n; ++j)
            for (int i = j; i < n; ++i) Xp[i + (size_t)j * n] = 0.0;
        if (np_) orc_la.dsyrk("L", "N", &n, &np_, &one, Vp, &n, &one, Xp, &n, 1, 1);
        if (nm_) orc_la.dsyrk("L", "N", &n, &nm_, &mone, Vn, &n, &one, Xp, &n, 1, 1);
        free(B); free(V); free(ev); free(Vp); free(Vn);
        if (info2 != 0) { free(A); free(work); free(iwork); free(isuppz); return -1; }
    } else if (M > 0) {
        orc_la.dsyrk("L", "N", &n, &M, &one, Z, &n, &zero, Xp, &n, 1, 1);
    } else {
        for (int j = 0; j < n; ++j)
            for (int i = j; i < n; ++i) Xp[i + (size_t)j * n] = 0.0;
    }
    for (size_t i = 0; i < nn; ++i) Q[i] += Xp[i];
    free(A); free(work); free(iwork); free(isuppz);
    return M;
}

/* largest eigenvalue, admm.c:731-752 (dsyevr RANGE='I', IL=IU=n, ABSTOL=1e-8) */
double orc_lambda_max(int n, const double *Ain) {
    size_t nn = (size_t)n * n;
    double *A = malloc(nn * sizeof(double));
    memcpy(A, Ain, nn * sizeof(double));
    int wn = orc_work_n > n ? orc_work_n : n;
    int lwork = 26 * wn, liwork = 10 * wn;
    double *work = malloc((size_t)lwork * sizeof(double));
    int *iwork = malloc((size_t)liwork * sizeof(int));
    int *isuppz = malloc((size_t)2 * n * sizeof(int));
    double zdummy[1];
    double VL = 0, VU = 0, abstol = orc_abstol, lam = NAN;
    int IL = n, IU = n, M = 0, info = 0, ldz = n;
    orc_la.dsyevr("N", "I", "L", &n, A, &n, &VL, &VU, &IL, &IU, &abstol, &M, &lam, zdummy, &ldz,
                  isuppz, work, &lwork, iwork, &liwork, &info, 1, 1, 1);
    free(A); free(work); free(iwork); free(isuppz);
    return info == 0 ? lam : NAN;
}

/* ------------------------------------------------------------------------- */
/* Basic SDP relaxation by the predictor-corrector IPM, ipm_mc_pk.c:28-347.
 * Returns the iteration count, or -1 if a factorisation fails. */
int orc_ipm(const double *L, int n, double *X, double *y, double *Z, double *phi) {
    size_t nn = (size_t)n * n;
    int inc = 1, info = 0, it, nni = (int)nn;
    double *dX = calloc(nn, sizeof(double)), *dZ = calloc(nn, sizeof(double));
    double *dX1 = calloc(nn, sizeof(double)), *tmp = calloc(nn, sizeof(double));
    double *tmp2 = calloc(nn, sizeof(double)), *Zi = calloc(nn, sizeof(double));
    double *Mm = calloc(nn, sizeof(double));
    double *dy = calloc((size_t)n, sizeof(double)), *dy1 = calloc((size_t)n, sizeof(double));
    double *b = malloc((size_t)n * sizeof(double));
    double one = 1.0, zero = 0.0, mone = -1.0;
    int ret = -1;

    for (int i = 0; i < n; ++i) y[i] = 0.0;
    for (int c = 0; c < n; ++c) {
        for (int r = 0; r < n; ++r) y[c] += fabs(L[r + (size_t)c * n]);
        y[c] += 1.1;
    }
    for (int i = 0; i < n; ++i) b[i] = 1.0;
    for (size_t i = 0; i < nn; ++i) X[i] = 0.0;
    for (int i = 0; i < n; ++i) X[i + (size_t)i * n] = 1.0;
    for (size_t i = 0; i < nn; ++i) Z[i] = 0.0;
    for (int i = 0; i < n; ++i) Z[i + (size_t)i * n] = y[i];
    orc_la.daxpy(&nni, &mone, L, &inc, Z, &inc);

    *phi = orc_la.ddot(&n, b, &inc, y, &inc);
    double psi = orc_la.ddot(&nni, L, &inc, X, &inc);
    double mu = orc_la.ddot(&nni, Z, &inc, X, &inc) / (2.0 * n);

    for (it = 1; *phi - psi > 1e-4; ++it) {
        if (it > 500) goto out;
        orc_la.dcopy(&nni, Z, &inc, Zi, &inc);
        orc_la.dpotrf("U", &n, Zi, &n, &info, 1);
        if (info != 0) goto out;
        orc_la.dpotri("U", &n, Zi, &n, &info, 1);
        if (info != 0) goto out;
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < j; ++k) Zi[j + (size_t)n * k] = Zi[k + (size_t)n * j];

        /* predictor */
        for (size_t j = 0; j < nn; ++j) Mm[j] = Zi[j] * X[j];
        orc_la.dcopy(&n, b, &inc, dy1, &inc);
        orc_la.dscal(&n, &mone, dy1, &inc);
        orc_la.dposv("U", &n, &inc, Mm, &n, dy1, &n, &info, 1);
        if (info != 0) goto out;
        for (size_t j = 0; j < nn; ++j) tmp[j] = -(dy1[j % n]) * X[j];
        orc_la.dsymm("L", "U", &n, &n, &one, Zi, &n, tmp, &n, &zero, dX1, &n, 1, 1);
        orc_la.daxpy(&nni, &mone, X, &inc, dX1, &inc);
        for (int j = 0; j < n; ++j)
            for (int k = 0; k <= j; ++k) {
                double v = 0.5 * (dX1[j + (size_t)n * k] + dX1[k + (size_t)n * j]);
                dX1[j + (size_t)n * k] = v;
                dX1[k + (size_t)n * j] = v;
            }

        /* corrector */
        for (int i = 0; i < n; ++i) dy[i] = Zi[i + (size_t)i * n];
        for (size_t j = 0; j < nn; ++j) tmp[j] = Zi[j] * dX1[j];
        orc_la.dsymv("U", &n, &mone, tmp, &n, dy1, &inc, &mu, dy, &inc, 1);
        for (size_t j = 0; j < nn; ++j) Mm[j] = Zi[j] * X[j];
        orc_la.dposv("U", &n, &inc, Mm, &n, dy, &n, &info, 1);
        if (info != 0) goto out;
        for (size_t j = 0; j < nn; ++j) tmp[j] = -(dy[j % n]) * X[j];
        for (size_t j = 0; j < nn; ++j) tmp2[j] = -(dy1[j % n]) * dX1[j];
        orc_la.daxpy(&nni, &one, tmp2, &inc, tmp, &inc);
        orc_la.dsymm("L", "U", &n, &n, &one, Zi, &n, tmp, &n, &zero, dX, &n, 1, 1);
        orc_la.daxpy(&nni, &mu, Zi, &inc, dX, &inc);
        orc_la.daxpy(&n, &one, dy1, &inc, dy, &inc);
        orc_la.daxpy(&nni, &one, dX1, &inc, dX, &inc);
        for (int j = 0; j < n; ++j)
            for (int k = 0; k <= j; ++k) {
                double v = 0.5 * (dX[j + (size_t)n * k] + dX[k + (size_t)n * j]);
                dX[j + (size_t)n * k] = v;
                dX[k + (size_t)n * j] = v;
            }
        for (size_t j = 0; j < nn; ++j) dZ[j] = 0.0;
        for (int i = 0; i < n; ++i) dZ[i + (size_t)i * n] = dy[i];

        /* step lengths by Cholesky line search */
        double ap = 1.0, ad = 1.0;
        for (int ls = 0;; ++ls) {
            if (ls > 400) goto out;
            orc_la.dcopy(&nni, X, &inc, tmp, &inc);
            orc_la.daxpy(&nni, &ap, dX, &inc, tmp, &inc);
            orc_la.dpotrf("U", &n, tmp, &n, &info, 1);
            if (info == 0) break;
            ap *= 0.8;
        }
        if (ap < 1.0) ap *= 0.95;
        for (int ls = 0;; ++ls) {
            if (ls > 400) goto out;
            orc_la.dcopy(&nni, Z, &inc, tmp, &inc);
            orc_la.daxpy(&nni, &ad, dZ, &inc, tmp, &inc);
            orc_la.dpotrf("U", &n, tmp, &n, &info, 1);
            if (info == 0) break;
            ad *= 0.8;
        }
        if (ad < 1.0) ad *= 0.95;

        orc_la.daxpy(&nni, &ap, dX, &inc, X, &inc);
        orc_la.daxpy(&n, &ad, dy, &inc, y, &inc);
        orc_la.daxpy(&nni, &ad, dZ, &inc, Z, &inc);
        mu = orc_la.ddot(&nni, Z, &inc, X, &inc) / (2.0 * n);
        if (ap + ad > 1.6) mu *= 0.5;
        if (ap + ad > 1.9) mu *= 0.2;
        *phi = orc_la.ddot(&n, b, &inc, y, &inc);
        psi = orc_la.ddot(&nni, L, &inc, X, &inc);
    }
    ret = it - 1;
out:
    free(dX); free(dZ); free(dX1); free(tmp); free(tmp2); free(Zi); free(Mm); free(dy); free(dy1); free(b);
    return ret;
}

/* ------------------------------------------------------------------------- */
/* (B B^T + I).  The reference builds B as a CHOLMOD triplet (admm.c:117-477) and
 * factors B B^T + I once per ADMM call (admm.c:486-487).  The oracle writes the
 * same triplet, entry for entry in the reference's order, and hands it to the
 * assembly + CG solve of orc_gram.c. */
/* (row, col) positions into the cut's vertex list, in the order admm.c writes them */
static const int TRI_RC[6][2] = {{0, 1}, {1, 0}, {2, 0}, {0, 2}, {1, 2}, {2, 1}};
static const int PENT_RC[20][2] = {{0, 1}, {1, 0}, {2, 0}, {0, 2}, {3, 0}, {0, 3}, {4, 0}, {0, 4}, {2, 1}, {1, 2},
                                   {3, 1}, {1, 3}, {4, 1}, {1, 4}, {3, 2}, {2, 3}, {4, 2}, {2, 4}, {4, 3}, {3, 4}};
static const int HEPT_RC[42][2] = {{0, 1}, {1, 0}, {0, 2}, {2, 0}, {0, 3}, {3, 0}, {0, 4}, {4, 0}, {0, 5}, {5, 0},
                                   {0, 6}, {6, 0}, {2, 1}, {1, 2}, {3, 1}, {1, 3}, {4, 1}, {1, 4}, {5, 1}, {1, 5},
                                   {6, 1}, {1, 6}, {3, 2}, {2, 3}, {4, 2}, {2, 4}, {5, 2}, {2, 5}, {6, 2}, {2, 6},
                                   {4, 3}, {3, 4}, {5, 3}, {3, 5}, {6, 3}, {3, 6}, {5, 4}, {4, 5}, {6, 4}, {4, 6},
                                   {6, 5}, {5, 6}};

static void expand_cut(const orc_ctx *c, int q, orc_clique *cl) {
    if (q < c->ntri) orc_tri_clique(c->tri + 4 * q, cl);
    else if (q < c->ntri + c->npent) orc_pent_clique(c->pent + 6 * (q - c->ntri), cl);
    else orc_hept_clique(c->hept + 8 * (q - c->ntri - c->npent), cl);
}

static void build_gram(const orc_ctx *c, orc_gram *G) {
    int m = c->ntri + c->npent + c->nhept, n = c->n;
    size_t nz = (size_t)6 * c->ntri + 20 * (size_t)c->npent + 42 * (size_t)c->nhept, w = 0;
    int *rows = malloc((nz + 1) * sizeof(int)), *cols = malloc((nz + 1) * sizeof(int));
    double *vals = malloc((nz + 1) * sizeof(double));
    orc_clique cl;
    for (int q = 0; q < m; ++q) {
        expand_cut(c, q, &cl);
        const int(*rc)[2] = cl.k == 3 ? TRI_RC : (cl.k == 5 ? PENT_RC : HEPT_RC);
        int cnt = cl.k * (cl.k - 1);
        for (int e = 0; e < cnt; ++e) {
            int a = rc[e][0], b = rc[e][1];
            rows[w] = q;
            cols[w] = cl.p[a] + cl.p[b] * n;
            vals[w] = -0.5 * cl.scale * cl.e[a] * cl.e[b];
            ++w;
        }
    }
    orc_gram_build(m, w, rows, cols, vals, 1.0, G);
    free(rows); free(cols); free(vals);
}

static double nrm2(const double *v, int n) {
    int inc = 1;
    return orc_la.dnrm2(&n, v, &inc);
}

static double fro_lower(const double *A, int n) {
    double dummy[1];
    return orc_la.dlansy("F", "L", &n, A, &n, dummy, 1, 1);
}

/* Studies of the projection's input: every W the ADMM projects is appended to this
 * file (int n, then the n x n column-major doubles) while it is open. */
static FILE *proj_dump = NULL;
void orc_set_projection_dump(const char *path) {
    if (proj_dump) fclose(proj_dump);
    proj_dump = path ? fopen(path, "wb") : NULL;
}

/* ADMM_solver, admm.c:49-771.  Works on c->X, c->y, c->Q, c->t, c->s, c->u and
 * the cut lists; leaves the safe bound in c->f and the heuristic's factor in c->Z. */
int orc_admm(orc_ctx *c, double *sigma, double tol, int *nbit) {
    int n = c->n, m = c->ntri + c->npent + c->nhept;
    size_t nn = (size_t)n * n;
    const double *L = c->L;
    double *X = c->X, *Q = c->Q, *y = c->y, *t = c->t, *s = c->s, *u = c->u;
    for (int q = 0; q < c->ntri; ++q) { s[q] = t[q] = c->tri_y[q]; u[q] = 0.0; }
    for (int q = 0; q < c->npent; ++q) { s[c->ntri + q] = t[c->ntri + q] = c->pent_y[q]; u[c->ntri + q] = 0.0; }
    for (int q = 0; q < c->nhept; ++q) {
        int o = c->ntri + c->npent + q;
        s[o] = t[o] = c->hept_y[q];
        u[o] = 0.0;
    }
    orc_gram G;
    build_gram(c, &G);
    double *tmp = malloc(nn * sizeof(double)), *rhs = malloc(((size_t)m + 1) * sizeof(double));
    double *res = malloc((size_t)n * sizeof(double)), *v = malloc(((size_t)m + 1) * sizeof(double));
    double *cg_x = malloc(((size_t)m + 1) * sizeof(double));
    double *evals = malloc((size_t)n * sizeof(double));
    double normL = fro_lower(L, n);
    *nbit = 0;
    int err_flag = 0;
    while (*nbit <= c->prm.ADMM_itermax) {
        (*nbit)++;
        double sg = *sigma;
        for (int i = 0; i < n; ++i) y[i] = L[i + (size_t)i * n] + Q[i + (size_t)i * n] + (X[i + (size_t)i * n] - 1.0) / sg;
        for (size_t i = 0; i < nn; ++i) tmp[i] = L[i] + Q[i] + X[i] / sg;
        for (int i = 0; i < m; ++i) t[i] = s[i];
        orc_op_B(n, tmp, c->ntri, c->tri, c->npent, c->pent, c->nhept, c->hept, t);
        for (int i = 0; i < m; ++i) t[i] += (u[i] - 1) / sg;
        orc_gram_solve(&G, t, cg_x);
        for (int i = 0; i < m; ++i) t[i] = cg_x[i];
        for (int i = 0; i < m; ++i) {
            v[i] = t[i] - u[i] / sg;
            s[i] = v[i] > 0 ? v[i] : 0;
        }
        for (size_t i = 0; i < nn; ++i) X[i] = L[i] + X[i] / sg;
        for (int i = 0; i < n; ++i) X[i + (size_t)i * n] -= y[i];
        orc_op_Bt(n, X, c->ntri, c->tri, c->npent, c->pent, c->nhept, c->hept, t);
        /* project_SDP(PP): X <- X_+ (lower), Q <- X_+ - W */
        memcpy(tmp, X, nn * sizeof(double));
        if (proj_dump) {
            fwrite(&n, sizeof(int), 1, proj_dump);
            fwrite(tmp, sizeof(double), (size_t)n * n, proj_dump);
        }
        int M = orc_project(n, tmp, X, Q, c->Z, evals, c->canon_sign);
        if (M < 0) { err_flag = 1; break; }
        c->M = M;
        for (size_t i = 0; i < nn; ++i) X[i] *= sg;
        double sca = sqrt(sg);
        for (size_t i = 0; i < (size_t)n * M; ++i) c->Z[i] *= sca;
        for (int i = 0; i < m; ++i) u[i] = (v[i] < 0) ? -sg * v[i] : 0;
        /* primal residual */
        for (int i = 0; i < n; ++i) res[i] = X[i + (size_t)i * n] - 1.0;
        double err_p = nrm2(res, n);
        for (int i = 0; i < m; ++i) rhs[i] = -1.0;
        orc_op_B(n, X, c->ntri, c->tri, c->npent, c->pent, c->nhept, c->hept, rhs);
        for (int i = 0; i < m; ++i) rhs[i] = rhs[i] > 0 ? rhs[i] : 0;
        err_p += nrm2(rhs, m);
        err_p /= (1 + sqrt(n));
        /* dual residual */
        for (int i = 0; i < m; ++i) rhs[i] = s[i] - t[i];
        double err_d = nrm2(rhs, m);
        for (size_t i = 0; i < nn; ++i) tmp[i] = L[i] + Q[i];
        for (int i = 0; i < n; ++i) tmp[i + (size_t)i * n] -= y[i];
        orc_op_Bt(n, tmp, c->ntri, c->tri, c->npent, c->pent, c->nhept, c->hept, t);
        err_d += fro_lower(tmp, n);
        err_d /= (1 + normL);
        /* objectives */
        double primal = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i; j < n; ++j) {
                if (i == j) primal += L[i + (size_t)i * n] * X[i + (size_t)i * n];
                else primal += 2 * L[j + (size_t)i * n] * X[j + (size_t)i * n];
            }
        double dual = 0.0;
        for (int i = 0; i < n; ++i) dual += y[i];
        for (int i = 0; i < m; ++i) dual += t[i];
        double gap = fabs(dual - primal) / (1 + fabs(dual) + fabs(primal));
        double err = err_p > err_d ? (err_p > gap ? err_p : gap) : (err_d > gap ? err_d : gap);
        double dp = log10(err_p), dd = log10(err_d);
        if (c->trace && c->trace_len + 4 <= c->trace_cap) {
            c->trace[c->trace_len++] = err_p;
            c->trace[c->trace_len++] = err_d;
            c->trace[c->trace_len++] = gap;
            c->trace[c->trace_len++] = *sigma;
        }
        if (dd - dp < -0.5) *sigma /= c->prm.scaleSigma;
        else if (dd - dp > 0.5) *sigma *= c->prm.scaleSigma;
        if (err < tol) break;
    }
    if (!err_flag) {
        /* safe bound, admm.c:724-763 */
        memcpy(tmp, L, nn * sizeof(double));
        for (int i = 0; i < n; ++i) tmp[i + (size_t)i * n] -= y[i];
        orc_op_Bt(n, tmp, c->ntri, c->tri, c->npent, c->pent, c->nhept, c->hept, s);
        double lmax = orc_lambda_max(n, tmp);
        if (isnan(lmax)) err_flag = 1;
        c->f = n * lmax;
        for (int i = 0; i < n; ++i) c->f += y[i];
        for (int i = 0; i < m; ++i) c->f += s[i];
    }
    orc_gram_free(&G);
    free(tmp); free(rhs); free(res); free(v); free(cg_x); free(evals);
    return err_flag ? -1 : 0;
}
