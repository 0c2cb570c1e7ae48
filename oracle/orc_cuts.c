/*
 * orc_cuts.c -- oracle: triangle / pentagonal / heptagonal separation and the
 * purge-dedup-append bookkeeping (cutting_planes.c), k-gonal simulated annealing
 * (qap_simulated_annealing.c).
 * TEST INFRASTRUCTURE ONLY (see mcb_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc_internal.h"

/* evaluateTriangleInequality, cutting_planes.c:20-39 */
static inline double tri_value(const double *X, int N, int type, int ii, int jj, int kk) {
    double a = X[ii + (size_t)jj * N], b = X[ii + (size_t)kk * N], c = X[jj + (size_t)kk * N];
    switch (type) {
    case 1: return -a - b - c - 1.0;
    case 2: return -a + b + c - 1.0;
    case 3: return a - b + c - 1.0;
    default: return a + b - c - 1.0;
    }
}

typedef struct { double v; long long scan; int i, j, k, type; } orc_cand;

static int cand_by_value(const void *a, const void *b) {
    const orc_cand *x = a, *y = b;
    if (x->v != y->v) return x->v > y->v ? -1 : 1; /* larger violation first */
    return x->scan < y->scan ? -1 : (x->scan > y->scan);
}
static int cand_by_scan(const void *a, const void *b) {
    const orc_cand *x = a, *y = b;
    return x->scan < y->scan ? -1 : (x->scan > y->scan);
}

/* getViolated_TriangleInequalities, cutting_planes.c:48-127.
 * mode ORC_TOPK_REFERENCE replays the reference's list-replacement procedure.
 * mode ORC_TOPK_CANONICAL keeps the K largest violations (ties to the earlier
 * scan position) and lists them in scan order; with distinct values both modes
 * select the same set.  Returns the maximum violation over all triples. */
double orc_sep_triangles(const double *X, int N, int K, double thr, int mode, int *out,
                         double *vals, int *count) {
    double maxAll = -ORC_BIG;
    int size = 0;
    if (mode == ORC_TOPK_REFERENCE) {
        int least = 0;
        double leastv = ORC_BIG;
        for (int type = 1; type <= 4; ++type)
            for (int ii = 0; ii < N; ++ii)
                for (int jj = 0; jj < ii; ++jj)
                    for (int kk = 0; kk < jj; ++kk) {
                        double v = tri_value(X, N, type, ii, jj, kk);
                        maxAll = v > maxAll ? v : maxAll;
                        if (!(v > thr)) continue;
                        if (size < K) {
                            int *o = out + 4 * size;
                            o[0] = ii; o[1] = jj; o[2] = kk; o[3] = type;
                            vals[size] = v;
                            if (size == 0 || v < leastv) { leastv = v; least = size; }
                            ++size;
                        } else if (v > leastv) {
                            int *o = out + 4 * least;
                            o[0] = ii; o[1] = jj; o[2] = kk; o[3] = type;
                            vals[least] = v;
                            leastv = ORC_BIG;
                            for (int q = 0; q < size; ++q)
                                if (vals[q] < leastv) { leastv = vals[q]; least = q; }
                        }
                    }
        *count = size;
        return maxAll;
    }
    /* canonical: collect all violated, select top K, list in scan order */
    size_t cap = 1024, nc = 0;
    orc_cand *cs = malloc(cap * sizeof(orc_cand));
    long long scan = 0;
    for (int type = 1; type <= 4; ++type)
        for (int ii = 0; ii < N; ++ii)
            for (int jj = 0; jj < ii; ++jj)
                for (int kk = 0; kk < jj; ++kk, ++scan) {
                    double v = tri_value(X, N, type, ii, jj, kk);
                    maxAll = v > maxAll ? v : maxAll;
                    if (!(v > thr)) continue;
                    if (nc == cap) { cap *= 2; cs = realloc(cs, cap * sizeof(orc_cand)); }
                    cs[nc].v = v; cs[nc].scan = scan; cs[nc].i = ii; cs[nc].j = jj; cs[nc].k = kk; cs[nc].type = type;
                    ++nc;
                }
    if ((long long)nc > K) {
        qsort(cs, nc, sizeof(orc_cand), cand_by_value);
        nc = (size_t)K;
    }
    qsort(cs, nc, sizeof(orc_cand), cand_by_scan);
    for (size_t q = 0; q < nc; ++q) {
        out[4 * q] = cs[q].i; out[4 * q + 1] = cs[q].j; out[4 * q + 2] = cs[q].k; out[4 * q + 3] = cs[q].type;
        vals[q] = cs[q].v;
    }
    *count = (int)nc;
    free(cs);
    return maxAll;
}

/* updateTriangleInequalities, cutting_planes.c:132-214 */
double orc_update_tri(orc_ctx *c, const double *s, int *added, int *subtracted) {
    int sub = 0, next = 0;
    for (int q = 0; q < c->ntri; ++q) {
        c->tri_y[q] = s[q];
        if (c->tri_y[q] < 1e-5) { ++sub; continue; }
        memmove(c->tri + 4 * next, c->tri + 4 * q, 4 * sizeof(int));
        c->tri_y[next] = c->tri_y[q];
        ++next;
    }
    c->ntri -= sub;
    int cnt = 0;
    double maxAll = orc_sep_triangles(c->X, c->n, c->prm.TriIneq, c->prm.violated_TriIneq, c->topk_mode,
                                      c->list_i, c->list_v, &cnt);
    int add = 0;
    for (int l = 0; l < cnt; ++l) {
        if (next == ORC_MAX_TRI) break;
        const int *cand = c->list_i + 4 * l;
        int found = 0;
        for (int q = 0; q < c->ntri; ++q) {
            const int *e = c->tri + 4 * q;
            if (e[3] == cand[3] && e[0] == cand[0] && e[1] == cand[1] && e[2] == cand[2]) { found = 1; break; }
        }
        if (!found) {
            memcpy(c->tri + 4 * next, cand, 4 * sizeof(int));
            c->tri_y[next] = 0.0;
            ++next;
            ++add;
        }
    }
    c->ntri += add;
    *added = add;
    *subtracted = sub;
    return maxAll;
}

/* ------------------------------------------------------------------------- */
/* qap_simulated_annealing, qap_simulated_annealing.c:12-206.
 * X must be the full symmetric matrix (the reference copies the lower triangle
 * to the upper one first, :15-17).  In glibc mode the draws come from the
 * global stream g; in counter mode from the stream keyed by `key`. */
typedef struct { int mode; orc_glibc *g; orc_stream st; } orc_draw;
static inline int draw_int(orc_draw *d) {
    if (d->mode == ORC_RNG_GLIBC) return orc_glibc_next(d->g);
    return (int)(orc_stream_next(&d->st) >> 33); /* 31 random bits, same range as rand() */
}
static inline double draw_unit(orc_draw *d) {
    if (d->mode == ORC_RNG_GLIBC) return (double)orc_glibc_next(d->g) / (double)2147483647;
    return (double)(orc_stream_next(&d->st) >> 11) * 0x1.0p-53;
}

double orc_qap_sa(const int *H, int k, const double *X, int n, int rng_mode, orc_glibc *g,
                  uint64_t key, int *ineq) {
    orc_draw d;
    d.mode = rng_mode;
    d.g = g;
    d.st.key = key;
    d.st.ctr = 0;
    const int inner_iter = n;
    const double reduce_temp = 0.6, increase_iter = 1.1;
    double t = k * k;
    double sumX = 0;
    for (int i = 0; i < n; ++i) {
        sumX += X[i + (size_t)i * n];
        for (int j = i + 1; j < n; ++j) sumX += 2 * fabs(X[j + (size_t)i * n]);
    }
    t *= sumX;
    t /= (n * (n - 1));
    double cost = ORC_BIG;
    int *perm = malloc((size_t)n * sizeof(int));
    int *best = malloc((size_t)k * sizeof(int));
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int i = n - 1; i > 0; --i) {
        int r = draw_int(&d) % i;
        int tmp = perm[i]; perm[i] = perm[r]; perm[r] = tmp;
    }
    for (int i = 0; i < k; ++i) best[i] = perm[i];
    double t1 = t;
    int m1 = inner_iter;
    double sol = 0;
    for (int i = 0; i < k; ++i) {
        sol += X[perm[i] + (size_t)perm[i] * n];
        for (int j = i + 1; j < k; ++j) sol += 2 * H[j + i * k] * X[perm[j] + (size_t)perm[i] * n];
    }
    int not_done = 1, sweeps = 0;
    while (not_done > 0) {
        not_done = 0;
        /* counter mode bounds the sweeps as the GPU build does */
        if (rng_mode == ORC_RNG_COUNTER && ++sweeps > ORC_SA_MAX_SWEEPS) break;
        for (int it = 0; it < m1; ++it) {
            int i1 = draw_int(&d) % k;
            int i2 = draw_int(&d) % n;
            if (i2 < i1) { int tmp = i1; i1 = i2; i2 = tmp; }
            double delta = 0.0;
            for (int i = 0; i < k; ++i)
                delta += H[i + k * i1] * (X[perm[i] + (size_t)n * perm[i2]] - X[perm[i] + (size_t)n * perm[i1]]);
            if (i2 < k)
                for (int i = 0; i < k; ++i)
                    delta += H[i + k * i2] * (X[perm[i] + (size_t)n * perm[i1]] - X[perm[i] + (size_t)n * perm[i2]]);
            delta *= 2.0;
            double tv1 = X[perm[i1] + (size_t)n * perm[i1]] + X[perm[i2] + (size_t)n * perm[i2]] -
                         2.0 * X[perm[i2] + (size_t)n * perm[i1]];
            double tv2 = 1.0;
            if (i2 < k) tv2 += -2 * H[i1 + k * i2] + 1.0;
            delta += tv1 * tv2;
            /* Counter mode: a delta that is zero up to rounding noise counts as exactly
             * zero, so the accept test (and whether it draws) does not depend on the
             * last bits of X.  glibc mode keeps the reference's behaviour. */
            if (rng_mode == ORC_RNG_COUNTER && fabs(delta) < ORC_SA_ZERO) delta = 0.0;
            double sol_temp = sol + delta;
            int accept;
            if (delta > 0) {
                double dt1 = delta / t1;
                if (dt1 > 5) accept = 0;
                else accept = draw_unit(&d) < exp(-dt1);
            } else {
                accept = 1;
            }
            if (accept) {
                if (fabs(delta) > 0.0001) not_done = 1;
                int tmp = perm[i1]; perm[i1] = perm[i2]; perm[i2] = tmp;
                sol = sol_temp;
                if (sol < cost) {
                    cost = sol;
                    for (int i = 0; i < k; ++i) best[i] = perm[i];
                }
            }
        }
        t1 *= reduce_temp;
        m1 = (int)round(m1 * increase_iter);
    }
    for (int i = 0; i < k; ++i) ineq[i] = best[i];
    free(perm);
    free(best);
    return cost;
}

/* H matrices of cutting_planes.c:242-244 and :438-441, built as e e^T */
static void kgon_H(int k, int type, int *H) {
    int e[7];
    for (int a = 0; a < k; ++a) e[a] = (a < type - 1) ? -1 : 1;
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) H[a + k * b] = e[a] * e[b];
}

/* symmetric full copy of X (qap_simulated_annealing.c:15-17 symmetrises in place) */
static double *sym_full(const orc_ctx *c) {
    int n = c->n;
    double *S = malloc((size_t)n * n * sizeof(double));
    memcpy(S, c->X, (size_t)n * n * sizeof(double));
    for (int row = 0; row < n; ++row)
        for (int col = 0; col < row; ++col) S[col + (size_t)n * row] = S[row + (size_t)n * col];
    return S;
}

/* getViolated_Pentagonal/HeptagonalInequalities, cutting_planes.c:224-309, 419-506.
 * Fills list (type, p[k]) and values; returns the minimum SA value. */
static double sep_kgon(orc_ctx *c, int k, int trials, int cap, int *list, double *vals, int *count) {
    int ntypes = (k == 5) ? 3 : 4, stride = k + 1, size = 0, least = 0;
    double leastv = -ORC_BIG, minAll = ORC_BIG;
    int H[49], kg[7];
    int n = c->n;
    if (n < k) { *count = 0; return minAll; } /* the reference would read past perm[] here */
    double *S = sym_full(c);
    for (int trial = 0; trial < trials; ++trial)
        for (int type = 1; type <= ntypes; ++type) {
            kgon_H(k, type, H);
            uint64_t key = orc_key2(orc_key2(orc_key2(c->node_key, (uint64_t)c->sep_round), (uint64_t)k),
                                    (uint64_t)(trial * 8 + type));
            double v = orc_qap_sa(H, k, S, n, c->rng_mode, &c->g, key, kg);
            minAll = v < minAll ? v : minAll;
            if (!(v < 1.0)) continue;
            if (size < cap) {
                int *o = list + stride * size;
                o[0] = type;
                for (int a = 0; a < k; ++a) o[1 + a] = kg[a];
                vals[size] = v;
                if (size == 0 || v > leastv) { leastv = v; least = size; }
                ++size;
            } else if (v < leastv) {
                int *o = list + stride * least;
                o[0] = type;
                for (int a = 0; a < k; ++a) o[1 + a] = kg[a];
                vals[least] = v;
                leastv = ORC_BIG;
                for (int q = 0; q < size; ++q)
                    if (vals[q] > leastv) { leastv = vals[q]; least = q; }
            }
        }
    free(S);
    *count = size;
    return minAll;
}

/* updatePentagonal/HeptagonalInequalities, cutting_planes.c:316-409, 512-605 */
static double update_kgon(orc_ctx *c, int k, const double *s, int *added, int *subtracted, int yoff) {
    int *cuts = (k == 5) ? c->pent : c->hept;
    double *cy = (k == 5) ? c->pent_y : c->hept_y;
    int *ncut = (k == 5) ? &c->npent : &c->nhept;
    int cap = (k == 5) ? ORC_MAX_PENT : ORC_MAX_HEPT;
    int listcap = (k == 5) ? c->prm.PentIneq : c->prm.HeptaIneq;
    int trials = (k == 5) ? c->prm.Pent_Trials : c->prm.Hepta_Trials;
    int stride = k + 1, sub = 0, next = 0;
    for (int q = 0; q < *ncut; ++q) {
        cy[q] = s[yoff + q];
        if (cy[q] < 1e-5) { ++sub; continue; }
        memmove(cuts + stride * next, cuts + stride * q, (size_t)stride * sizeof(int));
        cy[next] = cy[q];
        ++next;
    }
    *ncut -= sub;
    int ntypes = (k == 5) ? 3 : 4;
    int lcap = trials * ntypes < listcap ? trials * ntypes : listcap;
    int *list = malloc(((size_t)(lcap > 0 ? lcap : 1)) * stride * sizeof(int));
    double *vals = malloc(((size_t)(lcap > 0 ? lcap : 1)) * sizeof(double));
    int cnt = 0;
    double minAll = sep_kgon(c, k, trials, listcap, list, vals, &cnt);
    int add = 0;
    for (int l = 0; l < cnt; ++l) {
        if (next == cap) break;
        const int *cand = list + stride * l;
        int found = 0;
        for (int q = 0; q < *ncut; ++q)
            if (memcmp(cuts + stride * q, cand, (size_t)stride * sizeof(int)) == 0) { found = 1; break; }
        if (!found) {
            memcpy(cuts + stride * next, cand, (size_t)stride * sizeof(int));
            cy[next] = 0.0;
            ++next;
            ++add;
        }
    }
    *ncut += add;
    *added = add;
    *subtracted = sub;
    free(list);
    free(vals);
    return minAll;
}

double orc_update_pent(orc_ctx *c, const double *s, int *added, int *subtracted, int triag) {
    return update_kgon(c, 5, s, added, subtracted, triag);
}

double orc_update_hept(orc_ctx *c, const double *s, int *added, int *subtracted, int off) {
    return update_kgon(c, 7, s, added, subtracted, off);
}
