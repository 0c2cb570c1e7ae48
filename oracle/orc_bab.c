/*
 * orc_bab.c -- oracle: SDPbound (bounding.c), Evaluate (evaluate.c), the GW +
 * 1-opt heuristic (heuristic.c), the max-heap (heap.c) and a serial
 * branch-and-bound driver standing in for the MPI master/worker loop
 * (bab_functions.c:39-69, 226-334; main.c).
 * TEST INFRASTRUCTURE ONLY (see mcb_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <stdio.h>

#include "orc_internal.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

orc_ctx *orc_create(const orc_params *p, int N, const double *SL, int rng_mode, int topk_mode,
                    int canon_sign) {
    if (!orc_la.ready || N < 2 || N > ORC_NMAX) return NULL;
    orc_ctx *c = calloc(1, sizeof(orc_ctx));
    c->prm = *p;
    if (c->prm.adjust_TriIneq) c->prm.TriIneq = N * 10; /* process_input.c:122-123 */
    c->N = N;
    c->pb = N - 1;
    size_t NN = (size_t)N * N;
    c->SL = malloc(NN * sizeof(double));
    memcpy(c->SL, SL, NN * sizeof(double));
    c->rng_mode = rng_mode;
    c->topk_mode = topk_mode;
    c->canon_sign = canon_sign;
    orc_glibc_seed(&c->g, 2020); /* bab_functions.c:82 */
    c->best_sol = calloc((size_t)N, sizeof(int));
    c->L = calloc(NN, sizeof(double));
    c->X = calloc(NN, sizeof(double));
    c->Q = calloc(NN, sizeof(double));
    c->y = calloc((size_t)N, sizeof(double));
    c->Z = calloc(NN, sizeof(double));
    c->tri = malloc((size_t)ORC_MAX_TRI * 4 * sizeof(int));
    c->pent = malloc((size_t)ORC_MAX_PENT * 6 * sizeof(int));
    c->hept = malloc((size_t)ORC_MAX_HEPT * 8 * sizeof(int));
    c->tri_y = calloc(ORC_MAX_TRI, sizeof(double));
    c->pent_y = calloc(ORC_MAX_PENT, sizeof(double));
    c->hept_y = calloc(ORC_MAX_HEPT, sizeof(double));
    size_t mall = (size_t)ORC_MAX_TRI + ORC_MAX_PENT + ORC_MAX_HEPT;
    c->t = calloc(mall, sizeof(double));
    c->s = calloc(mall, sizeof(double));
    c->u = calloc(mall, sizeof(double));
    int K = c->prm.TriIneq > 1 ? c->prm.TriIneq : 1;
    c->list_i = malloc((size_t)K * 4 * sizeof(int));
    c->list_v = malloc((size_t)K * sizeof(double));
    c->M = 0;
    return c;
}

void orc_destroy(orc_ctx *c) {
    if (!c) return;
    free(c->SL); free(c->best_sol); free(c->L); free(c->X); free(c->Q); free(c->y); free(c->Z);
    free(c->tri); free(c->pent); free(c->hept); free(c->tri_y); free(c->pent_y); free(c->hept_y);
    free(c->t); free(c->s); free(c->u); free(c->list_i); free(c->list_v);
    free(c);
}

void orc_set_lb(orc_ctx *c, double lb, const int *sol) {
    c->LB = lb;
    if (sol) memcpy(c->best_sol, sol, (size_t)c->pb * sizeof(int));
}
double orc_get_lb(orc_ctx *c, int *sol) {
    if (sol) memcpy(sol, c->best_sol, (size_t)c->pb * sizeof(int));
    return c->LB;
}
void orc_set_diff(orc_ctx *c, double diff) { c->diff = diff; }
double orc_get_diff(orc_ctx *c) { return c->diff; }
void orc_set_trials(orc_ctx *c, int pt, int ht) { c->prm.Pent_Trials = pt; c->prm.Hepta_Trials = ht; }
void orc_get_trials(orc_ctx *c, int *pt, int *ht) { *pt = c->prm.Pent_Trials; *ht = c->prm.Hepta_Trials; }
void orc_set_admm_trace(orc_ctx *c, double *buf, int cap) { c->trace = buf; c->trace_cap = cap; c->trace_len = 0; }

/* updateSolution, bab_functions.c:114-134 + Bab_LBUpd, heap.c:185-193 */
int orc_update_solution(orc_ctx *c, const int *x) {
    double v = orc_evaluate_solution(c->N, c->SL, x);
    if (v > c->LB) {
        c->LB = v;
        memcpy(c->best_sol, x, (size_t)c->pb * sizeof(int));
        return 1;
    }
    return 0;
}

/* mc_1opt, heuristic.c:100-201 (works in the {-1,1} model on the subproblem) */
static double mc_1opt(int *x, const double *L, int N) {
    double *Lx = calloc((size_t)N, sizeof(double)), *d = malloc((size_t)N * sizeof(double));
    double *delta = malloc((size_t)N * sizeof(double));
    int *I = malloc((size_t)N * sizeof(int));
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) Lx[i] += L[j + (size_t)i * N] * x[j];
    double cost = 0.0;
    for (int i = 0; i < N; ++i) {
        d[i] = L[i + (size_t)i * N];
        cost += x[i] * Lx[i];
        delta[i] = d[i] - x[i] * Lx[i];
    }
    double best = -ORC_BIG;
    int index = 0;
    for (int i = 0; i < N; ++i)
        if (delta[i] > best) { best = delta[i]; index = i; }
    while (best > 0.001) {
        int nI = 0;
        for (int j = 0; j < N; ++j)
            if (fabs(L[index + (size_t)N * j]) > 0.001) I[nI++] = j;
        if (x[index] > 0)
            for (int i = 0; i < nI; ++i) Lx[I[i]] -= 2 * L[index + (size_t)I[i] * N];
        else
            for (int i = 0; i < nI; ++i) Lx[I[i]] += 2 * L[index + (size_t)I[i] * N];
        x[index] *= -1;
        cost += 4 * best;
        for (int i = 0; i < N; ++i) delta[i] = d[i] - x[i] * Lx[i];
        best = -ORC_BIG;
        index = 0;
        for (int i = 0; i < N; ++i)
            if (delta[i] > best) { best = delta[i]; index = i; }
    }
    free(Lx); free(d); free(delta); free(I);
    return cost;
}

/* runHeuristic / GW_heuristic / update_best, heuristic.c:10-91, 209-223.
 * Uses the factor c->Z (n x M) of the last projection. */
double orc_run_heuristic(orc_ctx *c, const orc_node *node, int *x) {
    int N = c->n, M = c->M, num = c->N;
    int *temp_x = malloc((size_t)N * sizeof(int));
    int *sol = malloc((size_t)c->pb * sizeof(int));
    double *v = malloc(((size_t)M + 1) * sizeof(double));
    double best = -ORC_BIG;
    for (int count = 0; count < num; ++count) {
        orc_stream st;
        if (c->rng_mode == ORC_RNG_COUNTER) {
            st.key = orc_key2(orc_key2(c->node_key, 0x48455552ull + (uint64_t)c->heur_calls), (uint64_t)count);
            st.ctr = 0;
        }
        for (int i = 0; i < M; ++i) {
            if (c->rng_mode == ORC_RNG_GLIBC) v[i] = ((double)orc_glibc_next(&c->g) / (double)2147483647) - 0.5;
            else v[i] = (double)(orc_stream_next(&st) >> 11) * 0x1.0p-53 - 0.5;
        }
        for (int i = 0; i < N; ++i) {
            double sca = 0.0;
            for (int j = 0; j < M; ++j) sca += v[j] * c->Z[(size_t)j * N + i];
            temp_x[i] = sca < 0 ? -1 : 1;
        }
        mc_1opt(temp_x, c->L, N);
        int index = 0;
        for (int i = 0; i < c->pb; ++i) {
            if (node->xfixed[i]) sol[i] = node->sol[i];
            else sol[i] = (temp_x[index++] + 1) / 2;
        }
        double hv = orc_evaluate_solution(c->N, c->SL, sol);
        if (best < hv) {
            memcpy(x, sol, (size_t)c->pb * sizeof(int));
            best = hv;
        }
    }
    c->heur_calls++;
    free(temp_x); free(sol); free(v);
    return best;
}

static void store_fracsol(orc_ctx *c, orc_node *node) {
    int index = 0, n = c->n;
    for (int i = 0; i < c->pb; ++i) {
        if (node->xfixed[i]) node->fracsol[i] = (double)node->sol[i];
        else {
            node->fracsol[i] = 0.5 * (c->X[(n - 1) + (size_t)index * n] + 1.0);
            ++index;
        }
    }
}

static void heur_start(const orc_ctx *c, const orc_node *node, int *x) {
    for (int i = 0; i < c->pb; ++i) x[i] = node->xfixed[i] ? node->sol[i] : 0;
}

/* SDPbound, bounding.c:25-250 */
static double sdpbound(orc_ctx *c, orc_node *node, int rank, orc_node_stats *st) {
    const orc_params *P = &c->prm;
    int *x = malloc((size_t)c->pb * sizeof(int));
    double bound, gap, oldf;
    double viol3 = 0.0, viol5 = 0.0;
    int count = 0, nbit = 0, done = 0, giveup = 0, prune = 0, total_nbit = 0;
    int ta, ts, pa, ps, ha, hs;
    double sigma = P->sigma0, tol = P->tol0;
    double fixedvalue = orc_fixed_value(c->N, c->SL, node->xfixed, node->sol);
    c->ntri = c->npent = c->nhept = 0;
    c->sep_round = 0;
    c->heur_calls = 0;
    /* glibc mode keeps the reference's stale factor from the previous node for
     * the first heuristic call (heuristic.c:7-8 read the global Z/M); counter
     * mode starts every node from an empty factor, as the root does. */
    if (c->rng_mode == ORC_RNG_COUNTER) c->M = 0;
    int ipm_it = orc_ipm(c->L, c->n, c->X, c->y, c->Q, &c->f);
    double basic_bound = c->f + fixedvalue;
    store_fracsol(c, node);
    heur_start(c, node, x);
    orc_run_heuristic(c, node, x);
    orc_update_solution(c, x);
    bound = c->f + fixedvalue;
    if (bound < c->LB + 1.0) { prune = 1; goto END; }
    if (P->use_diff && rank != 0 && bound > c->LB + c->diff + 1.0) { giveup = 1; goto END; }
    viol3 = orc_update_tri(c, c->s, &ta, &ts);
    c->sep_round++;
    while (!done) {
        ++count;
        oldf = c->f;
        if (orc_admm(c, &sigma, tol, &nbit) != 0) { bound = NAN; goto END; }
        total_nbit += nbit;
        tol *= P->scaleTol;
        if (tol < P->minTol) tol = P->minTol;
        bound = c->f + fixedvalue;
        prune = (bound < c->LB + 1.0) ? 1 : 0;
        if (!prune) {
            heur_start(c, node, x);
            orc_run_heuristic(c, node, x);
            orc_update_solution(c, x);
            prune = (bound < c->LB + 1.0) ? 1 : 0;
        }
        gap = bound - c->LB;
        if (count == P->triag_iter + P->pent_iter + P->hept_iter)
            if (gap - 1.0 > (oldf - c->f) * (P->max_outer_iter - count)) giveup = 1;
        if (count == P->max_outer_iter)
            if (gap - 1.0 > (oldf - c->f) * P->extra_iter) giveup = 1;
        if (count == P->max_outer_iter + P->extra_iter) giveup = 1;
        if (rank != 0 && giveup && !prune) {
            c->prm.Pent_Trials += 60;
            c->prm.Hepta_Trials += 50;
        }
        if (!prune && !giveup) {
            int triag = c->ntri, penta = c->npent;
            viol3 = orc_update_tri(c, c->s, &ta, &ts);
            if (P->include_Pent && (count >= P->triag_iter || viol3 < 0.2))
                viol5 = orc_update_pent(c, c->s, &pa, &ps, triag);
            if (P->include_Hepta && ((count >= P->triag_iter + P->pent_iter) || (viol3 < 0.2 && (1 - viol5 < 0.4))))
                orc_update_hept(c, c->s, &ha, &hs, triag + penta);
            c->sep_round++;
        }
        done = prune || giveup || (nbit >= P->ADMM_itermax);
        store_fracsol(c, node);
        if (getenv("MCB_TRACE")) {
            uint64_t ht = 1, hp = 1, hh = 1;
            for (int q = 0; q < 4 * c->ntri; ++q) ht = orc_key2(ht, (uint64_t)c->tri[q]);
            for (int q = 0; q < 6 * c->npent; ++q) hp = orc_key2(hp, (uint64_t)c->pent[q]);
            for (int q = 0; q < 8 * c->nhept; ++q) hh = orc_key2(hh, (uint64_t)c->hept[q]);
            fprintf(stderr, "TRACE round %d nbit %d f %.15g cuts %d %d %d viol3 %.12g viol5 %.12g lb %.1f h %016llx %016llx %016llx\n",
                    count, nbit, c->f, c->ntri, c->npent, c->nhept, viol3, viol5, c->LB, (unsigned long long)ht,
                    (unsigned long long)hp, (unsigned long long)hh);
            if (getenv("MCB_TRACE_SA") && count == atoi(getenv("MCB_TRACE_SA")))
                for (int q = 0; q < c->npent; ++q)
                    fprintf(stderr, "PENT %d %d %d %d %d %d\n", c->pent[6 * q], c->pent[6 * q + 1], c->pent[6 * q + 2],
                            c->pent[6 * q + 3], c->pent[6 * q + 4], c->pent[6 * q + 5]);
        }
    }
    bound = c->f + fixedvalue;
    if (rank == 0) c->diff = basic_bound - bound;
END:
    if (st) {
        st->bound = bound;
        st->basic_bound = basic_bound;
        st->n_sub = c->n;
        st->outer_iters = count;
        st->admm_iters = total_nbit;
        st->ipm_iters = ipm_it;
        st->n_tri = c->ntri;
        st->n_pent = c->npent;
        st->n_hept = c->nhept;
        st->pruned = prune;
        st->gaveup = giveup;
    }
    free(x);
    return bound;
}

/* Evaluate, evaluate.c:12-21 */
double orc_evaluate(orc_ctx *c, orc_node *node, int rank, orc_node_stats *st) {
    double t0 = now_s();
    orc_set_work_n(c->N);
    orc_set_abstol(c->rng_mode == ORC_RNG_COUNTER ? 0.0 : 1e-8);
    c->n = orc_create_subproblem(c->N, c->SL, node->xfixed, node->sol, c->L);
    c->node_key = orc_node_key(node->xfixed, node->sol, c->pb);
    double b = sdpbound(c, node, rank, st);
    if (st) st->seconds = now_s() - t0;
    return b;
}

/* ------------------------------------------------------------------------- */
/* max-heap keyed on upper_bound, heap.c:27-133 (same comparison and sift order) */
typedef struct { orc_node **d; int used, size; } orc_heap;
static int cmp_nodes(const orc_node *a, const orc_node *b) { return a->upper_bound > b->upper_bound ? 1 : -1; }
static void hswap(orc_heap *h, int i, int j) { orc_node *t = h->d[i]; h->d[i] = h->d[j]; h->d[j] = t; }
static void heapify_down(orc_heap *h, int cur) {
    int child = 2 * cur + 1;
    if (child + 1 < h->used && cmp_nodes(h->d[child + 1], h->d[child]) > 0) child++;
    while (child < h->used && cmp_nodes(h->d[cur], h->d[child]) < 0) {
        hswap(h, cur, child);
        cur = child;
        child = 2 * cur + 1;
        if (child + 1 < h->used && cmp_nodes(h->d[child + 1], h->d[child]) > 0) child++;
    }
}
static void heapify_up(orc_heap *h, int cur) {
    int parent = (cur - 1) / 2;
    while (cur > 0 && cmp_nodes(h->d[parent], h->d[cur]) < 0) {
        hswap(h, cur, parent);
        cur = parent;
        parent = (cur - 1) / 2;
    }
}
static orc_node *heap_pop(orc_heap *h) {
    orc_node *n = h->d[0];
    h->d[0] = NULL;
    h->used--;
    hswap(h, 0, h->used);
    heapify_down(h, 0);
    return n;
}
static int heap_push(orc_heap *h, orc_node *n) {
    if (h->used == h->size) return -1;
    h->d[h->used++] = n;
    heapify_up(h, h->used - 1);
    return 0;
}

static orc_node *new_node(const orc_node *parent, int pb) {
    orc_node *n = malloc(sizeof(orc_node));
    for (int i = 0; i < pb; ++i) {
        if (!parent) { n->xfixed[i] = 0; n->sol[i] = 0; }
        else { n->xfixed[i] = parent->xfixed[i]; n->sol[i] = n->xfixed[i] ? parent->sol[i] : 0; }
    }
    n->level = parent ? parent->level + 1 : 0;
    n->upper_bound = 0.0;
    return n;
}

/* getBranchingVariable, bab_functions.c:389-423 */
static int branching_var(const orc_ctx *c, const orc_node *node) {
    int ic = -1;
    if (c->prm.branchingStrategy == 0) {
        double mx = -ORC_BIG;
        for (int i = 0; i < c->pb; ++i)
            if (!node->xfixed[i] && fabs(0.5 - node->fracsol[i]) > mx) { ic = i; mx = fabs(0.5 - node->fracsol[ic]); }
    } else {
        double mn = ORC_BIG;
        for (int i = 0; i < c->pb; ++i)
            if (!node->xfixed[i] && fabs(0.5 - node->fracsol[i]) < mn) { ic = i; mn = fabs(0.5 - node->fracsol[ic]); }
    }
    return ic;
}

/* Serial B&B.  The root is evaluated with rank 0 (Init_PQ) and branched at once
 * (main.c:126-158); every other node is evaluated as a worker (rank 1).  Children inherit the parent's bound as their heap key
 * (the reference inserts them with an uninitialised key, bab_functions.c:275-282). */
int orc_bab(orc_ctx *c, double *opt, int *sol, double *root_bound, int max_nodes,
            orc_node_stats *log, int log_cap, int *log_count) {
    orc_heap h;
    h.size = 1000000;
    h.used = 0;
    h.d = calloc((size_t)h.size, sizeof(orc_node *));
    int nodes = 1, lc = 0, evaluated = 0;
    orc_node *root = new_node(NULL, c->pb);
    orc_node_stats st;
    double rb = orc_evaluate(c, root, 0, &st);
    evaluated++;
    if (log && lc < log_cap) log[lc++] = st;
    if (root_bound) *root_bound = rb;
    root->upper_bound = rb;
    if (c->LB + 1.0 < root->upper_bound && !c->prm.root) {
        /* the master branches the root directly (main.c:126-158) */
        int ic = branching_var(c, root);
        for (int xic = 0; xic <= 1 && ic >= 0; ++xic) {
            orc_node *ch = new_node(root, c->pb);
            ch->xfixed[ic] = 1;
            ch->sol[ic] = xic;
            ch->upper_bound = root->upper_bound;
            heap_push(&h, ch);
            nodes += 1;
        }
    }
    free(root);
    while (h.used > 0) {
        if (max_nodes > 0 && evaluated >= max_nodes) { nodes = -nodes; break; }
        orc_node *node = heap_pop(&h);
        node->upper_bound = orc_evaluate(c, node, 1, &st);
        evaluated++;
        if (log && lc < log_cap) log[lc++] = st;
        if (c->LB + 1.0 < node->upper_bound) {
            int ic = branching_var(c, node);
            if (ic >= 0) {
                for (int xic = 0; xic <= 1; ++xic) {
                    orc_node *ch = new_node(node, c->pb);
                    ch->xfixed[ic] = 1;
                    ch->sol[ic] = xic;
                    ch->upper_bound = node->upper_bound;
                    if (heap_push(&h, ch) != 0) { free(ch); nodes = -nodes; goto done; }
                }
                nodes += 2;
            }
        }
        free(node);
    }
done:
    while (h.used > 0) free(heap_pop(&h));
    free(h.d);
    if (opt) *opt = c->LB;
    if (sol) memcpy(sol, c->best_sol, (size_t)c->pb * sizeof(int));
    if (log_count) *log_count = lc;
    return nodes;
}

/* next value of the context's glibc stream (test helper: stream-position checks) */
int orc_debug_next_rand(orc_ctx *c) { return orc_glibc_next(&c->g); }
/* number of positive eigenvalues of the last projection */
int orc_debug_last_M(orc_ctx *c) { return c->M; }
/* copy out the current cut lists (test helper) */
void orc_debug_cuts(orc_ctx *c, int *nt, int *np, int *nh, int *tri, int *pent, int *hept) {
    *nt = c->ntri; *np = c->npent; *nh = c->nhept;
    if (tri) memcpy(tri, c->tri, (size_t)c->ntri * 4 * sizeof(int));
    if (pent) memcpy(pent, c->pent, (size_t)c->npent * 6 * sizeof(int));
    if (hept) memcpy(hept, c->hept, (size_t)c->nhept * 8 * sizeof(int));
}
/* copy out the current primal iterate (test helper) */
int orc_debug_X(orc_ctx *c, double *X) { memcpy(X, c->X, (size_t)c->n * c->n * sizeof(double)); return c->n; }
/* number of values drawn from the context's glibc stream since seeding (test helper) */
int orc_debug_rand_pos(orc_ctx *c) { return c->g.pos - 344; }
