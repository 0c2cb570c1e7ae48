/* mcb_madam_shim.c -- MADAM's Evaluate / SDPbound (admm.h:234,246) on top of
 * libmcbound, for linking the reference's own branch-and-bound driver
 * (bab_functions.c, heap.c, main.c) against the GPU bound.
 *
 * Build into the reference in place of evaluate.c, bounding.c, admm.c,
 * operators.c, cutting_planes.c, ipm_mc_pk.c and qap_simulated_annealing.c:
 *   cc -I<reference> -I<repo>/include -c mcb_madam_shim.c
 *   link with -L<repo>/madam_gb300 -lmcbound -lcudart -lcublas
 *
 * mcb_params and mcb_bab_node have the layouts of Parameters and BabNode, so
 * the reference's objects are passed as they are.  The context is created on
 * the first call from SP (the reference keeps one problem per process). */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "admm.h"
#include "mcbound.h"

/* The casts below are valid only while the layouts agree: checked field by field
 * at compile time, for Parameters through the reference's own field list
 * (PARAM_FIELDS, admm.h:58-81) and for BabNode (admm.h:147-155). */
_Static_assert(sizeof(mcb_params) == sizeof(Parameters), "mcb_params differs from Parameters");
#define P(type, name, format, def_value)                                                       \
    _Static_assert(offsetof(mcb_params, name) == offsetof(Parameters, name), "Parameters." #name); \
    _Static_assert(sizeof(((mcb_params *)0)->name) == sizeof(type), "Parameters." #name " type");
PARAM_FIELDS
#undef P
_Static_assert(sizeof(mcb_bab_node) == sizeof(BabNode), "mcb_bab_node differs from BabNode");
_Static_assert(offsetof(mcb_bab_node, xfixed) == offsetof(BabNode, xfixed), "BabNode.xfixed");
_Static_assert(offsetof(mcb_bab_node, sol) == offsetof(BabNode, sol.X), "BabNode.sol");
_Static_assert(offsetof(mcb_bab_node, fracsol) == offsetof(BabNode, fracsol), "BabNode.fracsol");
_Static_assert(offsetof(mcb_bab_node, level) == offsetof(BabNode, level), "BabNode.level");
_Static_assert(offsetof(mcb_bab_node, upper_bound) == offsetof(BabNode, upper_bound), "BabNode.upper_bound");
_Static_assert(MCB_NMAX == NMAX, "NMAX");

/* The one routine of operators.c that the kept files call: readData builds the
 * Laplacian with it (process_input.c:265-268).  X = diagonal matrix of y, n x n,
 * column-major, all off-diagonal entries zero (operators.c:44-54). */
void Diag(double *X, const double *y, int n) {
    memset(X, 0, (size_t)n * n * sizeof(double));
    for (int i = 0; i < n; ++i) X[i + (size_t)i * n] = y[i];
}

extern Parameters params;
extern double diff;

static mcb_ctx *g_ctx;

static mcb_ctx *ctx_for(const Problem *SP) {
    if (!g_ctx) {
        int st = 0;
        g_ctx = mcb_create((const mcb_params *)&params, SP->n, SP->L, 1, MCB_PROJ_FP64, NULL, &st);
        if (!g_ctx) {
            fprintf(stderr, "mcb_create: %s\n", mcb_strerror(st));
            exit(1);
        }
    }
    return g_ctx;
}

double SDPbound(BabNode *node, Problem *SP, Problem *PP, int rank) {
    (void)PP; /* the subproblem is built on the device */
    mcb_ctx *c = ctx_for(SP);
    double bound = 0.0;
    int sol[NMAX];
    mcb_set_lb(c, Bab_LBGet(), NULL);
    mcb_set_diff(c, diff);
    mcb_set_trials(c, params.Pent_Trials, params.Hepta_Trials);
    int rc = mcb_evaluate(c, (mcb_bab_node *)node, rank, &bound, NULL);
    if (rc != MCB_OK) {
        fprintf(stderr, "mcb_evaluate: %s (%s)\n", mcb_strerror(rc), mcb_last_error(c));
        exit(1);
    }
    if (mcb_get_lb(c, sol) > Bab_LBGet()) updateSolution(sol); /* heap.c:185-193 */
    diff = mcb_get_diff(c);
    mcb_get_trials(c, &params.Pent_Trials, &params.Hepta_Trials);
    return bound;
}

double Evaluate(BabNode *node, Problem *SP, Problem *PP, int rank) { return SDPbound(node, SP, PP, rank); }
