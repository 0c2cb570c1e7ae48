/* Serial driver for the reference built as a CPU oracle (oracle/_ref).  It takes
 * the place of the MPI main (main.c): rank 0 reads the instance and evaluates
 * the root (Init_PQ, bab_functions.c:39-69), then the same process runs the
 * worker step of bab_functions.c:226-334 without messages: pop, Evaluate with
 * rank 1, branch.  Children get the parent's bound as their heap key (the
 * reference inserts them with an uninitialised key).
 *
 * usage: madam_ref <graph> <params> [max_nodes]
 * prints one "node <k> level <l> n <n> bound <b> lb <lb>" line per evaluated
 * node and the reference's final block (bab_functions.c:353-373). */
#include <stdio.h>
#include <stdlib.h>

#include "admm.h"

extern Heap *heap;
extern Parameters params;
extern Problem *SP, *PP;
extern double root_bound;
extern FILE *output;
extern double TIME;
extern BabNode *BabRoot;

int num_workers_used = 0; /* defined by main.c in the reference */

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s graph params [max_nodes]\n", argv[0]);
        return 2;
    }
    long max_nodes = argc > 3 ? atol(argv[3]) : 0;
    TIME = MPI_Wtime();
    heap = Init_Heap(1000000);
    if (Bab_Init(3, argv, 0)) return 1;
    int over = Init_PQ();
    long evaluated = 1;
    printf("node %ld level %d n %d bound %.12f lb %.1f\n", evaluated, 0, PP->n, root_bound, Bab_LBGet());
    if (over != -1 && !params.root) {
        /* the master branches the root itself and hands both children out (main.c:126-158) */
        BabNode *root = Bab_PQPop();
        int ic0 = getBranchingVariable(root);
        for (int xic = 0; xic <= 1; ++xic) {
            BabNode *child = newNode(root);
            child->xfixed[ic0] = 1;
            child->sol.X[ic0] = xic;
            child->upper_bound = root->upper_bound;
            Bab_incEvalNodes();
            Bab_PQInsert(child);
        }
        free(root);
        while (!isPQEmpty()) {
            if (max_nodes > 0 && evaluated >= max_nodes) break;
            BabNode *node = Bab_PQPop();
            node->upper_bound = Evaluate(node, SP, PP, 1);
            ++evaluated;
            printf("node %ld level %d n %d bound %.12f lb %.1f\n", evaluated, node->level, PP->n,
                   node->upper_bound, Bab_LBGet());
            if (Bab_LBGet() + 1.0 < node->upper_bound) {
                int ic = getBranchingVariable(node);
                for (int xic = 0; xic <= 1; ++xic) {
                    BabNode *child = newNode(node);
                    child->xfixed[ic] = 1;
                    child->sol.X[ic] = xic;
                    child->upper_bound = node->upper_bound;
                    Bab_PQInsert(child);
                }
                Bab_incEvalNodes();
                Bab_incEvalNodes();
            }
            free(node);
        }
    }
    printFinalOutput(stdout, Bab_numEvalNodes());
    printFinalOutput(output, Bab_numEvalNodes());
    fclose(output);
    Bab_End();
    return 0;
}
