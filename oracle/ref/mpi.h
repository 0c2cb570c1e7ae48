/* Single-rank stand-in for the MPI calls the reference's bound path and
 * driver files compile against (bab_functions.c, process_input.c, admm.c).
 * Used only to build the reference itself as a CPU oracle (oracle/_ref).
 * Rank 0 is the only process: broadcasts are no-ops, point-to-point calls are
 * never reached by the serial driver, MPI_Wtime reads the monotonic clock. */
#ifndef MCB_REF_MPI_STUB_H
#define MCB_REF_MPI_STUB_H
#include <stddef.h>
#include <stdlib.h>
#include <time.h>

typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

static inline int MPI_Init(int *a, char ***b) { (void)a; (void)b; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
    (void)b; (void)n; (void)t; (void)root; (void)c; return 0;
}
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; abort(); return 0;
}
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) {
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; abort(); return 0;
}
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); return 0; }
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *d, const MPI_Datatype *t,
                                         MPI_Datatype *nt) {
    (void)n; (void)bl; (void)d; (void)t; *nt = 0; return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
#endif
