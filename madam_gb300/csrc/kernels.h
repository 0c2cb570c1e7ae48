// kernels.h -- host-side launchers of the sm_103a kernels (all take the device
// Slot array and launch on the given stream).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace mcb {
struct Slot;

// k_eig.cu (gate = 1: skip slots whose ADMM has stopped)
void launch_sym_copy(Slot *d, int ns, int nmax, int src, int gate, cudaStream_t st);
void launch_tridiag(Slot *d, int ns, int nmax, int gate, cudaStream_t st);
void launch_bisect(Slot *d, int ns, int nmax, double vl, int largest_only, int gate, cudaStream_t st);
void launch_invit(Slot *d, int ns, int nmax, int gate, cudaStream_t st);
void launch_backtrans(Slot *d, int ns, int nmax, int gate, cudaStream_t st);
void launch_canon_scale(Slot *d, int ns, int nmax, int gate, cudaStream_t st);
int syrk_tiles(int nmax);
void launch_syrk_post(Slot *d, int ns, int nmax, int mode, double *partials, cudaStream_t st);
size_t eig_dwork_doubles(int nmax);

// k_ipm.cu
void launch_ipm_init(Slot *d, int ns, cudaStream_t st);
void launch_ipm_iteration(Slot *d, int ns, int nmax, cudaStream_t st);

// k_admm.cu
void launch_admm_rhs(Slot *d, int ns, int nmax, int mmax, cudaStream_t st);
// k_cg's shared-memory limit (once per device, before any launch or capture); 0 on success
int cg_prepare();
void launch_cg(Slot *d, int ns, int mmax, int maxit, double rtol, cudaStream_t st);
// the FP32 copy of every active slot's (B B^T + I) values (after an upload of the system)
void launch_cg_values(Slot *d, int ns, cudaStream_t st);
void launch_admm_su(Slot *d, int ns, int mmax, cudaStream_t st);
void launch_build_W(Slot *d, int ns, int nmax, int emax, int mat, cudaStream_t st);
void launch_op_B(Slot *d, int m, const double *X, double *y, cudaStream_t st);
void launch_op_Bt(Slot *d, int ne, double *X, const double *t, cudaStream_t st);
void launch_admm_bx(Slot *d, int ns, int mmax, cudaStream_t st);
void launch_admm_finish(Slot *d, int ns, double scaleSigma, int itermax, cudaStream_t st);
void launch_safe_norm(Slot *d, int ns, cudaStream_t st);
void launch_safe_finish(Slot *d, int ns, cudaStream_t st);

// k_sep.cu
size_t trisel_bytes();
size_t sajob_bytes();
void launch_tri_separation(Slot *d, int ns, int nmax, void *sel, double thr, int K, unsigned int *out,
                           double *outv, unsigned int *bnd, double *bndv, int cap_out, int cap_bnd,
                           cudaStream_t st);
void tri_sel_readback(const void *sel_host, int slot, double *maxviol, int *take_all, int *need2, int *n_out,
                      int *n_bnd);
void launch_sa(Slot *d, void *jobs, int njobs, int *perm_scratch, int nmax, int *out_ineq, double *out_val,
               int total_runs, cudaStream_t st);
void sajob_fill(void *jobs_host, int idx, int slot, int k, int runs, int ntypes, uint64_t key, int out_off);

// k_sub.cu
// createSubproblem (evaluate.c:39-116) for every active slot, from the slot's own
// problem (Slot::SL, Slot::N) and its node lists
void launch_subproblem(Slot *d, int ns, const int *d_lists, int list_stride, double *d_fixed, cudaStream_t st);
}  // namespace mcb
