// noalloc.cu -- the PSD projection for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc while they bound nodes:
// a host process whose device memory is fully handed out by its own pool (a
// solver embedded in a larger GPU application that owns every byte it
// reserved), a caller that runs inside a memory budget enforced by its
// scheduler, or one that must not hit the allocator's implicit device
// synchronisation between launches.  mcb_project_psd_noalloc gives them the
// projection of operators.c:521-619 on buffers they already own: inputs and
// outputs are the caller's device pointers, and the only scratch -- the
// tridiagonalisation workspace, the inverse-iteration workspace and the
// tridiagonal vectors -- is the file-scope device array below, sized for
// n <= kNoAllocMaxN.
//
// The array lives as long as the library is loaded, once per GPU that loads it
// (about 5.3 MB).  Every call shares it and it keeps the last call's contents;
// everything a call reads from it is written first by the same call, so
// nothing needs clearing between calls.  Calls whose work overlaps on the GPU
// (different streams, or different host threads on one device) race on it and
// must not be issued concurrently.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mcbound.h"
#include "kernels.h"
#include "mcb_dev.cuh"

namespace {

constexpr int kNoAllocMaxN = MCB_NOALLOC_MAX_N;
constexpr size_t kScratchDoubles = (size_t)kNoAllocMaxN * kNoAllocMaxN   // tridiagonal reduction (A)
                                   + mcb::eig_dwork_doubles_max(kNoAllocMaxN)  // inverse iteration (6 n per thread)
                                   + 3 * (size_t)kNoAllocMaxN                  // d, e, tau
                                   + mcb::kAcc;                                // per-slot accumulators

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];
static __device__ __align__(256) mcb::Slot g_noalloc_slot;

struct DeviceAddrs {
    double *scratch = nullptr;
    mcb::Slot *slot = nullptr;
    bool ready = false;
};
constexpr int kMaxDevices = 64;
DeviceAddrs g_addrs[kMaxDevices];
std::mutex g_setup_mu;

// Device addresses of the scratch symbols on the current device: looked up once
// per device, with that device current (the names are host-side stand-ins).
int device_addrs(DeviceAddrs **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return MCB_ERR_NODEV;
    if (dev >= kMaxDevices) return MCB_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceAddrs &a = g_addrs[dev];
    if (!a.ready) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MCB_ERR_CUDA;
        a.scratch = (double *)p;
        p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_slot) != cudaSuccess || !p) return MCB_ERR_CUDA;
        a.slot = (mcb::Slot *)p;
        a.ready = true;
    }
    *out = &a;
    return MCB_OK;
}

}  // namespace

extern "C" int mcb_project_psd_noalloc(int n, const double *W, double *Xp, double *Q, double *Z, double *evals,
                                       int *M, void *stream) {
    if (n < 1 || n > kNoAllocMaxN || !W || !Xp || !Q || !Z || !evals || !M) return MCB_ERR_ARG;
    DeviceAddrs *a = nullptr;
    if (int rc = device_addrs(&a)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nn = (size_t)n * n;
    mcb::Slot h{};
    h.n = n;
    h.active = 1;
    h.W = const_cast<double *>(W);  // read only
    h.X = Xp;
    h.Q = Q;
    h.V = Z;
    h.ev = evals;
    h.A = a->scratch;
    h.dwork = a->scratch + nn;
    double *vec = h.dwork + mcb::eig_dwork_doubles_max(n);
    h.d = vec;
    h.e = vec + n;
    h.tau = vec + 2 * n;
    h.acc = vec + 3 * n;
    if (cudaMemcpyAsync(a->slot, &h, sizeof(mcb::Slot), cudaMemcpyHostToDevice, st) != cudaSuccess) return MCB_ERR_CUDA;
    // Q's strictly upper triangle is 0, as in the reference's full-array daxpy (operators.c:616-617)
    if (cudaMemsetAsync(Q, 0, nn * sizeof(double), st) != cudaSuccess) return MCB_ERR_CUDA;
    mcb::launch_sym_copy(a->slot, 1, n, 0, 0, st);
    mcb::launch_tridiag(a->slot, 1, n, 0, st);
    mcb::launch_bisect(a->slot, 1, n, 1e-8, 0, 0, st);
    mcb::launch_invit(a->slot, 1, n, 0, st);
    mcb::launch_backtrans(a->slot, 1, n, 0, st);
    mcb::launch_canon_scale(a->slot, 1, n, 0, st);
    mcb::launch_syrk_post(a->slot, 1, n, 0, nullptr, st);
    if (cudaGetLastError() != cudaSuccess) return MCB_ERR_CUDA;
    mcb::Slot back{};
    if (cudaMemcpyAsync(&back, a->slot, sizeof(mcb::Slot), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MCB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MCB_ERR_CUDA;
    *M = back.M;
    return back.status ? back.status : MCB_OK;
}
