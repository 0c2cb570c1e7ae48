"""The allocation-free projection entry point (for callers that may not call
cudaMalloc) against the allocating one, through the C ABI, on two calls in a row
that share the library's static scratch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym(n, seed, sign=0.0):
    A = np.random.default_rng(seed).standard_normal((n, n))
    if n == 1:  # a 1 x 1 matrix of the given sign
        return np.array([[sign * (1.0 + abs(A[0, 0]))]])
    return 1.5 * (A + A.T)


def test_noalloc_projection_matches_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    # calls in a row that share the scratch: its largest size (n = 512 fills it),
    # then smaller ones, so stale scratch from an earlier call would show, down to
    # the 1 x 1 matrices (one positive eigenvalue, then none)
    for n, seed, sign in ((512, 10, 0.0), (300, 11, 0.0), (97, 12, 0.0), (1, 13, 1.0), (1, 14, -1.0)):
        W = _sym(n, seed, sign)
        Xp, Q, Z, ev = gpu_lib.project(W)
        dW = torch.tensor(W.ravel(order="F"), dtype=torch.float64, device="cuda")
        dXp = torch.full((n * n,), np.nan, dtype=torch.float64, device="cuda")
        dQ = torch.full((n * n,), np.nan, dtype=torch.float64, device="cuda")
        dZ = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        dev = torch.zeros(n, dtype=torch.float64, device="cuda")
        M = gpu_lib.project_noalloc(n, dW.data_ptr(), dXp.data_ptr(), dQ.data_ptr(), dZ.data_ptr(), dev.data_ptr(),
                                    stream=stream)
        torch.cuda.synchronize()
        assert M == len(ev)
        if n == 1:
            assert M == (1 if sign > 0 else 0)
        scale = max(1.0, np.abs(W).max())
        Xn = dXp.cpu().numpy().reshape(n, n, order="F")
        Qn = dQ.cpu().numpy().reshape(n, n, order="F")
        Zn = dZ.cpu().numpy().reshape(n, n, order="F")[:, :M]
        assert np.abs(Xn - Xp).max() <= 1e-10 * scale * n
        assert np.abs(np.tril(Qn) - np.tril(Q)).max() <= 1e-10 * scale * n
        assert np.all(np.triu(Qn, 1) == 0.0)
        if M > 0:  # no factor and no eigenvalues to compare when nothing is positive
            assert np.abs(Zn - Z).max() <= 1e-8 * scale
            assert np.abs(dev.cpu().numpy()[:M] - ev).max() <= 1e-11 * scale


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    n = 513
    buf = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    vec = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(gpu_lib.MCBError):
        gpu_lib.project_noalloc(n, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), vec.data_ptr())
