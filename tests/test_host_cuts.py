"""The cut system the library assembles on the host for every ADMM call
(madam_gb300/csrc/host_cuts.h: packed cut encoding, B^T edge incidence, and the
CSR of B B^T + I that the device solver uses in place of CHOLMOD's factor,
admm.c:117-487), checked on the CPU against the oracle's restatement of the
reference's op_B / op_Bt (operators.c:62-150, 171-513).  A host-only harness
(tests/host_cuts_check.cu, no kernel launches) is compiled with nvcc."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
NVCC = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else shutil.which("nvcc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not NVCC:
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("hc") / "host_cuts_check")
    r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-o", exe,
                        os.path.join(HERE, "host_cuts_check.cu")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _cuts(rng, n, nt, np_, nh):
    tri = []
    for _ in range(nt):
        i, j, k = sorted(rng.choice(n, 3, replace=False), reverse=True)
        tri.append([int(i), int(j), int(k), int(rng.integers(1, 5))])
    pent = [[int(rng.integers(1, 4))] + [int(v) for v in rng.choice(n, 5, replace=False)] for _ in range(np_)]
    hept = [[int(rng.integers(1, 5))] + [int(v) for v in rng.choice(n, 7, replace=False)] for _ in range(nh)]
    if tri:
        tri.append(list(tri[0]))  # a repeated cut: its edges are shared with itself
    return tri, pent, hept


def _run(exe, n, tri, pent, hept, X, t):
    parts = [str(n), str(len(tri))] + [str(v) for c in tri for v in c]
    parts += [str(len(pent))] + [str(v) for c in pent for v in c]
    parts += [str(len(hept))] + [str(v) for c in hept for v in c]
    parts += ["%.17g" % v for v in X.ravel(order="F")] + ["%.17g" % v for v in t]
    r = subprocess.run([exe], input=" ".join(parts), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    v = np.array(r.stdout.split(), dtype=np.float64)
    m = len(t)
    return v[:m], v[m:m + n * n].reshape(n, n, order="F"), v[m + n * n:].reshape(m, m)


@pytest.mark.parametrize("seed,n,nt,np_,nh", [(1, 12, 30, 0, 0), (2, 16, 20, 8, 0), (3, 20, 25, 6, 5),
                                               (4, 9, 40, 10, 6), (5, 30, 0, 0, 9)])
def test_cut_system_against_the_oracle(orc, harness, seed, n, nt, np_, nh):
    rng = np.random.default_rng(seed)
    tri, pent, hept = _cuts(rng, n, nt, np_, nh)
    m = len(tri) + len(pent) + len(hept)
    A = rng.standard_normal((n, n))
    X = A + A.T
    t = rng.standard_normal(m)
    y, Z, Gm = _run(harness, n, tri, pent, hept, X, t)
    # B(X): the packed encoding reads the reference's signs
    yo = orc.op_B(X, tri=tri, pent=pent, hept=hept)
    assert np.allclose(y, yo, rtol=0, atol=1e-13 * np.abs(X).max()), np.abs(y - yo).max()
    # B^T(t) through the edge incidence is op_Bt's scatter (both triangles)
    Zo = orc.op_Bt(np.zeros((n, n)), t, tri=tri, pent=pent, hept=hept)
    assert np.allclose(Z, Zo, rtol=0, atol=1e-14 * max(1.0, np.abs(t).max())), np.abs(Z - Zo).max()
    # B B^T + I: row c of B is the full symmetric matrix op_Bt(0, e_c)
    rows = np.stack([orc.op_Bt(np.zeros((n, n)), np.eye(m)[c], tri=tri, pent=pent, hept=hept).ravel()
                     for c in range(m)])
    Go = rows @ rows.T + np.eye(m)
    assert np.array_equal(Gm, Gm.T)
    assert np.allclose(Gm, Go, rtol=0, atol=1e-14), np.abs(Gm - Go).max()
    # and it is what makes the solve well posed: symmetric positive definite, eigenvalues >= 1
    assert np.linalg.eigvalsh(Gm).min() >= 1.0 - 1e-12
