"""The SVD adjoint formula the CUDA kernel implements, checked on the CPU.

`adjoint_np` restates, in numpy, exactly what k_svd_adjoint computes (the same J, K, N,
P, Q products, the same gap-safe F). It is pinned here against torch.linalg.svd's own
backward (double precision, CPU) and against central finite differences (h = 1e-6),
for the loss sum_i w_i s_i + <G_U, U_k> + <G_V, V_k> with sign-fixed singular vectors.
The GPU tests compare the kernel against this restatement and against the same checks.
"""
import numpy as np
import pytest


def adjoint_np(U, S, V, dS, dU, dV, gap=0.0):
    """dA for one matrix: U (m, n), S (n), V (n, n), dU (m, k), dV (n, k)."""
    m, n = U.shape
    k = dU.shape[1]
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    J[:, :k] = U.T @ dU
    K[:, :k] = V.T @ dV
    si, sj = S[:, None], S[None, :]
    d = (sj - si) * (sj + si)
    mx = np.maximum(si, sj)
    den = d * d + (gap * mx * mx) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        F = np.where(den != 0, d / den, 0.0)
    np.fill_diagonal(F, 0.0)
    inv = np.where(S != 0, 1.0 / np.where(S != 0, S, 1.0), 0.0)
    N = np.diag(dS) + F * ((J - J.T) * sj + si * (K - K.T)) - J * inv[None, :]
    P = N @ V.T
    Q = inv[:k, None] * V[:, :k].T
    return U @ P + dU @ Q


def sign_fix(U, V):
    piv = np.argmax(np.abs(V), axis=0)
    sg = np.sign(V[piv, np.arange(V.shape[1])])
    sg[sg == 0] = 1
    return U * sg, V * sg


def svd_fixed(A):
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    U, V = sign_fix(U, Vt.T)
    return U, S, V


def loss(A, w, GU, GV, k):
    U, S, V = svd_fixed(A)
    return float(w @ S + np.sum(GU * U[:, :k]) + np.sum(GV * V[:, :k]))


@pytest.mark.parametrize("m,n,k", [(12, 8, 3), (16, 16, 4), (20, 6, 6)])
def test_formula_vs_finite_differences(m, n, k):
    from vecjac_gb300.autodiff import spaced_sigma_matrices
    A, _ = spaced_sigma_matrices(1, m, n, seed=m * n + k)
    A = A[0]
    rng = np.random.default_rng(3)
    w, GU, GV = rng.standard_normal(n), rng.standard_normal((m, k)), rng.standard_normal((n, k))
    U, S, V = svd_fixed(A)
    dA = adjoint_np(U, S, V, w, GU, GV)
    h = 1e-6
    for _ in range(4):
        E = rng.standard_normal((m, n))
        fd = (loss(A + h * E, w, GU, GV, k) - loss(A - h * E, w, GU, GV, k)) / (2 * h)
        an = float(np.sum(dA * E))
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


@pytest.mark.parametrize("m,n,k", [(12, 8, 3), (32, 16, 16)])
def test_formula_vs_torch(m, n, k):
    torch = pytest.importorskip("torch")
    from vecjac_gb300.autodiff import spaced_sigma_matrices
    A, _ = spaced_sigma_matrices(1, m, n, seed=7 + m)
    A = A[0]
    rng = np.random.default_rng(5)
    w, GU, GV = rng.standard_normal(n), rng.standard_normal((m, k)), rng.standard_normal((n, k))
    At = torch.tensor(A, requires_grad=True)
    Ut, St, Vht = torch.linalg.svd(At, full_matrices=False)
    Vt = Vht.mT
    with torch.no_grad():
        piv = torch.argmax(Vt.abs(), dim=0)
        sg = torch.sign(Vt[piv, torch.arange(n)])
    Ut, Vt = Ut * sg, Vt * sg
    L = (torch.tensor(w) * St).sum() + (torch.tensor(GU) * Ut[:, :k]).sum() + (torch.tensor(GV) * Vt[:, :k]).sum()
    L.backward()
    U, S, V = svd_fixed(A)
    dA = adjoint_np(U, S, V, w, GU, GV)
    assert np.max(np.abs(dA - At.grad.numpy())) <= 1e-9 * np.max(np.abs(dA))


def test_gap_broadening_is_bounded():
    # two equal singular values: the exact F is infinite; broadening keeps dA finite
    rng = np.random.default_rng(9)
    q1, _ = np.linalg.qr(rng.standard_normal((10, 6)))
    q2, _ = np.linalg.qr(rng.standard_normal((6, 6)))
    S = np.array([3.0, 2.0, 2.0, 1.0, 0.5, 0.25])
    dA = adjoint_np(q1, S, q2, np.ones(6), rng.standard_normal((10, 2)), rng.standard_normal((6, 2)), gap=1e-3)
    assert np.all(np.isfinite(dA))
    dA0 = adjoint_np(q1, S, q2, np.ones(6), np.zeros((10, 2)), np.zeros((6, 2)), gap=0.0)
    # with no vector cotangents the exact adjoint is U diag(dS) V^T
    assert np.allclose(dA0, (q1 * np.ones(6)) @ q2.T, atol=1e-14)
