"""The SVD adjoint kernel (vj_?svd_adjoint_batch_dev) and the differentiable batched SVD.

Checks, for the loss sum_i w_i s_i + <G_U, U_k> + <G_V, V_k>:
  * kernel vs the numpy restatement of the same formula, on the same U, S, V
    (FP64: 1e-12 relative to max |dA|; FP32: 2e-4, the FP32 rounding of the products
    amplified by 1/(relative gap) <= 1e3);
  * FP64 path vs central finite differences of the FP64 batched SVD (h = 1e-6,
    directional derivatives, 1e-5 relative: the forward's vectors carry n eps / gap
    rounding error, which the difference quotient divides by 2h);
  * FP32 path vs torch.linalg.svd's gradient in FP64 (5e-3 relative to max |dA|: the
    FP32 forward's vectors carry ~n eps_32 / relative-gap error).
"""
import numpy as np
import pytest

from test_adjoint_cpu import adjoint_np

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ad():
    from vecjac_gb300 import autodiff, build
    build.build()
    return autodiff


def problem(count, m, n, k, seed):
    from vecjac_gb300.autodiff import spaced_sigma_matrices
    A, _ = spaced_sigma_matrices(count, m, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    return A, rng.standard_normal((count, n)), rng.standard_normal((count, m, k)), rng.standard_normal((count, n, k))


def grad_ours(ad, A, w, GU, GV, k, dtype):
    import torch
    At = torch.tensor(A, dtype=dtype, device="cuda", requires_grad=True)
    S, Uk, Vk = ad.svd_k(At, k)
    t = lambda x: torch.tensor(x, dtype=dtype, device="cuda")
    L = (t(w) * S).sum() + (t(GU) * Uk).sum() + (t(GV) * Vk).sum()
    L.backward()
    return At.grad.double().cpu().numpy(), S.detach().double().cpu().numpy()


@pytest.mark.parametrize("dtype_name,m,n,k", [("float64", 32, 16, 4), ("float64", 64, 32, 32), ("float32", 128, 64, 16),
                                              ("float32", 64, 64, 8)])
def test_kernel_vs_restatement(ad, dtype_name, m, n, k):
    import torch
    dtype = getattr(torch, dtype_name)
    A, w, GU, GV = problem(6, m, n, k, seed=m + n + k)
    t = lambda x: torch.tensor(x, dtype=dtype, device="cuda")
    rng = np.random.default_rng(1)
    U = np.stack([np.linalg.qr(rng.standard_normal((m, n)))[0] for _ in range(6)])
    V = np.stack([np.linalg.qr(rng.standard_normal((n, n)))[0] for _ in range(6)])
    from vecjac_gb300.autodiff import spaced_sigma_matrices
    S = np.stack([spaced_sigma_matrices(1, n, n, seed=b)[1][0] for b in range(6)])
    U, V = U.astype(dtype_name).astype(np.float64), V.astype(dtype_name).astype(np.float64)
    S = S.astype(dtype_name).astype(np.float64)
    dA = ad.adjoint(t(U), t(S), t(V), t(w), t(GU), t(GV)).double().cpu().numpy()
    tol = 1e-12 if dtype_name == "float64" else 2e-4
    for b in range(6):
        ref = adjoint_np(U[b], S[b], V[b], w[b], GU[b], GV[b])
        assert np.max(np.abs(dA[b] - ref)) <= tol * np.max(np.abs(ref)), b


def test_fp64_vs_finite_differences(ad):
    import torch
    m, n, k, count = 32, 16, 4, 4
    A, w, GU, GV = problem(count, m, n, k, seed=21)
    g, _ = grad_ours(ad, A, w, GU, GV, k, torch.float64)

    def losses(X):
        with torch.no_grad():
            S, Uk, Vk = ad.svd_k(torch.tensor(X, dtype=torch.float64, device="cuda"), k)
        S, Uk, Vk = S.cpu().numpy(), Uk.cpu().numpy(), Vk.cpu().numpy()
        return np.einsum("bi,bi->b", w, S) + np.einsum("bij,bij->b", GU, Uk) + np.einsum("bij,bij->b", GV, Vk)

    rng = np.random.default_rng(4)
    h = 1e-6
    for _ in range(3):
        E = rng.standard_normal(A.shape)
        fd = (losses(A + h * E) - losses(A - h * E)) / (2 * h)
        an = np.einsum("bij,bij->b", g, E)
        assert np.all(np.abs(fd - an) <= 1e-5 * np.maximum(1.0, np.abs(an))), (fd, an)


def test_fp32_vs_torch_svd(ad):
    import torch
    m, n, k, count = 128, 64, 16, 64
    A, w, GU, GV = problem(count, m, n, k, seed=33)
    g, S = grad_ours(ad, A.astype(np.float32), w, GU, GV, k, torch.float32)
    At = torch.tensor(A, dtype=torch.float64, device="cuda", requires_grad=True)
    Ut, St, Vht = torch.linalg.svd(At, full_matrices=False)
    Vt = Vht.mT
    with torch.no_grad():
        piv = torch.argmax(Vt.abs(), dim=1, keepdim=True)
        sg = torch.sign(torch.gather(Vt, 1, piv))
    Ut, Vt = Ut * sg, Vt * sg
    t = lambda x: torch.tensor(x, dtype=torch.float64, device="cuda")
    L = (t(w) * St).sum() + (t(GU) * Ut[:, :, :k]).sum() + (t(GV) * Vt[:, :, :k]).sum()
    L.backward()
    ref = At.grad.cpu().numpy()
    assert np.max(np.abs(S - St.detach().cpu().numpy())) <= 64 * n * np.finfo(np.float32).eps * 10
    for b in range(count):
        assert np.max(np.abs(g[b] - ref[b])) <= 5e-3 * np.max(np.abs(ref[b])), b


@pytest.mark.late
def test_full_batch(ad):
    # the differentiable-batch workload itself: 4096 FP32 matrices 128 x 64, k = 16.
    # Forward: every sigma within 640 n eps_32 of the construction (sigma in [0.1, 10]);
    # backward: the adjoint kernel on the forward's own U, S, V against the restatement
    # of the formula, every matrix, 2e-4 relative to max |dA| as above.
    import torch
    count, m, n, k = 4096, 128, 64, 16
    A, Ss = ad.spaced_sigma_matrices(count, m, n, seed=91)
    rng = np.random.default_rng(92)
    w, GU, GV = rng.standard_normal((count, n)), rng.standard_normal((count, m, k)), rng.standard_normal((count, n, k))
    At = torch.tensor(A, dtype=torch.float32, device="cuda")
    S, U, V, info = ad.svd_batch_dev(At)
    assert int((info < 0).sum()) == 0
    S, U, V = ad._sort_and_fix(S, U, V)
    eps = np.finfo(np.float32).eps
    assert np.max(np.abs(S.double().cpu().numpy() - Ss)) <= 640 * n * eps
    t = lambda x: torch.tensor(x, dtype=torch.float32, device="cuda")
    dA = ad.adjoint(U, S, V, t(w), t(GU), t(GV)).double().cpu().numpy()
    Un, Sn, Vn = U.double().cpu().numpy(), S.double().cpu().numpy(), V.double().cpu().numpy()
    worst = 0.0
    for b in range(count):
        ref = adjoint_np(Un[b], Sn[b], Vn[b], w[b], GU[b], GV[b])
        worst = max(worst, np.max(np.abs(dA[b] - ref)) / np.max(np.abs(ref)))
    assert worst <= 2e-4, worst


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_gap_broadening(ad, dtype_name):
    # a repeated singular value: the broadened kernel stays finite and matches the formula
    import torch
    dtype = getattr(torch, dtype_name)
    rng = np.random.default_rng(8)
    m, n, k = 64, 32, 8
    U = np.linalg.qr(rng.standard_normal((m, n)))[0][None].astype(dtype_name).astype(np.float64)
    V = np.linalg.qr(rng.standard_normal((n, n)))[0][None].astype(dtype_name).astype(np.float64)
    S = np.linspace(5.0, 0.5, n)[None]
    S[0, 3] = S[0, 2]
    dS, dU, dV = rng.standard_normal((1, n)), rng.standard_normal((1, m, k)), rng.standard_normal((1, n, k))
    t = lambda x: torch.tensor(x, dtype=dtype, device="cuda")
    dA = ad.adjoint(t(U), t(S), t(V), t(dS), t(dU), t(dV), gap=1e-3).double().cpu().numpy()[0]
    ref = adjoint_np(U[0], S[0], V[0], dS[0], dU[0], dV[0], gap=1e-3)
    assert np.all(np.isfinite(dA))
    tol = 1e-12 if dtype_name == "float64" else 2e-4
    assert np.max(np.abs(dA - ref)) <= tol * np.max(np.abs(ref))


def test_adjoint_errors(ad):
    import torch
    from vecjac_gb300 import api
    f = api.lib().vj_dsvd_adjoint_batch_dev
    import ctypes as C
    z = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = C.c_void_p(z.data_ptr())
    # m < n
    assert f(C.c_longlong(1), C.c_ulonglong(4), C.c_ulonglong(8), C.c_ulonglong(1), p, p, p, p, p, p, p,
             C.c_double(0), None) == api.VJ_ERR_ARG
    # k > n
    assert f(C.c_longlong(1), C.c_ulonglong(8), C.c_ulonglong(4), C.c_ulonglong(5), p, p, p, p, p, p, p,
             C.c_double(0), None) == api.VJ_ERR_ARG
    # working set larger than shared memory
    assert f(C.c_longlong(1), C.c_ulonglong(4096), C.c_ulonglong(64), C.c_ulonglong(8), p, p, p, p, p, p, p,
             C.c_double(0), None) == api.VJ_ERR_ARG
    # empty batch
    assert f(C.c_longlong(0), C.c_ulonglong(8), C.c_ulonglong(4), C.c_ulonglong(1), p, p, p, p, p, p, p,
             C.c_double(0), None) == 0
