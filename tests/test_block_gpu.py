"""Block one-sided Jacobi in FP32 on the tensor cores (split-BF16x3 tcgen05 products with
FP32 accumulation): the Gram matrices of the block pairs, the block rotations, and whole
block sweeps, through the C ABI, against FP64 evaluations of the same products in numpy.

Tolerances: with the six-term split every product is as accurate as FP32 arithmetic, so
a Gram entry is held to 4 sqrt(m) eps32 |x_i| |x_j| + m eps32^2 terms and a rotated entry
to 8 sqrt(128) eps32 sum_k |x_k| |r_k| (FP32 accumulation of m or 128 exact products); the
three-term split (about 16 significant bits) to 2^-14 of the same scales.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
E32 = float(np.finfo(np.float32).eps)


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def pair_blocks(nb, step, k):
    N = nb - 1
    a, c = (step, N) if k == 0 else ((step + k) % N, (step + N - k) % N)
    return min(a, c), max(a, c)


def pair_cols(cplx, nb, step, k):
    """the 128 real columns of pair k: (plane, column) in the order of the library"""
    b = 32 if cplx else 64
    I, J = pair_blocks(nb, step, k)
    cols = list(range(I * b, I * b + b)) + list(range(J * b, J * b + b))
    return [(0, c) for c in cols] + ([(1, c) for c in cols] if cplx else [])


def planes(rng, cplx, rows, cols, scale=None):
    x = rng.standard_normal((1 + cplx, cols, rows)).astype(np.float32)  # [plane][column][row]
    if scale is not None:
        x *= scale[None, :, None].astype(np.float32)
    return x


def to_dev(x):
    import torch
    return torch.tensor(x, device="cuda")


@pytest.mark.parametrize("cplx,m,n,terms", [(0, 512, 256, 6), (1, 256, 128, 6), (0, 1000, 256, 6),
                                            (1, 4096, 256, 6), (0, 512, 256, 3)])
def test_gram(vj, cplx, m, n, terms):
    import torch
    rng = np.random.default_rng(m + n + cplx)
    # columns of very different lengths: the split keeps each product's relative accuracy
    X = planes(rng, cplx, m, n, scale=10.0 ** rng.uniform(-3, 3, n))
    Xd = to_dev(X)
    nb = n // (32 if cplx else 64)
    f = vj.lib().vj_block_gram_dev
    for step in range(nb - 1):
        S = torch.zeros((nb // 2, 128, 128), dtype=torch.float32, device="cuda")
        r = f(C.c_int(cplx), C.c_ulonglong(m), C.c_ulonglong(n), _p(Xd[0]), _p(Xd[1]) if cplx else None,
              C.c_ulonglong(m), C.c_int(step), C.c_int(terms), _p(S), None)
        assert r == nb // 2, r
        Sg = S.cpu().numpy().astype(np.float64)
        for k in range(nb // 2):
            Xk = np.stack([X[pl, c].astype(np.float64) for pl, c in pair_cols(cplx, nb, step, k)], axis=1)
            ref = Xk.T @ Xk
            nr = np.linalg.norm(Xk, axis=0)
            scale = np.outer(nr, nr)
            tol = (4 * np.sqrt(m) * E32 + m * E32 ** 2) if terms == 6 else 2.0 ** -14
            err = np.max(np.abs(Sg[k] - ref) / scale)
            assert err <= tol, (step, k, err, tol)


@pytest.mark.parametrize("cplx,m,n,terms", [(0, 512, 256, 6), (1, 384, 128, 6), (0, 200, 128, 6), (1, 256, 192, 3)])
def test_apply(vj, cplx, m, n, terms):
    import torch
    rng = np.random.default_rng(7 * m + n + cplx)
    G = planes(rng, cplx, m, n)
    W = planes(rng, cplx, n, n)
    nb = n // (32 if cplx else 64)
    step = nb // 2 - 1
    R = rng.standard_normal((nb // 2, 128, 128)).astype(np.float32)  # R[k][i][kk] = R_k(kk, i)
    Gd, Wd, Rd = to_dev(G), to_dev(W), to_dev(R)
    r = vj.lib().vj_block_apply_dev(C.c_int(cplx), C.c_ulonglong(m), C.c_ulonglong(n), _p(Gd[0]),
                                    _p(Gd[1]) if cplx else None, C.c_ulonglong(m), _p(Wd[0]),
                                    _p(Wd[1]) if cplx else None, C.c_ulonglong(n), C.c_int(step), C.c_int(terms),
                                    _p(Rd), None)
    assert r == nb // 2, r
    Gn, Wn = Gd.cpu().numpy(), Wd.cpu().numpy()
    tol = 8 * np.sqrt(128) * E32 if terms == 6 else 2.0 ** -14
    touched = set()
    for X, Xn, rows in ((G, Gn, m), (W, Wn, n)):
        for k in range(nb // 2):
            cols = pair_cols(cplx, nb, step, k)
            Xk = np.stack([X[pl, c].astype(np.float64) for pl, c in cols], axis=1)  # rows x 128
            Rk = R[k].T.astype(np.float64)  # Rk[kk][i]
            ref = Xk @ Rk
            got = np.stack([Xn[pl, c].astype(np.float64) for pl, c in cols], axis=1)
            scale = np.abs(Xk) @ np.abs(Rk)
            err = np.max(np.abs(got - ref) / scale)
            assert err <= tol, (k, err, tol)
            touched.update(cols)
        # columns of no pair of the step are not touched (all are, when every block is paired)
        for pl in range(1 + cplx):
            for c in range(n):
                if (pl, c) not in touched:
                    assert np.array_equal(Xn[pl, c], X[pl, c])


@pytest.mark.parametrize("cplx,m,n", [(0, 512, 256), (1, 512, 256)])
def test_sweeps_converge(vj, cplx, m, n):
    """Block sweeps from W = I: W stays unitary to FP32 accuracy, G stays G0 W, and the
    sweeps stop rotating (the columns orthogonal to the tolerance) within a few sweeps."""
    import torch
    rng = np.random.default_rng(11 + cplx)
    G0 = planes(rng, cplx, m, n, scale=10.0 ** rng.uniform(-2, 0, n))
    W0 = np.zeros((1 + cplx, n, n), np.float32)
    W0[0] = np.eye(n, dtype=np.float32)
    Gd, Wd = to_dev(G0), to_dev(W0)
    tol = 0.5 * np.sqrt(m) * E32
    mu = C.c_float(0)
    rots = []
    for _ in range(30):
        r = vj.lib().vj_block_sweep_dev(C.c_int(cplx), C.c_ulonglong(m), C.c_ulonglong(n), _p(Gd[0]),
                                        _p(Gd[1]) if cplx else None, C.c_ulonglong(m), _p(Wd[0]),
                                        _p(Wd[1]) if cplx else None, C.c_ulonglong(n), C.c_float(tol), C.c_int(1),
                                        C.c_int(6), C.byref(mu), None)
        assert r >= 0, r
        rots.append(r)
        if r == 0:
            break
    assert rots[-1] == 0, rots
    cx = lambda A: (A[0] + 1j * A[1]).T if cplx else A[0].T.astype(np.float64)  # [col][row] -> matrix
    G0m, Gm, Wm = cx(G0.astype(np.float64)), cx(Gd.cpu().numpy().astype(np.float64)), cx(
        Wd.cpu().numpy().astype(np.float64))
    assert np.max(np.abs(Wm.conj().T @ Wm - np.eye(n))) <= 8 * n * E32
    assert np.max(np.abs(Gm - G0m @ Wm)) <= 16 * np.sqrt(n) * E32 * np.max(np.abs(G0m)) * np.sqrt(n)
    # the columns of G are orthogonal to the tolerance and in descending order of norms
    # within every block pair's last visit
    H = Gm.conj().T @ Gm
    d = np.sqrt(np.real(np.diag(H)))
    off = np.abs(H - np.diag(np.diag(H))) / np.outer(d, d)
    assert np.max(off) <= 4 * tol, np.max(off)
    # singular values: those of G0 (the FP64 SVD of the FP32 input) within FP32 accuracy
    sv = np.sort(d)[::-1]
    s0 = np.linalg.svd(G0m, compute_uv=False)
    assert np.max(np.abs(sv - s0) / s0[0]) <= 32 * np.sqrt(n) * E32
