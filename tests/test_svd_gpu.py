"""One-sided Jacobi SVD on the GPU through the C ABI (dvjsvd_/zvjsvd_/svjsvd_/cvjsvd_).

Parity is bit-exact: the golden fixtures are outputs of VecJac compiled from its own
sources (with the project's column norm in place of BLAS xNRM2), and larger seeded cases
are compared with the oracle restatement. Size-independent properties (singular values
against LAPACK within 64 n eps for a well-conditioned matrix, orthogonality of U and V
within 16 n eps) cover sizes the CPU oracle cannot finish quickly.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


@pytest.fixture(scope="module")
def rst():
    O.build()
    return O.Restatement()


def same(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint8), b[~nb].view(np.uint8))


SVD_FILES = sorted(glob.glob(os.path.join(GOLD, "svd_*.npz")))
# the fixtures of the rare paths (rescaling, shears, rank deficiency, preset V, sweep caps,
# extreme condition) run after the common ones
EDGE = ("graded", "zerocol", "presetV", "swp", "k1e12")
SVD_PARAMS = [pytest.param(p, id=os.path.basename(p)[4:-4],
                           marks=[pytest.mark.late] if any(e in os.path.basename(p) for e in EDGE) else [])
              for p in SVD_FILES]


@pytest.mark.parametrize("path", SVD_PARAMS)
def test_golden(vj, path):
    g = np.load(path)
    kind = os.path.basename(path)[4]
    kw = dict(V=(g["V0"] if "V0" in g else None))
    if kind in "zc":
        kw.update(Gi=g["Gi"], Vi=(g["Vi0"] if "Vi0" in g else None))
    r = vj.vjsvd(kind, g["G"], g["js"], int(g["stp"]), int(g["swp"]), **kw)
    assert r[0] == int(g["ret"])
    for i, name in enumerate(["U", "V", "eS", "fS"] + (["Ui", "Vi"] if kind in "zc" else [])):
        assert same(r[1 + i], g[name]), name


CASES = [("d", 256, 128, 2), ("d", 192, 96 + 32, 4), ("s", 256, 128, 2), ("z", 128, 64, 2), ("c", 128, 64, 4),
         ("z", 96, 48, 4)]


@pytest.mark.parametrize("kind,m,n,sid", CASES)
def test_vs_oracle(vj, rst, kind, m, n, sid):
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(m, n, seed=m + n + ord(kind), complex_=(kind in "zc"))
    js, stp = rst.pjs(sid, n)
    kw = dict(Gi=A.imag) if kind in "zc" else {}
    ro = rst.vjsvd(kind, A.real, js, stp, **kw)
    rg = vj.vjsvd(kind, A.real, js, stp, **kw)
    assert rg[0] == ro[0] and rg[0] > 0
    for x, y in zip(ro[1:], rg[1:]):
        assert same(x, y)


def test_preset_v_and_swp_cap(vj, rst):
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(64, 32, seed=5)
    V0 = W.haar(32, np.random.default_rng(6)) * 0.25
    js, stp = rst.pjs(2, 32)
    for swp in (1, 3, 999):
        ro = rst.vjsvd("d", A, js, stp, swp=swp, V=V0)
        rg = vj.vjsvd("d", A, js, stp, swp=swp, V=V0)
        assert rg[0] == ro[0]
        for x, y in zip(ro[1:], rg[1:]):
            assert same(x, y)


@pytest.mark.parametrize("sid", [2, 4])
@pytest.mark.parametrize("n", [2, 16, 64, 250, 1024])
def test_pjs_tables(vj, rst, sid, n):
    t, stp = vj.pjs(sid, n)
    to, stpo = rst.pjs(sid, n)
    assert stp == stpo
    assert np.array_equal(t, to)


def test_pjs_errors(vj):
    assert vj.pjs(2, 7)[0] is None
    assert vj.pjs(3, 8)[0] is None


def test_argument_errors(vj):
    G = np.zeros((16, 32))
    js = np.zeros((31, 32), np.uint32)
    assert vj.vjsvd("d", G, js, 31)[0] == -1            # m < n
    G = np.zeros((20, 16))
    js = np.zeros((15, 16), np.uint32)
    assert vj.vjsvd("d", G, js, 15)[0] == -1            # m % 8
    G = np.zeros((32, 24))
    assert vj.vjsvd("d", G, np.zeros((23, 24), np.uint32), 23)[0] == -2  # (n/2) % 8
    G = np.zeros((32, 16))
    assert vj.vjsvd("d", G, np.zeros((15, 16), np.uint32), 15)[0] == 0  # zero matrix
    assert vj.vjsvd("s", np.zeros((32, 16), np.float32), np.zeros((15, 16), np.uint32), 15)[0] == -2
    G = np.ones((16, 16))
    G[0, 0] = np.inf
    assert vj.vjsvd("d", G, vj.pjs(2, 16)[0], 15)[0] == -80   # non-finite input
    G = np.ones((16, 16))
    assert vj.vjsvd("d", G, vj.pjs(2, 16)[0], 15, V=np.zeros((16, 16)))[0] == -13  # zero preset V


@pytest.mark.parametrize("kind,m,n", [("d", 1024, 512), ("z", 512, 256), ("s", 512, 256)])
def test_properties_large(vj, kind, m, n):
    """well-conditioned (sigma in [1e-3, 1]) matrices: sigma within 64 n eps of LAPACK's,
    ||U^H U - I||_F and ||V^H V - I||_F within 16 n eps"""
    from vecjac_gb300 import workloads as W
    cx = kind in "zc"
    A, s = W.svd_matrix(m, n, seed=77, lo=-3.0, complex_=cx)
    js, stp = vj.pjs(4, n)
    kw = dict(Gi=A.imag) if cx else {}
    r = vj.vjsvd(kind, A.real, js, stp, **kw)
    assert 0 < r[0] < 999
    eps = np.finfo(np.float64 if kind in "dz" else np.float32).eps
    sig = r[4].astype(np.float64) * np.exp2(r[3].astype(np.float64))
    ref = np.linalg.svd(A.astype(np.complex128 if cx else np.float64), compute_uv=False)
    err = np.max(np.abs(np.sort(sig)[::-1] - ref) / ref)
    assert err <= 64 * n * eps, err
    U = r[1].astype(np.float64) + (1j * r[5].astype(np.float64) if cx else 0)
    V = r[2].astype(np.float64) + (1j * r[6].astype(np.float64) if cx else 0)
    ou = np.linalg.norm(U.conj().T @ U - np.eye(n)) / (n * eps)
    ov = np.linalg.norm(V.conj().T @ V - np.eye(n)) / (n * eps)
    assert ou <= 16, ou
    # V accumulates every rotation of every sweep; the reference's own algorithm (to which
    # this result is bit-identical at smaller sizes) reaches 10-16 n eps at n = 128..256,
    # so V is held to 32 n eps
    assert ov <= 32, ov
    # A V = U diag(sigma)
    res = np.linalg.norm(A @ V - U * sig) / np.linalg.norm(A)
    assert res <= 16 * n * eps


@pytest.mark.late
@pytest.mark.parametrize("kind,m,n,sid", [("d", 256, 128, 4), ("z", 128, 64, 2), ("s", 256, 128, 4)])
def test_trace_matches_oracle(vj, rst, kind, m, n, sid):
    """vj_last_trace (the counterpart of the reference's JTRACE per-sweep log): the GPU's
    transformed pairs per sweep equal the restatement's, sweep for sweep."""
    from vecjac_gb300 import api
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(m, n, seed=3 * m + n, complex_=(kind in "zc"))
    js, stp = rst.pjs(sid, n)
    kw = dict(Gi=A.imag) if kind in "zc" else {}
    ro = rst.vjsvd(kind, A.real, js, stp, **kw)
    to = rst.last_swt()
    rg = vj.vjsvd(kind, A.real, js, stp, **kw)
    tg = api.last_trace()
    assert rg[0] == ro[0] > 0
    # one entry per sweep run (the last transforms nothing); the first 64 are kept
    assert tg["sweeps"] == ro[0] + 1 and len(to) == min(ro[0] + 1, 64)
    assert tg["rotations"] == to


@pytest.mark.late
def test_full_size_dvjsvd_1024(vj):
    """the benchmark's 1024 x 1024 FP64 matrix (sigma = 10^U(-6, 0), same seed) through the
    host entry: |sigma - sigma_exact| <= 4 n eps sigma_max, ||U^T U - I||_F <= 16 n eps,
    ||V^T V - I||_F <= 128 n eps, ||A V - U Sigma||_F <= n eps ||A||_F. The restatement
    (bit-identical at smaller sizes) measures 0.56, 3.8, 52 and 0.044 n eps on this
    matrix in 21 sweeps; V accumulates every rotation of every sweep."""
    from vecjac_gb300 import workloads as W
    m = n = 1024
    A, s = W.svd_matrix(m, n, seed=2024, lo=-6.0)
    js, stp = vj.pjs(4, n)
    r = vj.vjsvd("d", A, js, stp)
    assert 0 < r[0] < 999, r[0]
    eps = np.finfo(np.float64).eps
    sig = r[4] * np.exp2(r[3])
    assert np.max(np.abs(np.sort(sig)[::-1] - s)) <= 4 * n * eps * s[0]
    U, V = r[1], r[2]
    assert np.linalg.norm(U.T @ U - np.eye(n)) <= 16 * n * eps
    assert np.linalg.norm(V.T @ V - np.eye(n)) <= 128 * n * eps
    assert np.linalg.norm(A @ V - U * sig) <= n * eps * np.linalg.norm(A)


def test_device_entry(vj, rst):
    import torch
    from vecjac_gb300 import workloads as W
    m, n = 128, 64
    A, _ = W.svd_matrix(m, n, seed=3)
    js, stp = rst.pjs(2, n)
    ro = rst.vjsvd("d", A, js, stp)
    G = torch.tensor(A.T.copy(), dtype=torch.float64, device="cuda")   # column-major storage
    V = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    eS = torch.zeros(n, dtype=torch.float64, device="cuda")
    fS = torch.zeros(n, dtype=torch.float64, device="cuda")
    dj = torch.tensor(js.astype(np.int32), device="cuda")
    r = vj.vjsvd_dev("d", m, n, G, m, V, n, eS, fS, dj, stp)
    torch.cuda.synchronize()
    assert r == ro[0]
    assert same(G.cpu().numpy().T, ro[1])
    assert same(V.cpu().numpy().T, ro[2])
    assert same(eS.cpu().numpy(), ro[3]) and same(fS.cpu().numpy(), ro[4])
