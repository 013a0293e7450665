"""Mixed-precision SVD (FP32 presweeps + FP64 finishing sweeps) through the C ABI.

The mixed path is not bit-identical to dvjsvd_/zvjsvd_: its FP64 phase is the reference's
algorithm with a preset V (src/dvjsvd.c:88-96), applied to A V where V comes from rounds
of FP32 sweeps, each re-orthogonalised by two FP64 Newton-Schulz steps. It is checked against the oracle's FP64 SVD of
the same matrix (small sizes) and against the matrix's construction (larger sizes):
  |sigma_mixed - sigma_oracle| <= 32 n eps sigma_max,
  ||U^H U - I||_max, ||V^H V - I||_max <= 32 n eps,
  ||A V - U Sigma||_max <= 32 n eps ||A||_max.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


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


def run_mixed(vj, kind, A, sid=4, swp=999):
    import torch
    m, n = A.shape
    js, stp = vj.pjs(sid, n)
    G = torch.tensor(np.ascontiguousarray(A.real.T), dtype=torch.float64, device="cuda")
    Gi = torch.tensor(np.ascontiguousarray(A.imag.T), dtype=torch.float64, device="cuda") if kind == "z" else None
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.empty_like(V) if kind == "z" else None
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    r, r32, _ = vj.vjsvd_mixed_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, swp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n)
    torch.cuda.synchronize()
    U = G.cpu().numpy().T
    Vm = V.cpu().numpy().T
    if kind == "z":
        U = U + 1j * Gi.cpu().numpy().T
        Vm = Vm + 1j * Vi.cpu().numpy().T
    sig = fS.cpu().numpy() * np.exp2(eS.cpu().numpy())
    return r, r32, U, Vm, sig


def check_props(A, U, V, sig):
    n = A.shape[1]
    tol = 32 * n * EPS
    assert np.max(np.abs(U.conj().T @ U - np.eye(n))) <= tol
    assert np.max(np.abs(V.conj().T @ V - np.eye(n))) <= tol
    assert np.max(np.abs(A @ V - U * sig)) <= tol * np.max(np.abs(A)) * np.sqrt(n)


@pytest.mark.parametrize("kind,m,n", [("d", 128, 64), ("d", 96, 96), ("z", 128, 64), ("z", 64, 32)])
def test_mixed_vs_oracle(vj, rst, kind, m, n):
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(m, n, seed=5 + m + n, complex_=(kind == "z"))
    r, r32, U, V, sig = run_mixed(vj, kind, A)
    assert r >= 0 and r32 > 0, (r, r32)
    js, stp = rst.pjs(4, n)
    if kind == "z":
        ro = rst.vjsvd("z", A.real, js, stp, Gi=A.imag)
    else:
        ro = rst.vjsvd("d", A, js, stp)
    assert ro[0] >= 0
    so = ro[4] * np.exp2(ro[3])
    assert np.max(np.abs(np.sort(sig) - np.sort(so))) <= 32 * n * EPS * np.max(so)
    check_props(A, U, V, sig)


@pytest.mark.parametrize("kind,m,n", [("d", 512, 256), ("z", 256, 128)])
def test_mixed_relative_accuracy_vs_oracle(vj, rst, kind, m, n):
    """The target accuracy of the mixed path: with a column-scaled condition number <= 1e3
    (sigma log-uniform in [1e-3, 1], Haar factors, so every column mixes all of them) each
    singular value is within 64 n eps RELATIVE of the FP64 oracle's (the reference's
    algorithm in FP64, restated)."""
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(m, n, seed=41 + n, lo=-3.0, complex_=(kind == "z"))
    r, r32, U, V, sig = run_mixed(vj, kind, A)
    assert r >= 0 and r32 > 0, (r, r32)
    js, stp = rst.pjs(4, n)
    ro = rst.vjsvd("z", A.real, js, stp, Gi=A.imag) if kind == "z" else rst.vjsvd("d", A, js, stp)
    assert ro[0] >= 0
    so = np.sort(ro[4] * np.exp2(ro[3]))
    rel = np.max(np.abs(np.sort(sig) - so) / so)
    assert rel <= 64 * n * EPS, rel
    check_props(A, U, V, sig)


@pytest.mark.parametrize("kind,m,n", [("d", 1024, 1024), ("z", 1024, 512)])
def test_mixed_relative_accuracy_vs_plain(vj, kind, m, n):
    """The same bound at larger sizes against the plain FP64 path, which computes the
    reference's algorithm bit for bit (the FP64 oracle's result)."""
    import torch
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(m, n, seed=43 + n, lo=-3.0, complex_=(kind == "z"))
    r, r32, U, V, sig = run_mixed(vj, kind, A)
    assert r >= 0 and r32 > 0, (r, r32)
    js, stp = vj.pjs(4, n)
    G = torch.tensor(np.ascontiguousarray(A.real.T), dtype=torch.float64, device="cuda")
    Gi = torch.tensor(np.ascontiguousarray(A.imag.T), dtype=torch.float64, device="cuda") if kind == "z" else None
    Vd = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vdi = torch.empty_like(Vd) if kind == "z" else None
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    rp = vj.vjsvd_dev(kind, m, n, G, m, Vd, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vdi, ldVi=n)
    torch.cuda.synchronize()
    assert rp > 0
    sp = np.sort(fS.cpu().numpy() * np.exp2(eS.cpu().numpy()))
    rel = np.max(np.abs(np.sort(sig) - sp) / sp)
    assert rel <= 64 * n * EPS, rel


# the FP32 stages take block sweeps on the tensor cores by default from 16 block pairs per
# step (n >= 2048 real, 1024 complex); VJ_BLOCK=1 forces them at these sizes, VJ_BLOCK=0
# forces the column-pair sweeps
@pytest.mark.parametrize("blk", ["0", "1"])
@pytest.mark.parametrize("kind,m,n", [("d", 1024, 512), ("z", 512, 256)])
def test_mixed_large(vj, kind, m, n, blk, monkeypatch):
    from vecjac_gb300 import workloads as W
    monkeypatch.setenv("VJ_BLOCK", blk)
    A, s = W.svd_matrix(m, n, seed=11, complex_=(kind == "z"))
    r, r32, U, V, sig = run_mixed(vj, kind, A)
    assert vj.last_mixed_phases()["fp32_block_sweeps"] == (blk == "1")
    assert r >= 0 and r32 > 0
    # the reference's FP64 phase starts from columns orthogonal to twice its tolerance: it
    # confirms convergence within a few sweeps
    assert r <= 3, r
    assert np.max(np.abs(np.sort(sig)[::-1] - s)) <= 32 * n * EPS * s[0]
    check_props(A, U, V, sig)


@pytest.mark.late
def test_mixed_full_size(vj):
    # the benchmark's complex 4096 x 2048 matrix (sigma = 10^U(-8, 0)), same seed
    from vecjac_gb300 import workloads as W
    A, s = W.svd_matrix(4096, 2048, seed=2024, lo=-8.0, complex_=True)
    r, r32, U, V, sig = run_mixed(vj, "z", A)
    assert r >= 0 and r32 > 0, (r, r32)
    assert np.max(np.abs(np.sort(sig)[::-1] - s)) <= 32 * 2048 * EPS * s[0]
    check_props(A, U, V, sig)


@pytest.mark.parametrize("kind,m,n", [("d", 4608, 32), ("z", 4608, 32)])
def test_mixed_tall(vj, kind, m, n):
    # more rows than the register-resident presweep kernels hold: the two-pass kernel
    from vecjac_gb300 import workloads as W
    A, s = W.svd_matrix(m, n, seed=13, complex_=(kind == "z"))
    r, r32, U, V, sig = run_mixed(vj, kind, A)
    assert r >= 0 and r32 > 0
    assert np.max(np.abs(np.sort(sig)[::-1] - s)) <= 32 * n * EPS * s[0]
    check_props(A, U, V, sig)


@pytest.mark.parametrize("stages", [1, 3])
def test_mixed_stages(vj, stages):
    import torch
    from vecjac_gb300 import workloads as W
    m, n = 256, 128
    A, s = W.svd_matrix(m, n, seed=17, lo=-8.0)
    js, stp = vj.pjs(4, n)
    G = torch.tensor(np.ascontiguousarray(A.T), dtype=torch.float64, device="cuda")
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    r, r32, r64 = vj.vjsvd_mixed_dev("d", m, n, G, m, V, n, eS, fS, djs, stp, stages=stages)
    torch.cuda.synchronize()
    assert r >= 0 and r32 > 0 and r64 >= 0
    sig = fS.cpu().numpy() * np.exp2(eS.cpu().numpy())
    assert np.max(np.abs(np.sort(sig)[::-1] - s)) <= 32 * n * EPS * s[0]
    check_props(A, G.cpu().numpy().T, V.cpu().numpy().T, sig)


@pytest.mark.parametrize("blk", ["0", "1"])
def test_mixed_graded_and_rank_deficient(vj, rst, blk, monkeypatch):
    # column-graded (one-sided Jacobi's high relative accuracy must survive the FP32
    # stages) and rank-deficient (zero columns) matrices: singular values relative to the
    # oracle's FP64 SVD of the same matrix, with the column-pair and the block FP32 sweeps
    monkeypatch.setenv("VJ_BLOCK", blk)
    rng = np.random.default_rng(21)
    m, n = 256, 128
    B = rng.standard_normal((m, n))
    A = B * 10.0 ** (-np.linspace(0, 20, n))
    Z = rng.standard_normal((m, n))
    Z[:, [3, 40, 77]] = 0.0
    js, stp = rst.pjs(4, n)
    for M in (A, Z):
        r, r32, U, V, sig = run_mixed(vj, "d", M)
        assert r >= 0 and r32 > 0
        ro = rst.vjsvd("d", M, js, stp)
        so = np.sort(ro[4] * np.exp2(ro[3]))[::-1]
        sm = np.sort(sig)[::-1]
        nz = so > 0
        assert np.array_equal(sm > 0, nz)
        assert np.max(np.abs(sm[nz] - so[nz]) / so[nz]) <= 1e-12
        assert np.max(np.abs(V.T @ V - np.eye(n))) <= 32 * n * EPS


def test_mixed_errors(vj):
    import torch
    z = torch.zeros(64 * 32, dtype=torch.float64, device="cuda")
    v = torch.zeros(32 * 32, dtype=torch.float64, device="cuda")
    e = torch.zeros(32, dtype=torch.float64, device="cuda")
    f = torch.zeros(32, dtype=torch.float64, device="cuda")
    js, stp = vj.pjs(4, 32)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    # the reference's shape rules: m % 8 != 0 -> -1, (n/2) % 8 != 0 -> -2
    r, _, _ = vj.vjsvd_mixed_dev("d", 36, 32, z, 36, v, 32, e, f, djs, stp)
    assert r == -1
    r, _, _ = vj.vjsvd_mixed_dev("d", 64, 24, z, 64, v, 24, e, f, djs, stp)
    assert r == -2
    # a zero matrix: no sweeps, V = I, sigma = 0
    r, r32, _ = vj.vjsvd_mixed_dev("d", 64, 32, z, 64, v, 32, e, f, djs, stp)
    torch.cuda.synchronize()
    assert r == 0 and r32 == 0
    assert np.array_equal(v.cpu().numpy().reshape(32, 32), np.eye(32))
    assert not np.any(f.cpu().numpy() * np.exp2(e.cpu().numpy()))
