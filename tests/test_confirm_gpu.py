"""The finishing sweep's all-pairs check (preset = 2 of vj_?vjsvd_dev).

With preset = 2 the device SVD first checks every pair of its first sweep at once: a cheap
certificate (plain FP64 cosines with a rigorous error bound) for most pairs, the
reference's own compensated dot products and classification for the rest, and skips the
sweep when it would transform or swap nothing. The mixed-precision SVD uses it for its
finishing call. The outputs must be those of preset = 1 (the sweep run step by step) bit
for bit, whether the sweep is skipped (columns orthogonal to FP64 accuracy), decided
exactly for pairs near the tolerance, or needed (a pair far from orthogonal).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def columns(kind, m, n, seed):
    """G = Q diag(sigma) with Q's columns orthonormal to FP64 accuracy (Householder QR) and
    sigma descending, so that the pairs are orthogonal and in order."""
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((m, n))
    if kind == "z":
        A = A + 1j * rng.standard_normal((m, n))
    Q, _ = np.linalg.qr(A)
    sig = np.logspace(0, -6, n)
    return Q * sig


def run(vj, kind, G, js, stp, preset):
    import torch
    m, n = G.shape
    Gr = torch.tensor(np.ascontiguousarray(G.real.T), dtype=torch.float64, device="cuda")
    V = torch.eye(n, dtype=torch.float64, device="cuda")
    kw = {}
    if kind == "z":
        Gi = torch.tensor(np.ascontiguousarray(G.imag.T), dtype=torch.float64, device="cuda")
        Vi = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        kw = dict(Gi=Gi, ldGi=m, Vi=Vi, ldVi=n)
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    jd = torch.tensor(js.astype(np.int32), device="cuda")
    r = vj.vjsvd_dev(kind, m, n, Gr, m, V, n, eS, fS, jd, stp, swp=999, preset=preset, **kw)
    torch.cuda.synchronize()
    out = [Gr.cpu().numpy(), V.cpu().numpy(), eS.cpu().numpy(), fS.cpu().numpy()]
    if kind == "z":
        out += [kw["Gi"].cpu().numpy(), kw["Vi"].cpu().numpy()]
    return r, out


@pytest.mark.parametrize("kind", ["d", "z"])
@pytest.mark.parametrize("case", ["orthogonal", "near_tolerance", "one_pair_off"])
def test_check_matches_stepwise_sweep(vj, kind, case, monkeypatch, capfd):
    m, n = 512, 256
    G = columns(kind, m, n, 11 if kind == "d" else 12)
    tol = np.sqrt(m) * np.finfo(np.float64).eps / 2
    if case == "near_tolerance":
        # columns 0 and 1 at 0.95 of the reference's tolerance: no certificate, and the
        # exact decision is the reference's
        G[:, 1] = G[:, 1] + 0.95 * tol * np.linalg.norm(G[:, 1]) * G[:, 0] / np.linalg.norm(G[:, 0])
    elif case == "one_pair_off":
        G[:, 3] = G[:, 3] + 1e-9 * np.linalg.norm(G[:, 3]) * G[:, 2] / np.linalg.norm(G[:, 2])
    js, stp = vj.pjs(4, n)
    r1, o1 = run(vj, kind, G, js, stp, 1)
    monkeypatch.setenv("VJ_TRACE", "1")
    r2, o2 = run(vj, kind, G, js, stp, 2)
    monkeypatch.delenv("VJ_TRACE")
    err = capfd.readouterr().err
    assert r1 == r2 >= 0
    for a, b in zip(o1, o2):
        assert same(a, b)
    line = [l for l in err.splitlines() if "finishing sweep check" in l]
    print(kind, case, line)
    assert line
    if case == "one_pair_off":
        assert "sweep needed" in line[0]
    else:
        assert "sweep skipped" in line[0]
        # the certificate covers all but a few pairs of orthogonal columns
        assert int(line[0].split(":")[1].split()[0]) <= (n * (n - 1) // 2) // 100 + 1
