"""LAPACK xGESVJ as a second, independent oracle (oracle/lapack.py), on CPU.

The restatement's singular values against xGESVJ's, both one-sided Jacobi methods with
different pivoting and rotations:
  * plain matrices (sigma = 10^U(-6, 0)): |s - s_L| <= 4 n eps s_max;
  * column-graded matrices A = B D (B Gaussian, D spanning 12 decades in FP64, 5 in FP32):
    |s - s_L| <= 4 n eps s_L for EVERY singular value, the smallest included -- the
    relative accuracy that one-sided Jacobi has and bidiagonalisation does not
    (measured: <= 0.65 n eps).
Also the file driver (`python -m oracle.lapack`, the reference's src/tdgesvj.c) and the
exact `wide` encoder it uses.
"""
import os
import subprocess
import sys
from fractions import Fraction

import numpy as np
import pytest

from oracle import lapack as LA

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not LA.available(), reason="no LAPACK with xGESVJ in this numpy/scipy")


def graded(kind, m, n, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((m, n))
    if kind in "zc":
        B = B + 1j * rng.standard_normal((m, n))
    lo = -12 if kind in "dz" else -5
    return B * 10.0 ** rng.uniform(lo, 0, n)[None, :]


def sigma_of(eS, fS):
    eS, fS = np.asarray(eS, np.float64), np.asarray(fS, np.float64)
    ok = np.isfinite(eS)
    return np.sort(np.where(ok, np.ldexp(fS, np.where(ok, eS, 0).astype(np.int64)), 0.0))[::-1]


def check(kind, n, s, s_l, grade):
    eps = np.finfo(np.float64 if kind in "dz" else np.float32).eps
    s_l = np.sort(s_l)[::-1]
    if grade:
        assert np.all(np.abs(s - s_l) <= 4 * n * eps * s_l), np.max(np.abs(s - s_l) / s_l) / (n * eps)
    else:
        assert np.max(np.abs(s - s_l)) <= 4 * n * eps * s_l[0]


@pytest.fixture(scope="module")
def rst():
    from oracle import oracle as O
    O.build()
    return O.Restatement()


@pytest.mark.parametrize("kind,m,n", [("d", 128, 64), ("z", 96, 48), ("s", 128, 64), ("c", 128, 64)])
@pytest.mark.parametrize("grade", [False, True])
def test_restatement_vs_gesvj(rst, kind, m, n, grade):
    from vecjac_gb300 import workloads as W
    A = graded(kind, m, n, 7) if grade else W.svd_matrix(m, n, seed=3, complex_=(kind in "zc"))[0]
    js, stp = rst.pjs(4, n)
    r = rst.vjsvd(kind, A.real, js, stp, **(dict(Gi=A.imag) if kind in "zc" else {}))
    assert r[0] > 0
    info, s_l, U, V, st, _ = LA.gesvj(kind, A)
    assert info == 0 and int(st[1]) == n
    check(kind, n, sigma_of(r[3], r[4]), s_l, grade)


def test_gesvj_factors():
    # the second oracle itself: A V = U diag(s), V orthogonal
    A = graded("d", 64, 32, 1)
    info, s, U, V, st, _ = LA.gesvj("d", A)
    assert info == 0
    assert np.max(np.abs(A @ V - U * s)) <= 64 * 32 * np.finfo(float).eps * s[0]
    assert np.max(np.abs(V.T @ V - np.eye(32))) <= 64 * 32 * np.finfo(float).eps


@pytest.mark.parametrize("kind", "dz")
def test_file_driver(tmp_path, kind):
    from vecjac_gb300 import mtxio
    m, n = 48, 16
    A = graded(kind, m, n, 2)
    dt = np.complex128 if kind == "z" else np.float64
    base = str(tmp_path / "g")
    mtxio.write_matrix(base + ".G", A.astype(dt))
    r = subprocess.run([sys.executable, "-m", "oracle.lapack", str(m), str(n), base, kind], cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    f = r.stdout.strip().split(",")
    assert len(f) == 11 and f[0] == '"%s"' % base and int(f[3]) == 0
    info, s, U, V, st, sva = LA.gesvj(kind, A.astype(dt))
    raw = np.fromfile(base + ".SL", dtype=np.uint8)
    want = [Fraction(float(v)) * Fraction(float(st[0])) for v in sva]
    assert [mtxio.encode_wide(w) for w in want] == [bytes(raw[16 * i:16 * i + 16]) for i in range(n)]
    assert np.array_equal(mtxio.read_matrix(base + ".UL", m, n, dt), U)
    assert np.array_equal(mtxio.read_matrix(base + ".VL", n, n, dt), V)


def test_encode_wide():
    from vecjac_gb300 import mtxio
    rng = np.random.default_rng(5)
    a = rng.uniform(0.5, 2, 2000) * 2.0 ** rng.integers(-300, 300, 2000)
    b = rng.uniform(0.5, 2, 2000) * 2.0 ** rng.integers(-300, 300, 2000)
    for x, y in zip(a, b):
        p = Fraction(float(x)) * Fraction(float(y))
        q = mtxio.encode_wide(p, "q")
        v = int.from_bytes(q, "little")
        e, f = (v >> 112) & 0x7FFF, v & ((1 << 112) - 1)
        assert Fraction((1 << 112) | f) * Fraction(2) ** (e - 16383 - 112) == p   # exact in binary128
    if np.finfo(np.longdouble).nmant == 63:
        for x, y in zip(a, b):
            ld = np.longdouble(x) * np.longdouble(y)                          # rounded to nearest
            assert mtxio.encode_wide(Fraction(float(x)) * Fraction(float(y)), "l")[:10] == ld.tobytes()[:10]
    assert mtxio.encode_wide(0.0) == bytes(16) and mtxio.encode_wide(-1.5)[15] & 0x80
