"""The 2x2 properties of tests/props2x2.py on the oracle's outputs (CPU): they hold within
the bounds the full-size GPU test uses (orthogonality 8 eps, residual 12 eps, permutation
bits exact; measured 2.7 eps and 3.4 eps at most over these batches), and they catch a
planted error (a sine with the wrong sign, a swapped eigenvalue pair)."""
import numpy as np
import pytest

from props2x2 import props2x2

ORTH, RESID = 8.0, 12.0


@pytest.fixture(scope="module")
def rst():
    from oracle import oracle as O
    O.build()
    return O.Restatement()


def run(rst, kind, sgn, n, seed=3):
    import torch
    from vecjac_gb300 import workloads as W
    ins = W.pairs2x2(kind, n, seed=seed)
    r = rst.bjac2(kind, sgn * n, *ins)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x))
    if kind in "zc":
        a11, a22, a21, a21i = ins
        c, t, ti, l1, l2, p = r[1:]
    else:
        a11, a22, a21 = ins
        a21i = ti = np.zeros_like(a11)
        c, t, l1, l2, p = r[1:]
    return [T(x) for x in (a11, a22, a21, a21i, c, t, ti, l1, l2, p.astype(np.int64))]


@pytest.mark.parametrize("kind", "dszc")
@pytest.mark.parametrize("sgn", [-1, 1])
def test_oracle_within_bounds(rst, kind, sgn):
    o, r, bad, n = props2x2(kind, sgn, *run(rst, kind, sgn, 1 << 18))
    assert o <= ORTH and r <= RESID and bad == 0, (o, r, bad)


def test_planted_errors_are_caught(rst):
    a = run(rst, "d", -1, 1 << 12)
    t = a[5].clone()
    k = int(t.abs().argmax())        # a rotation that matters
    t[k] = -t[k]
    o, r, bad, _ = props2x2("d", -1, *(a[:5] + [t] + a[6:]))
    assert r > 1e3
    l1, l2 = a[7].clone(), a[8].clone()
    k = int((a[7] - a[8]).abs().argmax())
    l1[k], l2[k] = a[8][k], a[7][k]
    o, r, bad, _ = props2x2("d", -1, *(a[:7] + [l1, l2] + a[9:]))
    assert r > 1e3 and bad >= 1
