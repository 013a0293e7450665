"""zsplit_/zmerge_ and csplit_/cmerge_ (interleaved <-> split-plane complex matrices) on
the GPU, through the C ABI, against the oracle's restatement (src/zsplit.c, src/zmerge.c)
and the compiled reference's outputs stored in tests/golden/split_merge.npz: bit for bit,
signed zeros, infinities and NaN payloads included."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "split_merge.npz")


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


def bits(x):
    return np.ascontiguousarray(x).view(np.uint8)


@pytest.mark.parametrize("kind", "zc")
def test_golden(vj, kind):
    g = np.load(GOLD)
    r, Ar, Ai = vj.split(kind, g[kind + "_A"])
    assert r == 1
    assert np.array_equal(bits(Ar), bits(g[kind + "_Ar"])) and np.array_equal(bits(Ai), bits(g[kind + "_Ai"]))
    q, B = vj.merge(kind, g[kind + "_re"], g[kind + "_im"])
    assert q == 1
    assert np.array_equal(bits(B), bits(g[kind + "_B"]))


@pytest.mark.parametrize("kind,m,n", [("z", 4096, 300), ("c", 2048, 129), ("z", 8, 1), ("c", 0, 5)])
def test_vs_oracle(vj, rst, kind, m, n):
    rng = np.random.default_rng(m + n)
    dt = np.float64 if kind == "z" else np.float32
    re, im = rng.standard_normal((m, n)).astype(dt), rng.standard_normal((m, n)).astype(dt)
    A = np.empty((m, n), np.complex128 if kind == "z" else np.complex64, order="F")
    A.real, A.imag = re, im
    r, Ar, Ai = vj.split(kind, A)
    ro, Aro, Aio = rst.split(kind, A)
    assert r == ro == 1
    assert np.array_equal(bits(Ar), bits(Aro)) and np.array_equal(bits(Ai), bits(Aio))
    q, B = vj.merge(kind, re, im)
    qo, Bo = rst.merge(kind, re, im)
    assert q == qo == 1 and np.array_equal(bits(B), bits(Bo))


@pytest.mark.parametrize("kind", "zc")
def test_device_forms_with_leading_dimensions(vj, kind):
    """The device forms honour every leading dimension and leave the padding rows alone."""
    import torch
    m, n, ldA, ldP = 64, 9, 72, 80
    dt = torch.float64 if kind == "z" else torch.float32
    rng = np.random.default_rng(3)
    Ah = rng.standard_normal((n, ldA, 2))
    A = torch.tensor(Ah, dtype=dt, device="cuda")          # interleaved, column j at A[j]
    Ar = torch.full((n, ldP), 7.0, dtype=dt, device="cuda")
    Ai = torch.full((n, ldP), 7.0, dtype=dt, device="cuda")
    assert vj.split_dev(kind, m, n, A, ldA, Ar, ldP, Ai, ldP) == 1
    torch.cuda.synchronize()
    ref = torch.tensor(Ah, dtype=dt)
    assert torch.equal(Ar[:, :m].cpu(), ref[:, :m, 0]) and torch.equal(Ai[:, :m].cpu(), ref[:, :m, 1])
    assert bool((Ar[:, m:] == 7).all()) and bool((Ai[:, m:] == 7).all())
    B = torch.full((n, ldA, 2), -1.0, dtype=dt, device="cuda")
    assert vj.merge_dev(kind, m, n, Ar, ldP, Ai, ldP, B, ldA) == 1
    torch.cuda.synchronize()
    assert torch.equal(B[:, :m].cpu(), ref[:, :m]) and bool((B[:, m:] == -1).all())
    # the reference's codes for a bad leading dimension
    assert vj.split_dev(kind, m, n, A, m - 4, Ar, ldP, Ai, ldP) == -4
    assert vj.merge_dev(kind, m, n, Ar, ldP, Ai, ldP + 1, B, ldA) == -6
