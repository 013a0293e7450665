"""The C restatement (oracle/vjo.c) reproduces the reference's own outputs bit for bit.

The fixtures in tests/golden/ were produced by VecJac compiled from its sources
(tests/golden/make_golden.py); this pins the oracle that the GPU tests rely on.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def rst():
    O.build()
    return O.Restatement()


def same_bits(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("kind", list("dszc"))
@pytest.mark.parametrize("tag,sgn,internal", [("sin", -1, False), ("tan", 1, False), ("isec", -1, True),
                                              ("itan", 1, True)])
def test_bjac2_golden(rst, kind, tag, sgn, internal):
    g = np.load(os.path.join(GOLD, f"bjac2_{kind}.npz"))
    ins = [g["a11"], g["a22"], g["a21"]] + ([g["a21i"]] if kind in "zc" else [])
    n = ins[0].size
    r = rst.bjac2(kind, sgn * n, *ins, internal=internal, p=(g["p_in"].copy() if internal else None))
    assert r[0] >= 0
    names = ["c", "at", "sat", "l1", "l2", "p"] if kind in "zc" else ["c", "at", "l1", "l2", "p"]
    for name, arr in zip(names, r[1:]):
        assert same_bits(arr, g[f"{tag}_{name}"]), (kind, tag, name)


SVD_FILES = sorted(glob.glob(os.path.join(GOLD, "svd_*.npz")))


@pytest.mark.parametrize("path", SVD_FILES, ids=[os.path.basename(p)[4:-4] for p in SVD_FILES])
def test_svd_golden(rst, path):
    g = np.load(path)
    kind = os.path.basename(path)[4]
    kw = dict(js=g["js"], stp=int(g["stp"]), swp=int(g["swp"]), V=(g["V0"] if "V0" in g else None))
    if kind in "zc":
        kw.update(Gi=g["Gi"], Vi=(g["Vi0"] if "Vi0" in g else None))
    r = rst.vjsvd(kind, g["G"], **kw)
    assert r[0] == int(g["ret"])
    for i, name in enumerate(["U", "V", "eS", "fS"] + (["Ui", "Vi"] if kind in "zc" else [])):
        assert same_bits(r[1 + i], g[name]), name


def test_pjs_placeholder_contract(rst):
    """Each row is a permutation of 0..n-1 read as pairs with p < q; a sweep covers every pair."""
    for sid, n in ((2, 16), (4, 16), (2, 64), (4, 32)):
        t, stp = rst.pjs(sid, n)
        assert stp == (n - 1 if sid == 2 else n)
        seen = set()
        for row in t:
            assert sorted(row) == list(range(n))
            for k in range(0, n, 2):
                p, q = int(row[k]), int(row[k + 1])
                assert p < q
                seen.add((p, q))
        assert len(seen) == n * (n - 1) // 2


def test_nrm2_properties(rst):
    rng = np.random.default_rng(0)
    x = rng.standard_normal(1000)
    assert abs(rst.nrm2(x) - np.linalg.norm(x)) <= 4e-16 * 1000 * np.linalg.norm(x)
    assert rst.nrm2(x * 2.0 ** 900) == rst.nrm2(x) * 2.0 ** 900
    assert rst.nrm2(x * 2.0 ** -1000) > 0
    assert rst.nrm2(np.zeros(7)) == 0.0


def nan_same(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.dtype.kind != "f":
        return np.array_equal(a, b)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint8), b[~nb].view(np.uint8))


@pytest.mark.parametrize("kind", list("dszc"))
@pytest.mark.parametrize("tag,sgn", [("sin", -1), ("tan", 1)])
def test_bjac2_special_golden(rst, kind, tag, sgn):
    """inf and NaN inputs: identical to the reference up to NaN payloads"""
    g = np.load(os.path.join(GOLD, f"bjac2_{kind}_special.npz"))
    ins = [g["a11"], g["a22"], g["a21"]] + ([g["a21i"]] if kind in "zc" else [])
    n = ins[0].size
    r = rst.bjac2(kind, sgn * n, *ins)
    names = ["c", "at", "sat", "l1", "l2", "p"] if kind in "zc" else ["c", "at", "l1", "l2", "p"]
    for name, arr in zip(names, r[1:]):
        assert nan_same(arr, g[f"{tag}_{name}"]), (kind, tag, name)


def test_swt_trace(rst):
    """The restatement's per-sweep count of transformed pairs (the reference's JTRACE
    "sw swt" lines): one entry per sweep run, all nonzero but the last, which ends the
    run with nothing to transform."""
    from vecjac_gb300 import workloads as W
    A, _ = W.svd_matrix(128, 64, seed=1)
    js, stp = rst.pjs(4, 64)
    r = rst.vjsvd("d", A, js, stp)
    t = rst.last_swt()
    assert r[0] > 0 and len(t) == r[0] + 1 and t[-1] == 0 and all(x > 0 for x in t[:-1])
    assert t[0] == stp * 32        # the first sweep transforms every pair of a random matrix


@pytest.mark.parametrize("kind,m,n,sid", [("d", 256, 128, 2), ("d", 192, 128, 4), ("s", 256, 128, 2),
                                          ("z", 128, 64, 2), ("c", 128, 64, 4), ("z", 96, 48, 4)])
def test_reference_vs_restatement(rst, kind, m, n, sid):
    """The reference compiled from its own sources (oracle/_ref, x86 with AVX-512 only)
    against the restatement on the seeded matrices of the GPU parity test
    (test_svd_gpu.py::test_vs_oracle): bit for bit, sweep counts included, so that the GPU
    results that equal the restatement there equal the reference's."""
    import numpy as np
    from oracle import oracle as O
    from vecjac_gb300 import workloads as W
    if not os.path.exists(O.REF_PATH):
        pytest.skip("the reference is compiled only on an x86 host with AVX-512")
    ref = O.Reference()
    ref.mode(0)
    A, _ = W.svd_matrix(m, n, seed=m + n + ord(kind), complex_=(kind in "zc"))
    js, stp = rst.pjs(sid, n)
    kw = dict(Gi=A.imag) if kind in "zc" else {}
    rr = ref.vjsvd(kind, A.real, js=js, stp=stp, **kw)
    ro = rst.vjsvd(kind, A.real, js, stp, **kw)
    assert rr[0] == ro[0] > 0
    for x, y in zip(rr[1:], ro[1:]):
        x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8))


@pytest.mark.parametrize("kind", "dszc")
def test_reference_vs_restatement_bjac2(rst, kind):
    """The compiled reference against the restatement on the 2^18-element batches of the
    GPU parity test (test_bjac2_gpu.py::test_vs_oracle, benchmark distribution), in its
    three forms (sines, tangents, the masked secant variant): bit for bit."""
    import numpy as np
    from oracle import oracle as O
    from vecjac_gb300 import workloads as W
    if not os.path.exists(O.REF_PATH):
        pytest.skip("the reference is compiled only on an x86 host with AVX-512")
    ref = O.Reference()
    ref.mode(0)
    n = 1 << 18
    ins = W.pairs2x2(kind, n, seed=3)
    a21i = ins[3] if kind in "zc" else None
    lanes = 8 if kind in "dz" else 16
    for sgn, internal in ((-1, False), (1, False), (-1, True)):
        pin = (np.arange(n // lanes, dtype=np.uint32) % 3) * np.uint32(0x10001) if internal else None
        rr = ref.bjac2(kind, sgn * n, ins[0], ins[1], ins[2], a21i, internal=internal,
                       p=None if pin is None else pin.copy())
        ro = rst.bjac2(kind, sgn * n, ins[0], ins[1], ins[2], a21i, internal=internal,
                       p=None if pin is None else pin.copy())
        for x, y in zip(rr[1:], ro[1:]):
            x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), (kind, sgn, internal)


@pytest.mark.parametrize("kind", "zc")
def test_split_merge_golden(rst, kind):
    """zsplit_/zmerge_ (csplit_/cmerge_) of the restatement equal the compiled reference's
    outputs bit for bit, signed zeros, infinities and a NaN payload included."""
    g = np.load(os.path.join(GOLD, "split_merge.npz"))
    r, Ar, Ai = rst.split(kind, g[kind + "_A"])
    assert r == int(g[kind + "_split_ret"]) == 1
    assert same_bits(Ar, g[kind + "_Ar"]) and same_bits(Ai, g[kind + "_Ai"])
    q, B = rst.merge(kind, g[kind + "_re"], g[kind + "_im"])
    assert q == int(g[kind + "_merge_ret"]) == 1
    assert same_bits(B, g[kind + "_B"])
