"""Batched SVD of uneven matrices in one persistent launch (vj_?vjsvd_batch_dev).

Every matrix of the batch must give bit for bit what the oracle restatement gives for
that matrix padded to the reference's shape rules -- sweep count, U, V, eS, fS -- whatever
its neighbours in the batch; a zero matrix and a non-finite matrix inside the batch get
the reference's return values without disturbing the others; the autotuned block size
and a CUDA-graph replay give the same bits.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from vecjac_gb300 import build
    build.build()
    O.build()
    return O.Restatement()


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint8),
                                                                             b[~nb].view(np.uint8))


def uneven(count, seed, mmax=96):
    from vecjac_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    mats = []
    for i in range(count):
        m = int(rng.integers(16, mmax + 1))
        n = int(rng.integers(8, m + 1))
        A, _ = W.svd_matrix(m, n, seed=seed * 1000 + i, lo=-4.0)
        mats.append(A)
    return mats


@pytest.mark.parametrize("kind", ["d", "s"])
@pytest.mark.parametrize("strategy", [4, 2])
def test_batch_vs_oracle(env, kind, strategy):
    from vecjac_gb300 import batch as B
    rst = env
    mats = uneven(24, seed=7 if kind == "d" else 8)
    mats.append(np.zeros((24, 16)))                        # zero matrix: returns 0
    bad = np.ones((32, 16))
    bad[3, 4] = np.inf
    mats.append(bad)                                         # non-finite: -80
    res = B.svd_batch(mats, kind, strategy=strategy, block=128)
    dt = np.float64 if kind == "d" else np.float32
    for A, r in zip(mats, res):
        m2, n2 = B.padded_shape(A.shape[0], A.shape[1], kind)
        P = np.zeros((m2, n2), dt)
        P[:A.shape[0], :A.shape[1]] = A
        js, stp = rst.pjs(strategy, n2)
        o = rst.vjsvd(kind, P, js, stp)
        assert r[0] == o[0], (A.shape, r[0], o[0])
        if o[0] < 0:
            continue
        for x, y in zip(r[1:], o[1:]):
            assert same(x, y), A.shape


@pytest.mark.parametrize("kind", ["d", "s"])
def test_batch_autotune_and_graph(env, kind):
    import torch
    from vecjac_gb300 import batch as B
    mats = uneven(64, seed=11, mmax=160)
    if kind == "s":
        mats = [A.astype(np.float32) for A in mats]
    b = B.Batch(mats, kind)
    blk, occ = B.autotune(b, 4, sample=32)
    assert blk in (64, 128, 256) and occ in (2, 3, 4, 5)
    b.run(4, block=blk, occupancy=occ)
    torch.cuda.synchronize()
    first = b.results()
    # every launch configuration gives the same bits (each matrix's arithmetic is fixed)
    for rb, ro in ((64 if blk != 64 else 128, 0), (256, 3), (128, 4), (64, 6)):
        ref = B.Batch(mats, kind)
        ref.run(4, block=rb, occupancy=ro)
        torch.cuda.synchronize()
        for x, y in zip(first, ref.results()):
            assert x[0] == y[0]
            for u, v in zip(x[1:], y[1:]):
                assert same(u, v)
    g = B.capture(b, 4, block=blk, occupancy=occ)
    g.replay()
    torch.cuda.synchronize()
    for x, y in zip(first, b.results()):
        assert x[0] == y[0]
        for u, v in zip(x[1:], y[1:]):
            assert same(u, v)


@pytest.mark.late
def test_full_size_fp32_batch(env):
    """20,000 FP32 matrices with the uneven workload's shapes (m ~ U{16..512},
    n ~ U{8..m}; Gaussian entries, which build in seconds) in one persistent launch:
    every matrix converges, and a random sample of 500 has its singular values within
    4 n eps sigma_max of LAPACK's and V orthogonal within 96 n eps (n the padded column
    count; the restatement, bit-identical per matrix, measures 0.62 and 26-38 n eps)."""
    import torch
    from vecjac_gb300 import batch as B
    from vecjac_gb300 import workloads as W
    m, n = W.uneven_shapes(20000, 31)
    rng = np.random.default_rng(32)
    mats = [rng.standard_normal((int(a), int(b))).astype(np.float32) for a, b in zip(m, n)]
    b = B.Batch(mats, "s")
    blk, occ = B.autotune(b, 4)
    b.run(4, block=blk, occupancy=occ)
    torch.cuda.synchronize()
    info = b.info.cpu().numpy()
    assert np.all(info > 0) and np.all(info < 999), (info.min(), info.max())
    eps = np.finfo(np.float32).eps
    for i in np.random.default_rng(0).choice(len(mats), 500, replace=False):
        m2, n2 = int(b.m[i]), int(b.n[i])
        eS = b.eS[b.offS[i]:b.offS[i] + n2].double().cpu().numpy()
        fS = b.fS[b.offS[i]:b.offS[i] + n2].double().cpu().numpy()
        V = b.V[b.offV[i]:b.offV[i] + n2 * n2].double().cpu().numpy().reshape((n2, n2), order="F")
        nn = mats[i].shape[1]
        sig = np.sort(fS * np.exp2(eS))[::-1][:nn]
        ref = np.linalg.svd(mats[i].astype(np.float64), compute_uv=False)
        assert np.max(np.abs(sig - ref)) <= 4 * n2 * eps * ref[0], i
        assert np.linalg.norm(V.T @ V - np.eye(n2)) <= 96 * n2 * eps, i
