"""Seeded synthetic inputs for the Jacobi SVD and the batched 2x2 EVD.

The reference draws its test data from RDRAND (src/rnd.h:34), which cannot be replayed;
these generators produce the same kinds of inputs from a seed:

* ``pairs2x2``: SoA 2x2 Hermitian batches (a11, a22, a21[, a21i]) with entries
  ``±2^e * u``, ``e`` uniform in [-300, 300] (FP64) or [-40, 40] (FP32), ``u`` uniform in
  [1, 2) -- the distribution of the 2^28 / 2^27 element batched-EVD workload
  (``pairs2x2_torch``: the same, drawn with torch on a device).
* ``svd_matrix``: ``A = U diag(sigma) V^H`` with Haar-random orthogonal/unitary factors
  (QR of a Gaussian matrix, columns fixed by the phase of diag(R)) and log-uniform sigma
  sorted descending -- the 1024x1024 real and 4096x2048 complex SVD workloads.
* ``graded16``: a 16x16 matrix whose entries span the whole exponent range, built by the
  rule of the reference's etc/dgsex.c (columns j < 8: 2^(1023-j-|i-j|); j >= 8:
  2^(-51-j-|i-j|)); it drives the rescaling and shear paths of the SVD.
  ``graded32_f32`` is the same rule over the FP32 range.
* ``uneven_shapes`` / ``uneven_batch``: shapes, matrices and singular values of the
  20,000-matrix uneven batch.
"""
import numpy as np


def pairs2x2(kind, n, seed):
    """SoA inputs of ``n`` 2x2 matrices; kind in 'dszc'."""
    rng = np.random.default_rng(seed)
    dt = np.float64 if kind in "dz" else np.float32
    lo, hi = (-300, 300) if kind in "dz" else (-40, 40)
    out = []
    for _ in range(4 if kind in "zc" else 3):
        e = rng.integers(lo, hi + 1, n, dtype=np.int32)
        u = rng.uniform(1.0, 2.0, n)
        s = rng.integers(0, 2, n) * 2.0 - 1.0
        out.append(np.ldexp(s * u, e).astype(dt))
    return out


def pairs2x2_torch(kind, n, seed, device="cuda"):
    """The pairs2x2 distribution drawn with torch on ``device`` (a seeded torch.Generator
    there), for batches too large to build on the host: e.g. the 2^28-element FP64 batch
    of the batched-EVD workload in 6 GB of device memory."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    dt = torch.float64 if kind in "dz" else torch.float32
    lo, hi = (-300, 300) if kind in "dz" else (-40, 40)
    out = []
    for _ in range(4 if kind in "zc" else 3):
        e = torch.randint(lo, hi + 1, (n,), generator=g, device=device, dtype=torch.int32)
        u = torch.rand(n, generator=g, device=device, dtype=dt) + 1.0
        sg = torch.randint(0, 2, (n,), generator=g, device=device, dtype=torch.int32).to(dt) * 2 - 1
        out.append(torch.ldexp(sg * u, e.to(dt)).to(dt))
        del e, u, sg
    return out


def edge2x2(kind, n, seed):
    """2x2 inputs drawn from special values: signed zeros, extremes, subnormals."""
    rng = np.random.default_rng(seed)
    dt = np.float64 if kind in "dz" else np.float32
    fi = np.finfo(dt)
    vals = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, fi.max, -fi.max, fi.max / 3, fi.tiny, -fi.tiny,
                     fi.smallest_subnormal, -fi.smallest_subnormal, fi.tiny / 3, 1e-30, -7e25], dt)
    return [rng.choice(vals, n).astype(dt) for _ in range(4 if kind in "zc" else 3)]


def haar(k, rng, complex_=False):
    A = rng.standard_normal((k, k))
    if complex_:
        A = A + 1j * rng.standard_normal((k, k))
    Q, R = np.linalg.qr(A)
    d = np.diag(R)
    return Q * (d / np.abs(d))


def svd_matrix(m, n, seed, lo=-6.0, complex_=False):
    """A = U diag(sigma) V^H, sigma = 10^U(lo, 0) sorted descending. Returns (A, sigma)."""
    rng = np.random.default_rng(seed)
    U = haar(m, rng, complex_)[:, :n]
    V = haar(n, rng, complex_)
    s = np.sort(10.0 ** rng.uniform(lo, 0.0, n))[::-1]
    return (U * s) @ V.conj().T, s


def graded16():
    i = np.arange(16)[:, None]
    j = np.arange(16)[None, :]
    e = np.where(j < 8, 1023 - j - np.abs(i - j), -51 - j - np.abs(i - j))
    return np.ldexp(1.0, e)


def graded32_f32():
    """The graded16 rule carried to the FP32 exponent range, 32x32 (the FP32 drivers' shape
    rules): columns j < 16: 2^(127-j-|i-j|); j >= 16: 2^(-23-j-|i-j|)."""
    i = np.arange(32)[:, None]
    j = np.arange(32)[None, :]
    e = np.where(j < 16, 127 - j - np.abs(i - j), -23 - j - np.abs(i - j))
    return np.ldexp(1.0, e).astype(np.float32)


def uneven_shapes(count, seed, mmin=16, mmax=512, nmin=8):
    rng = np.random.default_rng(seed)
    m = rng.integers(mmin, mmax + 1, count)
    n = np.array([rng.integers(nmin, mm + 1) for mm in m])
    return m, n


def uneven_batch(count, seed, kind="d", threads=None):
    """The uneven-batch workload with its singular values: m ~ U{16..512}, n ~ U{8..m},
    A = Q1 diag(sigma) Q2^T (Q1, Q2 from QR of Gaussian matrices), sigma = 10^U(-4, 0).
    Returns (matrices, sigmas sorted descending); the matrices are built on host threads."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    m, n = uneven_shapes(count, seed)
    seeds = np.random.default_rng(seed + 1).integers(0, 2 ** 63 - 1, count)
    dt = np.float64 if kind == "d" else np.float32

    def one(i):
        r = np.random.default_rng(int(seeds[i]))
        q1, _ = np.linalg.qr(r.standard_normal((int(m[i]), int(n[i]))))
        q2, _ = np.linalg.qr(r.standard_normal((int(n[i]), int(n[i]))))
        s = np.sort(10.0 ** r.uniform(-4.0, 0.0, int(n[i])))[::-1]
        return ((q1 * s) @ q2.T).astype(dt), s

    with ThreadPoolExecutor(threads or os.cpu_count()) as ex:
        out = list(ex.map(one, range(count)))
    return [a for a, _ in out], [s for _, s in out]
