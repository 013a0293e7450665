"""Batched SVD of many uneven real matrices in one persistent launch, with an autotuner
for the launch configuration (CTA size and the kernel's register bound, i.e. resident
CTAs per SM) and CUDA-graph capture of the launch.

`svd_batch(mats, kind)` pads every matrix to the reference's shape rules (zero rows and
columns; dvjsvd_/svjsvd_ need m % 8 / % 16 and (n/2) % 8 / % 16), packs all of them into
one device buffer, runs `vj_?vjsvd_batch_dev` once and returns per-matrix results. The
padded shapes are what the reference itself would be given for these matrices, so every
result equals the reference's on the padded matrix.
"""
import ctypes as C
import time

import numpy as np

from . import api

_TUNED = {}
# the library's default register bound (resident 256-thread CTAs per SM) per precision
DEFAULT_OCC = {"s": 4, "d": 2}


def padded_shape(m, n, kind):
    L = 8 if kind == "d" else 16
    n2 = -(-n // (2 * L)) * 2 * L
    m2 = max(-(-m // L) * L, n2)
    return int(m2), int(n2)


class Batch:
    """Device-resident packed batch (torch tensors); `run()` launches the persistent kernel."""

    def __init__(self, mats, kind="d"):
        import torch
        self.kind = kind
        self.dt = torch.float64 if kind == "d" else torch.float32
        shapes = [padded_shape(A.shape[0], A.shape[1], kind) for A in mats]
        self.orig = [A.shape for A in mats]
        self.count = len(mats)
        m = np.array([s[0] for s in shapes], np.int64)
        n = np.array([s[1] for s in shapes], np.int64)
        offG = np.concatenate([[0], np.cumsum(m * n)[:-1]]).astype(np.int64)
        offV = np.concatenate([[0], np.cumsum(n * n)[:-1]]).astype(np.int64)
        offS = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)
        hostG = np.zeros(int((m * n).sum()), np.float64 if kind == "d" else np.float32)
        for A, (mm, nn), o in zip(mats, shapes, offG):
            P = np.zeros((mm, nn), hostG.dtype)
            P[:A.shape[0], :A.shape[1]] = A
            hostG[o:o + mm * nn] = P.reshape(-1, order="F")
        self.m, self.n, self.offG, self.offV, self.offS = m, n, offG, offV, offS
        self.G0 = torch.from_numpy(hostG).cuda()
        self.G = self.G0.clone()
        self.V = torch.zeros(int((n * n).sum()), dtype=self.dt, device="cuda")
        self.eS = torch.zeros(int(n.sum()), dtype=self.dt, device="cuda")
        self.fS = torch.zeros_like(self.eS)
        self.info = torch.zeros(self.count, dtype=torch.int64, device="cuda")
        cost = m.astype(np.float64) * n.astype(np.float64) ** 2
        self.order_np = np.argsort(-cost, kind="stable").astype(np.int32)
        d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        self.dm, self.dn = d(m), d(n)
        self.doffG, self.doffV, self.doffS = d(offG), d(offV), d(offS)
        self.dorder = d(self.order_np)

    def run(self, strategy=4, swp=999, block=128, stream=None, reset=True, occupancy=0):
        """Enqueue the batch (asynchronous). reset=True first restores G from the packed input.
        block: threads per CTA (64, 128, 256); occupancy: the kernel's register bound in
        resident 256-thread CTAs per SM (2..6, 0 = the library's default)."""
        if reset:
            self.G.copy_(self.G0)
        f = getattr(api.lib(), "vj_%svjsvd_batch_tuned_dev" % self.kind)
        f.restype = C.c_longlong
        p = lambda t: C.c_void_p(t.data_ptr())
        r = f(C.c_longlong(self.count), p(self.dm), p(self.dn), p(self.G), p(self.doffG), p(self.V), p(self.doffV),
              p(self.eS), p(self.fS), p(self.doffS), p(self.dorder), C.c_long(strategy), C.c_uint(swp), p(self.info),
              C.c_int(block), C.c_int(occupancy), C.c_void_p(stream) if stream else None)
        if r != 0:
            raise RuntimeError("batched SVD launch failed: %d" % r)

    def results(self):
        """[(info, U, V, eS, fS)] per matrix, in the padded shapes."""
        G = self.G.cpu().numpy()
        V = self.V.cpu().numpy()
        eS = self.eS.cpu().numpy()
        fS = self.fS.cpu().numpy()
        info = self.info.cpu().numpy()
        out = []
        for b in range(self.count):
            mm, nn = int(self.m[b]), int(self.n[b])
            oG, oV, oS = int(self.offG[b]), int(self.offV[b]), int(self.offS[b])
            out.append((int(info[b]), G[oG:oG + mm * nn].reshape((mm, nn), order="F"),
                        V[oV:oV + nn * nn].reshape((nn, nn), order="F"), eS[oS:oS + nn], fS[oS:oS + nn]))
        return out

    def flops(self, sweeps):
        """Algorithmic FLOPs: sweeps * n(n-1)/2 * (12m + 6n) per matrix (sweeps per matrix)."""
        m, n = self.m.astype(np.float64), self.n.astype(np.float64)
        return float(np.sum(np.asarray(sweeps, np.float64) * n * (n - 1) / 2 * (12 * m + 6 * n)))


def autotune(batch, strategy=4, blocks=(64, 128, 256), occupancies=None, sample=None):
    """Pick the launch configuration for this batch's size mix: the CTA size (threads per
    matrix) and the kernel's register bound (resident CTAs per SM), by timing candidates
    on a random sample of the batch's matrices (CUDA events, after one warm-up): first the
    CTA sizes at the default bound, then the bounds at the best CTA size. The sample is
    large enough to fill the GPU several times (2432 matrices by default), so that it
    measures throughput rather than its largest matrix. Returns (block, occupancy); cached
    per (precision, coarse size histogram)."""
    import torch
    if occupancies is None:
        occupancies = (3, 4, 5) if batch.kind == "s" else (2, 3, 4)
    key = (batch.kind, tuple(np.histogram(batch.n, bins=[0, 32, 64, 128, 256, 513])[0] > 0), tuple(blocks),
           tuple(occupancies))
    if key in _TUNED:
        return _TUNED[key]
    rng = np.random.default_rng(0)
    size = min(batch.count, sample or 2432)
    idx = rng.choice(batch.count, size, replace=False)
    mats = []
    G = batch.G0.cpu().numpy()
    for b in idx:
        mm, nn = int(batch.m[b]), int(batch.n[b])
        o = int(batch.offG[b])
        mats.append(G[o:o + mm * nn].reshape((mm, nn), order="F"))
    sub = Batch(mats, batch.kind)

    def timed(blk, occ):
        sub.run(strategy, block=blk, occupancy=occ)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sub.run(strategy, block=blk, occupancy=occ)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    d = DEFAULT_OCC[batch.kind]
    times = {}
    for blk in blocks:
        times[(blk, d)] = timed(blk, d)
    best_blk = min(blocks, key=lambda b_: times[(b_, d)])
    for occ in occupancies:
        if (best_blk, occ) not in times:
            times[(best_blk, occ)] = timed(best_blk, occ)
    best = min(times, key=times.get)
    _TUNED[key] = best
    return best


def capture(batch, strategy=4, swp=999, block=128, occupancy=0):
    """Capture restore-and-run of the batch into a CUDA graph; returns the graph (replay())."""
    import torch
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        batch.run(strategy, swp, block, stream=s.cuda_stream, occupancy=occupancy)   # warm-up outside capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        batch.run(strategy, swp, block, stream=torch.cuda.current_stream().cuda_stream, occupancy=occupancy)
    return g


def svd_batch(mats, kind="d", strategy=4, swp=999, block=None):
    """SVD of every matrix in `mats` (real numpy arrays of any m >= n <= 512) in one launch."""
    import torch
    b = Batch(mats, kind)
    blk, occ = (block, 0) if block else autotune(b, strategy)
    b.run(strategy, swp, blk, occupancy=occ)
    torch.cuda.synchronize()
    return b.results()
