"""Differentiable batched SVD: torch.autograd.Function over the C ABI (ctypes).

Forward: `vj_?vjsvd_batch_dev` (one persistent launch for the whole batch of same-shape
matrices; FP32 svjsvd_ / FP64 dvjsvd_ per matrix), then singular values sorted in
descending order and every (u_j, v_j) pair sign-fixed so that the largest-magnitude entry
of v_j is positive (a locally constant choice, so finite differences see the same branch).
Backward: `vj_?svd_adjoint_batch_dev`, the hand-written adjoint kernel, with the gap-safe
1/(s_j^2 - s_i^2) terms.

`svd_k(A, k)` returns (S, U_k, V_k) with A (B, m, n) on the GPU, m >= n, and the
reference's shape rules (FP32: m % 16 == 0, (n/2) % 16 == 0; FP64: % 8). This is a test
and measurement facility for the adjoint; no CPU path exists.
"""
import ctypes as C

import numpy as np

from . import api


def _p(t):
    return C.c_void_p(t.data_ptr())


_BLOCK = {}


def _tuned_block(A, strategy, swp):
    """Launch configuration of the batched kernel for this matrix shape and precision: the
    CTA size (64, 128, 256 threads) at the default register bound, then the register bound
    (resident 256-thread CTAs per SM) at the best size, each timed on up to 2432 of the
    matrices (after one warm-up); the fastest (block, occupancy) is kept for the process."""
    import torch
    key = (tuple(A.shape[1:]), A.dtype, strategy)
    if key not in _BLOCK:
        sub = A[: min(A.shape[0], 2432)]

        def timed(blk, occ):
            svd_batch_dev(sub, strategy, swp, block=(blk, occ))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            svd_batch_dev(sub, strategy, swp, block=(blk, occ))
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

        d = 4 if A.dtype == torch.float32 else 2
        times = {(blk, d): timed(blk, d) for blk in (64, 128, 256)}
        best_blk = min((64, 128, 256), key=lambda b: times[(b, d)])
        for occ in ((3, 4, 5) if A.dtype == torch.float32 else (2, 3, 4)):
            if (best_blk, occ) not in times:
                times[(best_blk, occ)] = timed(best_blk, occ)
        _BLOCK[key] = min(times, key=times.get)
    return _BLOCK[key]


def svd_batch_dev(A, strategy=4, swp=999, block=None):
    """SVD of every matrix of A (B, m, n) CUDA tensor (float32 or float64) in one launch
    (block: threads per CTA, or (threads, register bound in resident 256-thread CTAs per
    SM); None = autotuned per shape). Returns (S (B, n), U (B, m, n), V (B, n, n),
    sweeps (B,)) unsorted, as the kernel leaves them."""
    import torch
    if block is None:
        block = _tuned_block(A, strategy, swp)
    block, occ = block if isinstance(block, tuple) else (block, 0)
    Bn, m, n = A.shape
    kind = "s" if A.dtype == torch.float32 else "d"
    L = 16 if kind == "s" else 8
    if m < n or m % L or n % 2 or (n // 2) % L:
        raise ValueError("shape %dx%d breaks the %svjsvd_ rules" % (m, n, kind))
    dev = A.device
    G = A.transpose(1, 2).contiguous()          # column-major m x n per matrix
    V = torch.empty((Bn, n, n), dtype=A.dtype, device=dev)
    eS = torch.empty((Bn, n), dtype=A.dtype, device=dev)
    fS = torch.empty_like(eS)
    info = torch.empty(Bn, dtype=torch.int64, device=dev)
    mm = torch.full((Bn,), m, dtype=torch.int64, device=dev)
    nn = torch.full((Bn,), n, dtype=torch.int64, device=dev)
    ar = torch.arange(Bn, dtype=torch.int64, device=dev)
    offG, offV, offS = ar * (m * n), ar * (n * n), ar * n
    f = getattr(api.lib(), "vj_%svjsvd_batch_tuned_dev" % kind)
    stream = torch.cuda.current_stream().cuda_stream
    r = f(C.c_longlong(Bn), _p(mm), _p(nn), _p(G), _p(offG), _p(V), _p(offV), _p(eS), _p(fS), _p(offS), None,
          C.c_long(strategy), C.c_uint(swp), _p(info), C.c_int(block), C.c_int(occ), C.c_void_p(stream))
    if r != 0:
        raise RuntimeError("batched SVD launch failed: %d" % r)
    S = fS * torch.exp2(eS)
    # G holds U column-major (n, m) per matrix; V is column-major too
    return S, G.transpose(1, 2), V.transpose(1, 2), info


def _sort_and_fix(S, U, V):
    import torch
    S, idx = torch.sort(S, dim=1, descending=True)
    U = torch.gather(U, 2, idx[:, None, :].expand_as(U))
    V = torch.gather(V, 2, idx[:, None, :].expand_as(V))
    piv = torch.argmax(V.abs(), dim=1, keepdim=True)
    sgn = torch.sign(torch.gather(V, 1, piv))
    sgn = torch.where(sgn == 0, torch.ones_like(sgn), sgn)
    return S, U * sgn, V * sgn


def adjoint(U, S, V, dS, dUk, dVk, gap=0.0):
    """dA (B, m, n) from the adjoint kernel; U (B, m, n), V (B, n, n), dUk (B, m, k), dVk (B, n, k)."""
    import torch
    Bn, m, n = U.shape
    k = dUk.shape[2]
    kind = "s" if U.dtype == torch.float32 else "d"
    cm = lambda t: t.transpose(1, 2).contiguous()
    Uc, Vc, dUc, dVc = cm(U), cm(V), cm(dUk), cm(dVk)
    Sc, dSc = S.contiguous(), dS.contiguous()
    dA = torch.empty((Bn, n, m), dtype=U.dtype, device=U.device)
    f = getattr(api.lib(), "vj_%ssvd_adjoint_batch_dev" % kind)
    ft = C.c_float if kind == "s" else C.c_double
    r = f(C.c_longlong(Bn), C.c_ulonglong(m), C.c_ulonglong(n), C.c_ulonglong(k), _p(Uc), _p(Sc), _p(Vc), _p(dSc),
          _p(dUc), _p(dVc), _p(dA), ft(gap), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if r != 0:
        raise RuntimeError("SVD adjoint launch failed: %d" % r)
    return dA.transpose(1, 2)


def _function():
    import torch

    class BatchedSVD(torch.autograd.Function):
        @staticmethod
        def forward(ctx, A, k, gap):
            S, U, V, _ = svd_batch_dev(A.detach())
            S, U, V = _sort_and_fix(S, U, V)
            ctx.save_for_backward(U, S, V)
            ctx.k, ctx.gap = k, gap
            return S, U[:, :, :k].contiguous(), V[:, :, :k].contiguous()

        @staticmethod
        def backward(ctx, dS, dUk, dVk):
            U, S, V = ctx.saved_tensors
            z = lambda t, shape: torch.zeros(shape, dtype=U.dtype, device=U.device) if t is None else t
            dS = z(dS, S.shape)
            dUk = z(dUk, (U.shape[0], U.shape[1], ctx.k))
            dVk = z(dVk, (V.shape[0], V.shape[1], ctx.k))
            return adjoint(U, S, V, dS, dUk, dVk, ctx.gap), None, None

    return BatchedSVD


_FN = None


def svd_k(A, k, gap=0.0):
    """(S, U_k, V_k) of every matrix in A (B, m, n), differentiable through the adjoint kernel."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(A, int(k), float(gap))


def spaced_sigma_matrices(count, m, n, seed, lo=0.1, hi=10.0, min_gap=1e-3, dtype=np.float64):
    """The differentiable-batch workload: A = Q1 diag(s) Q2^T with Q1, Q2 Haar (QR of seeded
    Gaussians) and s drawn uniform in [lo, hi], redrawn until every relative gap between
    neighbouring singular values is >= min_gap. Returns (A (count, m, n), s (count, n))."""
    rng = np.random.default_rng(seed)
    A = np.empty((count, m, n), dtype)
    Ss = np.empty((count, n))
    for b in range(count):
        while True:
            s = np.sort(rng.uniform(lo, hi, n))[::-1]
            if np.all((s[:-1] - s[1:]) / s[:-1] >= min_gap):
                break
        q1, r1 = np.linalg.qr(rng.standard_normal((m, n)))
        q1 *= np.sign(np.diag(r1))
        q2, r2 = np.linalg.qr(rng.standard_normal((n, n)))
        q2 *= np.sign(np.diag(r2))
        A[b] = (q1 * s) @ q2.T
        Ss[b] = s
    return A, Ss
