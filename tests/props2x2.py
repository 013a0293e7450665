"""Size-independent properties of a batch of 2x2 Hermitian eigendecompositions (the
quantities the reference's 2x2 accuracy drivers report through src/wnrme.c), evaluated in
FP64 with torch on whatever device the tensors live on, in chunks.

For A = [[a11, conj(a21)], [a21, a22]] and the outputs (c, s, l1, l2, p), with s the sine
(n < 0) or c times the tangent (n > 0), complex s = re + i im:
  U = [[c, -conj(s)], [s, c]],   A = U diag(l1, l2) U^H
  orthogonality  |c^2 + |s|^2 - 1|                           / eps
  residual       ||A - U diag(l1, l2) U^H||_F / ||A||_F       / eps
  permutation    bit (i mod L) of p[i / L] == (l1 < l2) wherever l1 != l2
Returns (max orthogonality / eps, max residual / eps, permutation mismatches, count).
"""


def props2x2(kind, sgn, a11, a22, a21, a21i, c, t, ti, l1, l2, p, chunk=1 << 24):
    import torch
    eps = torch.finfo(torch.float64 if kind in "dz" else torch.float32).eps
    lanes = 8 if kind in "dz" else 16
    n = a11.numel()
    worst_o, worst_r, bad = 0.0, 0.0, 0
    shifts = torch.arange(lanes, device=p.device, dtype=torch.int64)
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        f = lambda x: x[lo:hi].to(torch.float64)
        A11, A22, C, L1, L2 = f(a11), f(a22), f(c), f(l1), f(l2)
        cplx = kind in "zc"
        A21 = torch.complex(f(a21), f(a21i)) if cplx else torch.complex(f(a21), torch.zeros_like(A11))
        S = torch.complex(f(t), f(ti)) if cplx else torch.complex(f(t), torch.zeros_like(A11))
        if sgn > 0:
            S = S * C
        orth = (C * C + S.abs() ** 2 - 1).abs()
        # U = [[C, -conj(S)], [S, C]]
        r11 = A11 - (C * L1 * C + (S.abs() ** 2) * L2)
        r22 = A22 - ((S.abs() ** 2) * L1 + C * L2 * C)
        r21 = A21 - (S * L1 * C - C * L2 * S)
        nrm = torch.sqrt(A11 ** 2 + A22 ** 2 + 2 * A21.abs() ** 2)
        res = torch.sqrt(r11 ** 2 + r22 ** 2 + 2 * r21.abs() ** 2) / nrm
        worst_o = max(worst_o, float(orth.max()) / eps)
        worst_r = max(worst_r, float(res.max()) / eps)
        words = p[lo // lanes:hi // lanes].to(torch.int64)
        bits = ((words[:, None] >> shifts[None, :]) & 1).reshape(-1).to(torch.bool)
        neq = L1 != L2
        bad += int((bits[neq] != (L1 < L2)[neq]).sum())
    return worst_o, worst_r, bad, n
