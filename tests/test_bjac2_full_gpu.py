"""The batched 2x2 EVD at the benchmark's full sizes (2^28 real, 2^27 complex elements per
launch), through size-independent properties (tests/props2x2.py): orthogonality of every
rotation within 8 eps, residual ||A - U diag(l1, l2) U^H||_F / ||A||_F within 12 eps,
permutation bits equal to (l1 < l2) wherever l1 != l2; and 4096 whole lane groups drawn
at random from each full-size launch, bit for bit against the oracle on the same inputs
(the whole batch would take the oracle minutes; the same bounds hold for the oracle's own
outputs, tests/test_bjac2_props_cpu.py).
"""
import numpy as np
import pytest

from props2x2 import props2x2

pytestmark = [pytest.mark.gpu, pytest.mark.late]


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


@pytest.mark.parametrize("kind,lg", [("d", 28), ("s", 28), ("z", 27), ("c", 27)])
@pytest.mark.parametrize("sgn", [-1, 1])
def test_full_size_properties(vj, kind, lg, sgn):
    import torch
    from vecjac_gb300 import workloads as W
    n = 1 << lg
    lanes = 8 if kind in "dz" else 16
    dt = torch.float64 if kind in "dz" else torch.float32
    ins = W.pairs2x2_torch(kind, n, seed=lg + ord(kind) + sgn, device="cuda")
    outs = [torch.empty(n, dtype=dt, device="cuda") for _ in range(5 if kind in "zc" else 4)]
    p = torch.zeros(n // lanes, dtype=torch.int32, device="cuda")
    if kind in "zc":
        r = vj.bjac2_dev(kind, sgn * n, ins[0], ins[1], ins[2], ins[3], *outs, p)
        c, t, ti, l1, l2 = outs
        a21i = ins[3]
    else:
        r = vj.bjac2_dev(kind, sgn * n, ins[0], ins[1], ins[2], None, outs[0], outs[1], None, outs[2], outs[3], p)
        c, t, l1, l2 = outs
        a21i = ti = torch.zeros(1, dtype=dt, device="cuda").expand(n)
    torch.cuda.synchronize()
    assert r == 1
    o, res, bad, count = props2x2(kind, sgn, ins[0], ins[1], ins[2], a21i, c, t, ti, l1, l2, p)
    assert count == n
    assert o <= 8.0 and res <= 12.0 and bad == 0, (o, res, bad)
    # a random sample of whole lane groups of the full-size launch, bit for bit
    from oracle import oracle as O
    O.build()
    g = np.sort(np.random.default_rng(lg + ord(kind)).choice(n // lanes, 4096, replace=False))
    idx = (g[:, None] * lanes + np.arange(lanes)[None, :]).reshape(-1)
    it = torch.tensor(idx, device="cuda")
    take = lambda x: x[it].cpu().numpy()
    sample_in = [take(x) for x in ins[:(4 if kind in "zc" else 3)]]
    ro = O.Restatement().bjac2(kind, sgn * len(idx), *sample_in)
    got = [take(x) for x in outs] + [p[torch.tensor(g, device="cuda")].cpu().numpy().view(np.uint32)]
    for x, y in zip(got, ro[1:]):
        assert np.array_equal(np.ascontiguousarray(x).view(np.uint8), np.ascontiguousarray(y).view(np.uint8))
    del ins, outs, p
    torch.cuda.empty_cache()
