"""The 2x2 host entry points with page-locked output arrays.

When every output array is page-locked host memory (and the GPU reads host memory in
place), ?bjac2_ runs one launch that reads the inputs and writes the outputs over the
host link, with no staging copies. Its results must be those of the staged path bit for
bit, for every kind and both signs of n.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


def pinned(n, dt):
    import torch
    tdt = {np.float64: torch.float64, np.float32: torch.float32, np.uint32: torch.int32}[dt]
    return torch.zeros(n, dtype=tdt, pin_memory=True).numpy().view(dt)


@pytest.mark.parametrize("kind", ["d", "z", "s", "c"])
@pytest.mark.parametrize("sign", [1, -1])
def test_pinned_outputs_match_pageable(vj, kind, sign):
    from vecjac_gb300 import workloads as W
    n = 1 << 18
    ins = W.pairs2x2(kind, n, seed=5 + (sign > 0))
    ref = vj.bjac2(kind, sign * n, *ins)
    dt = np.float64 if kind in "dz" else np.float32
    lanes = 8 if kind in "dz" else 16
    outs = dict(c=pinned(n, dt), at=pinned(n, dt), l1=pinned(n, dt), l2=pinned(n, dt), p=pinned(n // lanes, np.uint32))
    if kind in "zc":
        outs["sat"] = pinned(n, dt)
    got = vj.bjac2(kind, sign * n, *ins, **outs)
    assert got[0] == ref[0] == 1
    for x, y in zip(got[1:], ref[1:]):
        assert np.array_equal(np.ascontiguousarray(x).view(np.uint8), np.ascontiguousarray(y).view(np.uint8))
