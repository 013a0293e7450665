"""The allocation-free SVD entry point (vj_dvjsvd_dev_noalloc) against the regular one.

Some callers cannot allocate GPU memory while they run (for instance when their own pool
owns the device, or when a cudaMalloc, which can synchronise the device or fail for lack
of memory, is not allowed in the middle of their work); this entry point keeps its scratch
in a fixed array inside the library instead. Two calls in a row
must each give exactly what vj_dvjsvd_dev gives for the same input, which also shows
that the second call does not see the first call's leftovers in the shared array.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_regular(vj, A, sid):
    import torch
    m, n = A.shape
    js, stp = vj.pjs(sid, n)
    G = torch.tensor(A.T.copy(), dtype=torch.float64, device="cuda")
    V = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    eS = torch.zeros(n, dtype=torch.float64, device="cuda")
    fS = torch.zeros(n, dtype=torch.float64, device="cuda")
    dj = torch.tensor(js.astype(np.int32), device="cuda")
    r = vj.vjsvd_dev("d", m, n, G, m, V, n, eS, fS, dj, stp)
    torch.cuda.synchronize()
    return r, G.cpu().numpy(), V.cpu().numpy(), eS.cpu().numpy(), fS.cpu().numpy()


def _run_noalloc(vj, A, sid):
    import torch
    lib = vj.lib()
    f = lib.vj_dvjsvd_dev_noalloc
    f.restype = C.c_longlong
    m, n = A.shape
    G = torch.tensor(A.T.copy(), dtype=torch.float64, device="cuda")
    V = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    eS = torch.zeros(n, dtype=torch.float64, device="cuda")
    fS = torch.zeros(n, dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    r = f(C.c_ulonglong(m), C.c_ulonglong(n), p(G), C.c_ulonglong(m), p(V), C.c_ulonglong(n), p(eS), p(fS),
          C.c_long(sid), C.c_uint(999), C.c_int(0), None)
    torch.cuda.synchronize()
    return r, G.cpu().numpy(), V.cpu().numpy(), eS.cpu().numpy(), fS.cpu().numpy()


def test_noalloc_matches_regular_twice():
    import vecjac_gb300 as vj
    from vecjac_gb300 import build
    from vecjac_gb300 import workloads as W
    build.build()
    cases = [(W.svd_matrix(256, 128, seed=31)[0], 4), (W.svd_matrix(128, 96 + 32, seed=32)[0], 2)]
    for A, sid in cases:
        ra = _run_regular(vj, A, sid)
        rb = _run_noalloc(vj, A, sid)
        assert rb[0] == ra[0] and rb[0] > 0
        for x, y in zip(ra[1:], rb[1:]):
            assert np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_noalloc_rejects_large_n():
    import torch
    import vecjac_gb300 as vj
    lib = vj.lib()
    f = lib.vj_dvjsvd_dev_noalloc
    f.restype = C.c_longlong
    n = 528
    G = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    r = f(C.c_ulonglong(n), C.c_ulonglong(n), C.c_void_p(G.data_ptr()), C.c_ulonglong(n), C.c_void_p(G.data_ptr()),
          C.c_ulonglong(n), C.c_void_p(G.data_ptr()), C.c_void_p(G.data_ptr()), C.c_long(4), C.c_uint(1), C.c_int(0),
          None)
    assert r == vj.VJ_ERR_ARG
