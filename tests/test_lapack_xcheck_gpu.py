"""The GPU SVD against LAPACK xGESVJ (oracle/lapack.py) at sizes the CPU restatement takes
long for: the same bounds as the CPU cross-check (plain: 4 n eps s_max absolute; graded
over 12 (FP64) / 5 (FP32) decades: 4 n eps relative on every singular value).
"""
import numpy as np
import pytest

from oracle import lapack as LA
from test_lapack_xcheck_cpu import check, graded, sigma_of

pytestmark = [pytest.mark.gpu, pytest.mark.late,
              pytest.mark.skipif(not LA.available(), reason="no LAPACK with xGESVJ in this numpy/scipy")]


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


@pytest.mark.parametrize("kind,m,n,grade", [("d", 512, 256, False), ("d", 512, 256, True), ("z", 256, 128, True),
                                            ("s", 512, 256, True), ("c", 256, 128, True)])
def test_gpu_vs_gesvj(vj, kind, m, n, grade):
    from vecjac_gb300 import api
    from vecjac_gb300 import workloads as W
    A = graded(kind, m, n, 11) if grade else W.svd_matrix(m, n, seed=13, complex_=(kind in "zc"))[0]
    js, stp = api.pjs(4, n)
    r = vj.vjsvd(kind, A.real, js, stp, **(dict(Gi=A.imag) if kind in "zc" else {}))
    assert r[0] > 0
    info, s_l, *_ = LA.gesvj(kind, A)
    assert info == 0
    check(kind, n, sigma_of(r[3], r[4]), s_l, grade)
