"""Host-pointer entry points called from several host threads at once.

The reference's routines share nothing between calls (apart from its trace file), so a
caller may run them on several threads. This library's host forms share the device's
staging buffers and streams, and take a per-device lock around them: concurrent calls
must give exactly the results of the same calls made one after another. ctypes releases
the GIL for the duration of each foreign call, so the threads below are inside the
library at the same time.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = 4


@pytest.fixture(scope="module")
def vj():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    return vecjac_gb300


def run_threads(fns):
    out = [None] * len(fns)
    err = []

    def body(i):
        try:
            out[i] = fns[i]()
        except Exception as e:  # reported after the join
            err.append(e)

    ts = [threading.Thread(target=body, args=(i,)) for i in range(len(fns))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not err, err
    return out


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("kind", ["d", "z", "s", "c"])
def test_bjac2_concurrent(vj, kind):
    dt = np.float64 if kind in "dz" else np.float32
    n = 1 << 16
    ins = []
    for t in range(THREADS):
        rng = np.random.default_rng(100 + t)
        e = rng.integers(-30, 31, size=(4, n))
        u = 1.0 + rng.random((4, n))
        s = np.where(rng.random((4, n)) < 0.5, -1.0, 1.0)
        ins.append((s * u * np.exp2(e)).astype(dt))

    def call(x):
        if kind in "zc":
            return vj.bjac2(kind, -n, x[0], x[1], x[2], x[3])
        return vj.bjac2(kind, -n, x[0], x[1], x[2])

    serial = [call(x) for x in ins]
    for _ in range(3):
        conc = run_threads([lambda x=x: call(x) for x in ins])
        for s_, c_ in zip(serial, conc):
            assert s_[0] == c_[0] == 1
            for a, b in zip(s_[1:], c_[1:]):
                assert same(a, b)


def test_dvjsvd_concurrent(vj):
    m, n = 128, 64
    js, stp = vj.pjs(4, n)
    mats = []
    for t in range(THREADS):
        rng = np.random.default_rng(200 + t)
        q1, _ = np.linalg.qr(rng.standard_normal((m, n)))
        q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
        mats.append((q1 * np.logspace(0, -6, n)) @ q2.T)
    serial = [vj.vjsvd("d", A, js, stp) for A in mats]
    conc = run_threads([lambda A=A: vj.vjsvd("d", A, js, stp) for A in mats])
    for s_, c_ in zip(serial, conc):
        assert s_[0] == c_[0] and s_[0] >= 0
        for a, b in zip(s_[1:], c_[1:]):
            assert same(a, b)


def test_zsplit_concurrent(vj):
    m, n = 256, 48
    ins = []
    for t in range(THREADS):
        rng = np.random.default_rng(300 + t)
        ins.append(np.asfortranarray(rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))))
    from vecjac_gb300 import api
    serial = [api.split("z", A) for A in ins]
    conc = run_threads([lambda A=A: api.split("z", A) for A in ins])
    for s_, c_ in zip(serial, conc):
        assert s_[0] == c_[0] == 1
        for a, b in zip(s_[1:], c_[1:]):
            assert same(a, b)
