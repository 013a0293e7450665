"""The command-line drivers t?vjsvd.exe with the real library on the GPU: for each
precision, the files the driver writes are the host entry point's results on the same
input and pivot table, bit for bit (U and V in the drivers' raw layout, sigma decoded from
the binary128 file equal to fS 2^eS), and the CSV line carries the same return value.
A row count that is not a multiple of the vector length is passed through to the
library, which rejects it with -1 as the reference does; the driver still writes its
files, as the reference's does.

The driver runs as a second process on the GPU this test process already uses; under an
exclusive compute mode that is impossible and the test is skipped.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.late]

CASES = [("d", 64, 32, 2), ("z", 64, 32, 4), ("s", 64, 32, 2), ("c", 64, 32, 4)]


@pytest.fixture(scope="module")
def env():
    import vecjac_gb300
    from vecjac_gb300 import build
    build.build()
    exes = dict(zip(build.CLI_KINDS, build.build_cli(programs=(("tvjsvd.cpp", "t%svjsvd.exe"),))))
    try:
        mode = subprocess.run(["nvidia-smi", "--query-gpu=compute_mode", "--format=csv,noheader", "-i", "0"],
                              capture_output=True, text=True, timeout=60).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        mode = ""
    if mode and mode != "Default":
        pytest.skip("compute mode %s: a second process cannot use the GPU" % mode)
    return vecjac_gb300, exes


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("kind,m,n,J", CASES)
def test_driver_matches_host_entry(env, tmp_path, kind, m, n, J):
    from vecjac_gb300 import api, mtxio
    from vecjac_gb300 import workloads as W
    vj, exes = env
    cplx = kind in "zc"
    dt = np.float64 if kind in "dz" else np.float32
    A, _ = W.svd_matrix(m, n, seed=m + n + ord(kind), complex_=cplx)
    Ar, Ai = A.real.astype(dt), (A.imag.astype(dt) if cplx else None)
    base = str(tmp_path / ("m" + kind))
    G = (Ar + 1j * Ai).astype(np.complex128 if dt == np.float64 else np.complex64) if cplx else Ar
    mtxio.write_matrix(base + ".G", G)
    r = subprocess.run([exes[kind], str(J), str(m), str(n), base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr)
    f = r.stdout.strip().split(",")
    info = int(f[6] if cplx else f[5])
    js, stp = api.pjs(J, n)
    ref = vj.vjsvd(kind, Ar, js, stp, **(dict(Gi=Ai) if cplx else {}))
    assert info == ref[0] and info > 0
    U = mtxio.read_matrix("%s.U%d" % (base, J), m, n, G.dtype)
    V = mtxio.read_matrix("%s.V%d" % (base, J), n, n, G.dtype)
    if cplx:
        assert same(np.ascontiguousarray(U.real), np.ascontiguousarray(ref[1])) and same(
            np.ascontiguousarray(U.imag), np.ascontiguousarray(ref[5]))
        assert same(np.ascontiguousarray(V.real), np.ascontiguousarray(ref[2])) and same(
            np.ascontiguousarray(V.imag), np.ascontiguousarray(ref[6]))
    else:
        assert same(np.ascontiguousarray(U), np.ascontiguousarray(ref[1]))
        assert same(np.ascontiguousarray(V), np.ascontiguousarray(ref[2]))
    S = mtxio.read_wide("%s.S%d" % (base, J), n)
    eS, fS = ref[3].astype(np.float64), ref[4].astype(np.float64)
    want = np.where(np.isneginf(eS), 0.0, np.ldexp(fS, np.where(np.isfinite(eS), eS, 0).astype(np.int64)))
    assert np.array_equal(S, want)


def test_driver_passes_the_library_error_through(env, tmp_path):
    from vecjac_gb300 import mtxio
    _, exes = env
    m, n = 36, 16   # 36 % 8 != 0: the reference's -1
    base = str(tmp_path / "bad")
    mtxio.write_matrix(base + ".G", np.random.default_rng(1).standard_normal((m, n)))
    r = subprocess.run([exes["d"], "2", str(m), str(n), base], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert int(r.stdout.strip().split(",")[5]) == -1
    assert os.path.getsize(base + ".U2") == m * n * 8 and os.path.getsize(base + ".S2") == n * 16
