"""The command-line drivers t?vjsvd.exe (csrc/tvjsvd.cpp) on CPU, linked against a stub
of the library (tests/cli_stub.cpp) that writes known patterns: argument handling and exit
codes as in the reference's src/t?vjsvd.c, the raw column-major files of src/mtxio.c with
padded leading dimensions, complex split/merge, the CSV line, and the two encodings of the
reference's `wide` singular values -- binary128 checked against an exact decoding and
against gcc's __float128, x87 extended against this host's long double.

The real executables (linked against libvecjac_gb300.so) are run on the GPU in
tests/test_cli_gpu.py; here they are only checked to fail loudly without a GPU.
"""
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "tests", "cli_stub.cpp")
SVD_DRIVER = (("tvjsvd.cpp", "t%svjsvd.exe"),)
KINDS = {"d": (np.float64, False, 8), "z": (np.float64, True, 8), "s": (np.float32, False, 16),
         "c": (np.float32, True, 16)}


@pytest.fixture(scope="module")
def stub_exes(tmp_path_factory):
    from vecjac_gb300 import build
    out = str(tmp_path_factory.mktemp("cli"))
    exes = build.build_cli(out_dir=out, extra_sources=[STUB], link_lib=False, programs=SVD_DRIVER)
    return dict(zip(build.CLI_KINDS, exes))


def shape(kind):
    # m not a multiple of the vector length: the drivers pad the leading dimension
    return (36, 16) if KINDS[kind][0] == np.float64 else (40, 32)


def make_input(d, kind, seed=0):
    from vecjac_gb300 import mtxio
    dt, cplx, _ = KINDS[kind]
    m, n = shape(kind)
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((m, n)).astype(dt)
    if cplx:
        G = (G + 1j * rng.standard_normal((m, n)).astype(dt)).astype(np.complex128 if dt == np.float64 else np.complex64)
    base = os.path.join(d, "mat_" + kind)
    mtxio.write_matrix(base + ".G", G)
    return base, G, m, n


def run(exe, *args, env=None):
    return subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=60,
                          env=dict(os.environ, **(env or {})))


def expected_sigma(kind, n):
    """The stub's (eS, fS) pattern as exact values."""
    dt = KINDS[kind][0]
    rng_ = 2000 if dt == np.float64 else 200
    out = []
    for j in range(n):
        f = Fraction(1) + Fraction((j * 2654435761) % (1 << 20), 1 << 20)
        if j == 0:
            out.append(Fraction(0))
        elif j == 1:
            out.append(f)
        else:
            e = (j * 37) % rng_ - rng_ // 2
            out.append(f * Fraction(2) ** e)
    return out


def decode_q_exact(b):
    x = int.from_bytes(bytes(b), "little")
    s, e, f = x >> 127, (x >> 112) & 0x7FFF, x & ((1 << 112) - 1)
    assert e != 0x7FFF
    v = Fraction(0) if (e == 0 and f == 0) else Fraction((1 << 112) | f) * Fraction(2) ** (e - 16383 - 112)
    return -v if s else v


@pytest.mark.parametrize("kind", "dzsc")
@pytest.mark.parametrize("J", [2, 4])
def test_outputs(stub_exes, tmp_path, kind, J):
    from vecjac_gb300 import mtxio
    dt, cplx, _ = KINDS[kind]
    base, G, m, n = make_input(str(tmp_path), kind)
    # stale, longer output files are cut to size
    for ext in ("U", "V", "S"):
        with open("%s.%s%d" % (base, ext, J), "wb") as f:
            f.write(b"\xff" * (20 * m * n))
    r = run(stub_exes[kind], J, m, n, base)
    assert r.returncode == 0, (r.returncode, r.stderr)
    f = r.stdout.strip().split(",")
    assert f[0] == '"%s"' % base and int(f[1]) == J and int(f[2]) == m and int(f[3]) == n
    if cplx:
        assert len(f) == 9 and int(f[6]) == 9 and all(float(f[k]) >= 0 for k in (4, 5, 7, 8))
    else:
        assert len(f) == 6 and int(f[5]) == 7 and float(f[4]) >= 0
    cdt = G.dtype
    U = mtxio.read_matrix("%s.U%d" % (base, J), m, n, cdt)
    V = mtxio.read_matrix("%s.V%d" % (base, J), n, n, cdt)
    col = np.arange(n, dtype=dt)[None, :]
    if cplx:
        assert np.array_equal(U.real, (2 * G.real + col).astype(dt))
        assert np.array_equal(U.imag, (dt(0.5) - G.imag).astype(dt))
    else:
        assert np.array_equal(U, (2 * G + col).astype(dt))
    Vx = (1000 * np.arange(n)[:, None] + np.arange(n)[None, :]).astype(dt)
    assert np.array_equal(V.real if cplx else V, Vx)
    if cplx:
        assert np.array_equal(V.imag, -Vx)
    raw = np.fromfile("%s.S%d" % (base, J), dtype=np.uint8)
    assert raw.size == 16 * n
    want = expected_sigma(kind, n)
    assert [decode_q_exact(raw[16 * i:16 * i + 16]) for i in range(n)] == want
    S = mtxio.read_wide("%s.S%d" % (base, J), n)
    assert np.array_equal(S, np.array([float(w) for w in want]))


def test_x87_extended(stub_exes, tmp_path):
    from vecjac_gb300 import mtxio
    if np.finfo(np.longdouble).nmant != 63:
        pytest.skip("this host's long double is not the x87 format")
    base, G, m, n = make_input(str(tmp_path), "d")
    r = run(stub_exes["d"], 2, m, n, base, env={"VJ_WIDE": "l"})
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(base + ".S2", dtype=np.uint8)
    for i in range(n):
        f = 0.0 if i == 0 else 1 + ((i * 2654435761) % (1 << 20)) / (1 << 20)
        e = 0 if i < 2 else (i * 37) % 2000 - 1000
        ld = np.ldexp(np.longdouble(f), e)
        assert bytes(raw[16 * i:16 * i + 10]) == ld.tobytes()[:10], i
        assert bytes(raw[16 * i + 10:16 * i + 16]) == bytes(6)
    assert np.array_equal(mtxio.read_wide(base + ".S2", n, "l"), np.array([float(w) for w in expected_sigma("d", n)]))


def test_binary128_matches_gcc(stub_exes, tmp_path):
    # gcc's __float128 of the same values, built by exact scaling
    src = tmp_path / "q.c"
    src.write_text("""
        #include <stdio.h>
        #include <string.h>
        int main(void) {
          double f; int e;
          while (scanf("%lf %d", &f, &e) == 2) {
            __float128 q = (__float128)f;
            for (; e > 0; --e) q *= 2;
            for (; e < 0; ++e) q /= 2;
            unsigned char b[16]; memcpy(b, &q, 16);
            for (int k = 0; k < 16; ++k) printf("%02x", b[k]);
            printf("\\n");
          }
          return 0;
        }""")
    exe = tmp_path / "q"
    c = subprocess.run(["gcc", "-O0", str(src), "-o", str(exe)], capture_output=True, text=True)
    if c.returncode != 0:
        pytest.skip("no __float128 in this host's gcc")
    base, G, m, n = make_input(str(tmp_path), "d")
    assert run(stub_exes["d"], 2, m, n, base).returncode == 0
    raw = np.fromfile(base + ".S2", dtype=np.uint8)
    lines = []
    for j in range(n):
        f = 1 + ((j * 2654435761) % (1 << 20)) / (1 << 20)
        e = 0 if j == 1 else ((j * 37) % 2000 - 1000)
        lines.append("%r %d" % (0.0 if j == 0 else f, e))
    q = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [bytes(raw[16 * i:16 * i + 16]).hex() for i in range(n)]
    assert got == q.stdout.split()


def test_exit_codes(stub_exes, tmp_path):
    base, G, m, n = make_input(str(tmp_path), "d")
    exe = stub_exes["d"]
    assert run(exe).returncode == 1
    assert run(exe, 2, m, n).returncode == 1
    assert run(exe, 3, m, n, base).returncode == 2         # only strategies 2 and 4
    assert run(exe, 2, 0, n, base).returncode == 3
    assert run(exe, 2, "36x", n, base).returncode == 3     # trailing characters
    assert run(exe, 2, m, 0, base).returncode == 4
    assert run(exe, 2, m, 15, base).returncode == 4        # odd
    assert run(exe, 2, m, 48, base).returncode == 4        # n > m
    assert run(exe, 2, 64, 24, base).returncode == 4       # (n/2) % 8
    assert run(exe, 2, m, n, "").returncode == 5
    assert run(exe, 2, m, n, base + "_missing").returncode == 5
    assert run(exe, 2, m + 4, n, base).returncode == 5     # file shorter than (m+4) n entries
    assert run(exe, 2, "0x24", "0x10", base).returncode == 0   # strtoull base detection
    # FP32: (n/2) % 16
    base_s, _, ms, ns = make_input(str(tmp_path), "s")
    assert run(stub_exes["s"], 2, ms, 16, base_s).returncode == 4


def test_real_driver_fails_loudly_without_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from vecjac_gb300 import build
    build.build()
    exes = build.build_cli(programs=SVD_DRIVER)
    base, G, m, n = make_input(str(tmp_path), "d")
    r = run(exes[0], 2, m, n, base)
    assert r.returncode != 0
    assert "GPU" in r.stderr
    assert not os.path.exists(base + ".U2")
