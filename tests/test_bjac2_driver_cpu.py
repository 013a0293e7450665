"""The 2x2 accuracy drivers t?bjac2.exe (csrc/tbjac2.cpp) on CPU, linked against a
stand-in that forwards ?bjac2_ to the oracle (tests/bjac2_oracle_standin.cpp), whose
results the library's equal bit for bit: the reference's arguments, input files (those
of its generator, src/gen2rand.c), CSV columns and number format, error exits, and the
metrics themselves against a numpy long-double evaluation of the same definitions.

The real executables run on the GPU in tests/test_bjac2_driver_gpu.py and must print the
same metrics as the stand-in.
"""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NUM = re.compile(r"^[ -]\d\.\d{21}E[+-]\d{4}$")


def standin_exes(out):
    from oracle import oracle as O
    from vecjac_gb300 import build
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    # the oracle library resolves through -L/-l and an rpath
    exes = build.build_cli(out_dir=out, link_lib=False, programs=(("tbjac2.cpp", "t%sbjac2.exe"),),
                           extra_sources=[os.path.join(ROOT, "tests", "bjac2_oracle_standin.cpp")],
                           extra_flags=["-L" + libdir, "-lvjo", "-Wl,-rpath," + libdir])
    return dict(zip(build.CLI_KINDS, exes))


@pytest.fixture(scope="module")
def exes(tmp_path_factory):
    return standin_exes(str(tmp_path_factory.mktemp("bjac2drv")))


def gen_files(base, kind, lg, batches, seed):
    """Files in the generator's layout: exact eigenvalues (.k, .l) and the entries of
    U diag(l1, l2) U^H rounded to the precision (.f, .g, .h or .r/.j)."""
    rng = np.random.default_rng(seed)
    dt = np.float64 if kind in "dz" else np.float32
    n = (1 << lg) * batches
    l1 = rng.uniform(-1, 1, n) * 2.0 ** rng.integers(-20, 20, n)
    l2 = rng.uniform(-1, 1, n) * 2.0 ** rng.integers(-20, 20, n)
    phi = rng.uniform(-np.pi / 2, np.pi / 2, n)
    c, s = np.cos(phi).astype(np.longdouble), np.sin(phi).astype(np.longdouble)
    L1, L2 = l1.astype(np.longdouble), l2.astype(np.longdouble)
    a11 = c * c * L1 + s * s * L2
    a22 = s * s * L1 + c * c * L2
    a21 = c * s * (L1 - L2)
    files = {"k": l1, "l": l2, "f": a11, "g": a22}
    if kind in "zc":
        alpha = rng.uniform(0, 2 * np.pi, n)
        files["r"] = a21 * np.cos(alpha).astype(np.longdouble)
        files["j"] = a21 * np.sin(alpha).astype(np.longdouble)
    else:
        files["h"] = a21
    for k, v in files.items():
        np.asarray(v, dtype=np.float64).astype(dt).tofile(base + "." + k)
    return {k: np.asarray(v, dtype=np.float64).astype(dt) for k, v in files.items()}


def metrics(kind, f, j, lg):
    """The driver's metrics of batch j, evaluated with numpy long double from the oracle's
    outputs on the same inputs (no fused multiply-add: agreement to a few units of the
    metric's own rounding)."""
    from oracle import oracle as O
    L = np.longdouble
    n = 1 << lg
    sl = slice(j * n, (j + 1) * n)
    R = O.Restatement()
    if kind in "zc":
        r = R.bjac2(kind, -n, f["f"][sl], f["g"][sl], f["r"][sl], f["j"][sl])
        c, sr, si, l1, l2 = (np.asarray(x).astype(L) for x in r[1:6])
        ar, ai = f["r"][sl].astype(L), f["j"][sl].astype(L)
    else:
        r = R.bjac2(kind, -n, f["f"][sl], f["g"][sl], f["h"][sl])
        c, sr, l1, l2 = (np.asarray(x).astype(L) for x in r[1:5])
        si = np.zeros_like(sr)
        ar, ai = f["h"][sl].astype(L), np.zeros_like(sr)
    s = np.hypot(sr, si)
    a11, a22 = f["f"][sl].astype(L), f["g"][sl].astype(L)
    ort = np.max(np.abs(c * c + s * s - 1))
    d11 = c * c * l1 + s * s * l2 - a11
    d22 = s * s * l1 + c * c * l2 - a22
    d21 = np.hypot((l1 - l2) * c * sr - ar, (l1 - l2) * c * si - ai)
    nrm = lambda x, y, z: np.hypot(np.hypot(x, y), np.sqrt(L(2)) * z)
    ren = np.max(nrm(d11, d22, d21) / nrm(a11, a22, np.hypot(ar, ai)))
    x1, x2 = np.abs(f["k"][sl].astype(L)), np.abs(f["l"][sl].astype(L))
    L1, L2 = np.abs(l1), np.abs(l2)
    Lb, Ls, xb, xs = np.maximum(L1, L2), np.minimum(L1, L2), np.maximum(x1, x2), np.minimum(x1, x2)
    eb, es = np.abs(Lb - xb), np.abs(Ls - xs)
    return ort, ren, np.max(np.hypot(eb, es) / np.hypot(xb, xs)), np.max(eb / xb), np.max(es / xs)


@pytest.mark.parametrize("kind", "dzsc")
def test_driver_output(exes, tmp_path, kind):
    lg, batches = 10, 3
    base = str(tmp_path / ("g" + kind))
    f = gen_files(base, kind, lg, batches, seed=ord(kind))
    r = subprocess.run([exes[kind], base, str(lg), str(batches)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    assert lines[0] == '"B","Ts","ORT","REN","RLN","RLX","RLM"'
    assert len(lines) == 1 + batches
    eps = np.finfo(np.float64 if kind in "dz" else np.float32).eps
    for j, line in enumerate(lines[1:]):
        fields = line.split(",")
        assert len(fields) == 7 and int(fields[0]) == j and float(fields[1]) >= 0
        assert all(NUM.match(x) for x in fields[2:]), fields
        got = [float(x) for x in fields[2:]]
        want = metrics(kind, f, j, lg)
        # orthogonality and residual: a few eps; eigenvalues: within the conditioning of
        # entries rounded to the precision
        assert got[0] <= 8 * eps and got[1] <= 8 * eps, got
        for g, w in zip(got, want):
            assert abs(g - float(w)) <= 0.05 * float(w) + 4 * float(np.finfo(np.longdouble).eps), (got, want)
    if kind in "zc":
        # the worst element of each batch on standard error
        err = [l for l in r.stderr.strip().split("\n") if l]
        assert len(err) == batches and all(l.startswith("%d," % j) for j, l in enumerate(err))


def test_driver_errors(exes, tmp_path):
    base = str(tmp_path / "e")
    gen_files(base, "d", 4, 1, seed=1)
    run = lambda *a: subprocess.run([exes["d"]] + [str(x) for x in a], capture_output=True, text=True, timeout=60)
    assert run(base, 4).returncode == 1                                 # usage
    r = run(base, 2, 1)                                                 # 4 elements: not a multiple of 8
    assert r.returncode == 1 and "multiple of 8" in r.stderr
    r = run(base + "x", 4, 1)
    assert r.returncode == 1 and "Cannot open" in r.stderr
    r = run(base, 4, 0)                                                 # no batches
    assert r.returncode == 0 and r.stdout == ""
    assert run(base, 4, 2).returncode == 1                              # the files hold one batch
    r = subprocess.run([exes["s"], base, "3", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "multiple of 16" in r.stderr           # FP32: 8 elements


def test_real_driver_fails_loudly_without_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from vecjac_gb300 import build
    build.build()
    exe = build.build_cli(programs=(("tbjac2.cpp", "t%sbjac2.exe"),))[0]
    base = str(tmp_path / "n")
    gen_files(base, "d", 4, 1, seed=2)
    r = subprocess.run([exe, base, "4", "1"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "failed in the library" in r.stderr
