"""The pair rotation of the mixed SVD's plain-dot FP64 sweeps (vecjac_gb300/csrc/presweep.cuh),
compiled for the host by tests/presweep_host.cpp: whole one-sided Jacobi sweeps with the
kernel's own pair arithmetic, with column scales, short-form rotations and tracked squared
norms (the FP64 sweeps' form) against the plain form (no scales, norms recomputed at every
step), on graded, clustered and rank-deficient real and complex matrices. The two forms
must take the same number of sweeps (one fewer allowed) to the same accuracy: singular
values against the construction, V's orthogonality, the residual A V - G. A second build
lowers the column-scale threshold so that the general form of the rotation (the one that
returns the scales to 1) is exercised too."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
EPS = 2.0 ** -52


def build(tmp_path_factory, name, flags=()):
    out = str(tmp_path_factory.mktemp(name) / "presweep_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", *flags,
                        os.path.join(HERE, "presweep_host.cpp"), "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return build(tmp_path_factory, "presweep")


@pytest.fixture(scope="module")
def exe_general(tmp_path_factory):
    return build(tmp_path_factory, "presweep_general", ["-DVJ_PRESWEEP_COL_SCALE_MIN=0.9"])


def run(exe, kind, m, n, spec, seed):
    r = subprocess.run([exe, kind, str(m), str(n), spec, str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = {}
    for line in r.stdout.split("\n"):
        f = line.split()
        if f:
            rows[f[0]] = dict(sweeps=int(f[1]), sig=float(f[2]), orth=float(f[3]), resid=float(f[4]),
                              short=int(f[5]), general=int(f[6]), tracked=int(f[7]), exact=int(f[8]))
    return rows["plain"], rows["scaled"]


def check(plain, scaled, n):
    # same convergence and accuracy (plain dot products on sigma down to 1e-6: about 1e-11
    # relative in either form)
    assert scaled["sweeps"] <= plain["sweeps"] + 1
    for r in (plain, scaled):
        assert r["sig"] <= 1e-9, r
        assert r["orth"] <= 64 * n * EPS, r
        assert r["resid"] <= 8 * n * EPS, r
    assert scaled["sig"] <= max(4 * plain["sig"], 1e-13)
    # the plain form never uses scales or tracked norms
    assert plain["short"] == 0 and plain["tracked"] == 0


@pytest.mark.parametrize("kind,m,n,seed", [("r", 96, 32, 1), ("c", 64, 32, 2), ("r", 128, 64, 5)])
def test_graded(exe, kind, m, n, seed):
    plain, scaled = run(exe, kind, m, n, "graded", seed)
    check(plain, scaled, n)
    # most steps take the tracked norms and most rotations the short form
    assert scaled["tracked"] >= 0.8 * (scaled["tracked"] + scaled["exact"])
    assert scaled["short"] >= 0.95 * (scaled["short"] + scaled["general"])


@pytest.mark.parametrize("kind", ["r", "c"])
def test_clustered_computes_norms(exe, kind):
    # all singular values within 1e-7 of each other: every pair's tracked norms are too
    # close for the angle, so every step computes them
    plain, scaled = run(exe, kind, 64, 32, "clustered", 3)
    check(plain, scaled, 32)
    assert scaled["tracked"] == 0


@pytest.mark.parametrize("kind", ["r", "c"])
def test_rank_deficient(exe, kind):
    plain, scaled = run(exe, kind, 64, 32, "zerocols", 4)
    check(plain, scaled, 32)


@pytest.mark.parametrize("kind,spec", [("r", "graded"), ("c", "zerocols")])
def test_general_form(exe_general, kind, spec):
    plain, scaled = run(exe_general, kind, 96 if kind == "r" else 64, 32, spec, 1 if kind == "r" else 4)
    check(plain, scaled, 32)
    assert scaled["general"] > 0.02 * (scaled["short"] + scaled["general"])
