"""The integer-pipe FP64 division of the 2x2 kernels (csrc/idiv.cuh, ddiv_int) on the host.

tests/idiv_host.cpp compiles the header itself with the CUDA intrinsics it uses modelled
exactly (bit casts, round-toward-zero conversions) and the FP32 reciprocal estimate taken
as the correctly rounded 1/x moved by K ulps. Every quotient must be bit-identical to the
host's IEEE division:
  * K in -2..2 (rcp.approx.ftz.f32 is documented within 1 ulp): no pair may need the FP64
    fallback -- the one-step corrections alone are exact;
  * estimates 16 to 4096 ulps off (relative error up to 2^-11): the range check must
    route the pairs it cannot correct to the FP64 unit, never return a wrong quotient.
    The check is sound while a digit estimate is off by less than 2^10, i.e. for a
    reciprocal error below 2^-10; far beyond that (2^-7) the 64-bit remainder can wrap
    into range and a wrong quotient can pass, which the device's estimate (about 2^-21)
    never comes near;
  * zeros, subnormals, infinities, NaN, and quotients at the edges of the normal range.
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("idiv") / "idiv_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "idiv_host.cpp"), "-o",
                        out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run(exe, *args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    per_k = [tuple(int(x) for x in l.split()) for l in lines if l and not l.startswith("special")]
    special = [l for l in lines if l.startswith("special")][0].split()
    return per_k, int(special[1]), int(special[2])


def test_within_the_estimate_bound(exe):
    per_k, bad, count = run(exe, 2000000, 88172645463325252)
    assert [k for k, _, _ in per_k] == [-2, -1, 0, 1, 2]
    assert all(m == 0 and f == 0 for _, m, f in per_k), per_k
    assert bad == 0 and count > 200000


def test_bad_estimates_fall_back(exe):
    per_k, bad, _ = run(exe, 200000, 12345, "stress")
    assert all(m == 0 for _, m, _ in per_k), per_k
    assert all(f > 0 for _, _, f in per_k), per_k
    assert bad == 0
