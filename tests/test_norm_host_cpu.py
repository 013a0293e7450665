"""The project's column norm (csrc/svd_norm.cuh: warp_nrm2), run on the host by
tests/norm_host.cpp with a warp emulated by 32 threads over exact models of the CUDA
intrinsics, against the oracle's restatement (vjo_dnorm / vjo_snorm): every lane's result
bit for bit on seeded columns of 1 to 5000 rows -- values near 1, graded values over the
whole exponent range, zero columns, and columns with an infinity or a NaN."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from oracle import oracle as O
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    out = str(tmp_path_factory.mktemp("norm") / "norm_host")
    r = subprocess.run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-frounding-math", "-pthread",
                        os.path.join(HERE, "norm_host.cpp"), "-L" + libdir, "-lvjo", "-Wl,-rpath," + libdir, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("kind", "ds")
def test_norm_matches_the_oracle(exe, kind):
    r = subprocess.run([exe, kind, "150", "21"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cases, bad = (int(x) for x in r.stdout.split())
    assert cases == 150 and bad == 0, (r.stdout, r.stderr[-800:])
