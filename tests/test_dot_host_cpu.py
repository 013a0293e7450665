"""The SVD's scaled compensated dot products (csrc/svd_dot.cuh: pair_dot and the FP64
chain_dot), run on the host by tests/dot_host.cpp with a warp emulated by 32 threads (each
lane's own code; shuffles through a barrier) over exact models of the CUDA intrinsics,
against the oracle's restatement of src/ddpscl.c / src/zdpscl.c: bit for bit on seeded
columns of one lane group to thousands of rows, values that keep the straight-line
blocks, graded values that take the general path (subnormal scaled values), and scale
exponents that overflow (a NaN result must be a NaN in both)."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from oracle import oracle as O
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    out = str(tmp_path_factory.mktemp("dot") / "dot_host")
    r = subprocess.run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-frounding-math", "-pthread",
                        os.path.join(HERE, "dot_host.cpp"), "-L" + libdir, "-lvjo", "-Wl,-rpath," + libdir, "-o", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("kind", "dzsc")
def test_dots_match_the_oracle(exe, kind):
    r = subprocess.run([exe, kind, "60", "11"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cases, bad = (int(x) for x in r.stdout.split())
    assert cases == 60 and bad == 0, (r.stdout, r.stderr[-800:])
