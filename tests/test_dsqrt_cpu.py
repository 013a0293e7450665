"""The FP64 square root of the 2x2 kernels' fast path (vecjac_gb300/csrc/dsqrt.cuh),
compiled for the host by tests/dsqrt_host.cpp over exact models of the CUDA intrinsics it
uses: correctly rounded (equal to IEEE sqrt) on random arguments in [1, 2^1024), powers of
two, perfect squares, the neighbours of squared midpoints (the hardest cases for the
rounding test) and the largest doubles, with the FP32 reciprocal-root estimate moved by up
to 28 FP32 ulps either way."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dsqrt") / "dsqrt_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "dsqrt_host.cpp"),
                        "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_correctly_rounded(exe):
    r = subprocess.run([exe, str(400000), "3"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [tuple(int(v) for v in line.split()) for line in r.stdout.split("\n") if line.strip()]
    within = {k: bad for k, bad in rows if abs(k) <= 28}
    assert within and all(bad == 0 for bad in within.values()), within
