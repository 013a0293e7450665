"""The 2x2 lanes of the batched EVD kernels (csrc/jac2.cuh with the integer-pipe division
of csrc/idiv.cuh), compiled for the host by tests/jac2_host.cpp over exact models of the
CUDA intrinsics (tests/cuda_host_shim.h), against the oracle's ?bjac2_: bit for bit on
2^20 elements per precision in both output forms, with zeros, subnormals, extremes,
infinities and NaN mixed into the benchmark's +-2^e * u inputs. This checks the device
source's arithmetic on far more inputs than a GPU test run compares; the GPU tests check
the kernels built from it."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from oracle import oracle as O
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    out = str(tmp_path_factory.mktemp("jac2") / "jac2_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "jac2_host.cpp"),
                        "-L" + libdir, "-lvjo", "-Wl,-rpath," + libdir, "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("kind", "dzsc")
def test_lanes_match_the_oracle(exe, kind):
    r = subprocess.run([exe, kind, str(1 << 20), "77"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    checked, bad = (int(x) for x in r.stdout.split())
    assert checked == 2 << 20 and bad == 0, (r.stdout, r.stderr[-500:])
