"""The AVX-512-semantics primitives of csrc/vj_fp.cuh (min/max, getexp, getmant, ilogb,
scale2, scalef, in FP64 and FP32), compiled for the host by tests/fp_host.cpp, against
the oracle's restatement of the same instructions (oracle/vjo_fp.h): bit for bit on
random bit patterns of every class, NaN payloads, and shifts over the whole range."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def test_primitives_match_the_oracle(tmp_path):
    exe = str(tmp_path / "fp_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "fp_host.cpp"), "-o",
                        exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "500000", "99"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    checked, bad = (int(x) for x in r.stdout.split())
    assert checked > 8000000 and bad == 0, (r.stdout, r.stderr[-500:])
