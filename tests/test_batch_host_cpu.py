"""The batched SVD's per-matrix driver (csrc/batch_core.cuh: svd_one -- the whole one-sided
Jacobi SVD of one matrix by one CTA), run on the host by tests/batch_host.cpp: one CTA of
32 lanes as fibers on one thread (lock step from barrier to barrier; shuffles and
__syncthreads are barriers), the device source compiled over exact models of the CUDA
intrinsics. Every matrix's return value, U, V, eS and fS equal the oracle's restatement
of the reference driver bit for bit: Gaussian matrices, graded columns (rescaling and
shears), zero columns and sweep caps, with both pivot orderings."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from oracle import oracle as O
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    cuda_inc = "/usr/local/cuda/include"
    out = str(tmp_path_factory.mktemp("batch") / "batch_host")
    r = subprocess.run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-frounding-math", "-I" + cuda_inc,
                        "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "batch_host.cpp"), "-L" + libdir,
                        "-lvjo", "-Wl,-rpath," + libdir, "-o", out], capture_output=True, text=True)
    if r.returncode != 0 and not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("no CUDA headers")
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.parametrize("kind,cases", [("d", 6), ("s", 3)])
def test_svd_one_matches_the_oracle(exe, kind, cases):
    r = subprocess.run([exe, kind, str(cases), "13"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    n, bad = (int(x) for x in r.stdout.split())
    assert n == cases and bad == 0, (r.stdout, r.stderr[-800:])
