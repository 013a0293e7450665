"""The 2x2 accuracy drivers t?bjac2.exe with the real library on the GPU: on the same
generator files they print exactly what the drivers linked against the oracle stand-in
print (every column but the timing, and the complex drivers' worst-element lines), since
the library's results equal the oracle's bit for bit.

The driver runs as a second process on the GPU this test process already uses; under an
exclusive compute mode that is impossible and the test is skipped.
"""
import subprocess

import pytest

from test_bjac2_driver_cpu import gen_files, standin_exes

pytestmark = [pytest.mark.gpu, pytest.mark.late]


@pytest.fixture(scope="module")
def exes(tmp_path_factory):
    from vecjac_gb300 import build
    build.build()
    real = build.build_cli(programs=(("tbjac2.cpp", "t%sbjac2.exe"),))
    try:
        mode = subprocess.run(["nvidia-smi", "--query-gpu=compute_mode", "--format=csv,noheader", "-i", "0"],
                              capture_output=True, text=True, timeout=60).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        mode = ""
    if mode and mode != "Default":
        pytest.skip("compute mode %s: a second process cannot use the GPU" % mode)
    return dict(zip(build.CLI_KINDS, real)), standin_exes(str(tmp_path_factory.mktemp("standin")))


@pytest.mark.parametrize("kind", "dzsc")
def test_driver_matches_standin(exes, tmp_path, kind):
    real, standin = exes
    base = str(tmp_path / ("g" + kind))
    gen_files(base, kind, 16, 2, seed=100 + ord(kind))
    a = subprocess.run([real[kind], base, "16", "2"], capture_output=True, text=True, timeout=300)
    b = subprocess.run([standin[kind], base, "16", "2"], capture_output=True, text=True, timeout=300)
    assert a.returncode == 0 and b.returncode == 0, (a.stderr, b.stderr)
    drop_ts = lambda out: [l.split(",")[:1] + l.split(",")[2:] for l in out.strip().split("\n")]
    assert drop_ts(a.stdout) == drop_ts(b.stdout)
    assert a.stderr == b.stderr
