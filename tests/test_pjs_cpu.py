"""The closed-form pivot pairs (csrc/pjs.cuh) that the GPU table generator and the batched
SVD kernel evaluate on the device, compiled for the host by tests/pjs_host.cpp: for every
even n up to 1024 and both orderings (id 2 round-robin, id 4 modulus), every pair equals
the oracle's loop-built table and the pair contract holds."""
import os
import subprocess


HERE = os.path.dirname(os.path.abspath(__file__))


def test_closed_forms_match_the_oracle_tables(tmp_path):
    from oracle import oracle as O
    O.build()
    libdir = os.path.dirname(O.VJO_PATH)
    exe = str(tmp_path / "pjs_host")
    r = subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(HERE, "pjs_host.cpp"), "-L" + libdir, "-lvjo",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "1024"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    checked, bad, contract = (int(x) for x in r.stdout.split())
    assert checked == 1024 and bad == 0 and contract == 0, r.stdout
