"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports every
entry point that include/vecjac_gb300.h declares (no compute calls without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def libpath():
    from vecjac_gb300 import build
    return build.build()


def declared():
    src = open(os.path.join(ROOT, "include", "vecjac_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"if", "defined", "sizeof"}
    return sorted({n for n in names if n not in skip})


def test_exports_every_declared_symbol(libpath):
    import ctypes
    lib = ctypes.CDLL(libpath)
    names = declared()
    assert "dbjac2_" in names and "dvjsvd_" in names and "pjs" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_gpu_errors_cleanly(libpath):
    """Without a GPU the entry points fail with VJ_ERR_NO_GPU instead of computing on the CPU."""
    import numpy as np
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import vecjac_gb300 as vj
    a = np.ones(8)
    assert vj.bjac2("d", -8, a, a, a)[0] == vj.VJ_ERR_NO_GPU
