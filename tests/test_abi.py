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


def _svd_call(lib, kind, m, n, ldG, ldV, ptr, G=None, V=None, work=None, Gi=None, Vi=None, ldGi=None, ldVi=None,
              lp64=False):
    import ctypes as C
    u = lambda x: C.byref((C.c_uint if lp64 else C.c_ulonglong)(x))
    ctr = C.byref(C.c_uint(1))
    f = getattr(lib, kind + "vjsvd_")
    f.restype = C.c_int if lp64 else C.c_longlong
    G, V, work = (ptr if x is None else x for x in (G, V, work))
    if kind in "zc":
        Gi, Vi = (ptr if x is None else x for x in (Gi, Vi))
        return f(u(m), u(n), G, u(ldG), Gi, u(ldGi if ldGi is not None else ldG), V, u(ldV), Vi,
                 u(ldVi if ldVi is not None else ldV), ptr, ptr, ptr, ctr, ctr, work, ptr)
    return f(u(m), u(n), G, u(ldG), V, u(ldV), ptr, ptr, ptr, ctr, ctr, work, ptr)


def _check_svd_codes(lib, kind, lp64=False):
    import ctypes as C
    import numpy as np
    import torch
    buf = np.zeros(1 << 12, np.float64)
    al = (buf.ctypes.data + 63) & ~63
    A, B = C.c_void_p(al), C.c_void_p(al + 8)           # 64-byte aligned, misaligned
    L = 8 if kind in "dz" else 16
    m, n = 4 * L, 2 * L
    call = lambda **kw: _svd_call(lib, kind, kw.pop("m", m), kw.pop("n", n), kw.pop("ldG", m), kw.pop("ldV", n), A,
                                  lp64=lp64, **kw)
    assert call(n=0) == 0
    assert call(m=n - 2, ldG=n) == -1                    # m < n
    assert call(m=m + 1, ldG=m + L) == -1                # m % L
    assert call(n=n + 1) == -2                           # odd n
    assert call(n=2 * L + 2, m=8 * L, ldG=8 * L, ldV=4 * L) == -2    # (n/2) % L
    assert call(G=B) == -3
    assert call(ldG=m - L) == -4
    assert call(ldG=m + 1) == -4
    if kind in "zc":
        assert call(Gi=B) == -5
        assert call(ldGi=m + 1) == -6
        assert call(V=B) == -7
        assert call(ldV=n + 1) == -8
        assert call(Vi=B) == -9
        assert call(ldVi=n - L) == -10
        assert call(work=B) == -16
    else:
        assert call(V=B) == -5
        assert call(ldV=n - L) == -6
        assert call(ldV=n + 1) == -6
        assert call(work=B) == -12
    if not torch.cuda.is_available():
        assert call() == -100001                          # VJ_ERR_NO_GPU: no CPU fallback


@pytest.mark.parametrize("kind", "dzsc")
def test_svd_argument_codes(libpath, kind):
    """The reference's argument checks and codes, in its order (src/dvjsvd.c:43-67,
    src/zvjsvd.c:43-80 and the FP32 twins): they all return before the GPU is touched."""
    import ctypes as C
    lib = C.CDLL(libpath)
    assert lib.vj_abi_int_bits() == 64
    _check_svd_codes(lib, kind)


@pytest.fixture(scope="module")
def lp64_path(tmp_path_factory):
    # device code is not run here: ptxas at -O0 keeps this build short
    from vecjac_gb300 import build
    return build.build(lp64=True, out_dir=str(tmp_path_factory.mktemp("lp64")), extra=["-Xptxas", "-O0"])


def test_lp64_build(lp64_path):
    """The flavour for callers built with the reference's ABI=lp64 (32-bit fint/fnat): it
    says so, exports the same symbols, and reads 32-bit arguments."""
    import ctypes as C
    lib = C.CDLL(lp64_path)
    assert lib.vj_abi_int_bits() == 32
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    for kind in "dzsc":
        _check_svd_codes(lib, kind, lp64=True)
    f = lib.dbjac2_
    f.restype = C.c_int
    assert f(C.byref(C.c_int(12)), *([C.c_void_p(8)] * 8)) == -1


@pytest.mark.parametrize("kind", "dzsc")
def test_bjac2_length_code(libpath, kind):
    """|n| must be a multiple of the vector length (8 FP64, 16 FP32): -1 otherwise."""
    import ctypes as C
    import numpy as np
    lib = C.CDLL(libpath)
    f = getattr(lib, kind + "bjac2_")
    f.restype = C.c_longlong
    L = 8 if kind in "dz" else 16
    buf = np.zeros(64, np.float64)
    p = C.c_void_p(buf.ctypes.data)
    args = [p] * (10 if kind in "zc" else 8)
    for bad in (L + 2, -(L + 2), L // 2):
        assert f(C.byref(C.c_longlong(bad)), *args) == -1, bad


@pytest.mark.parametrize("lp64", [False, True])
def test_c_caller(libpath, lp64_path, tmp_path, lp64):
    """include/vecjac_gb300.h compiles as C11 and a C caller links and runs against the
    library (ILP64 and LP64 flavours) with the reference's calling convention."""
    import subprocess
    import torch
    lib = lp64_path if lp64 else libpath
    exe = str(tmp_path / "c_caller")
    cmd = ["gcc", "-std=c11", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include")]
    cmd += (["-DVJ_LP64"] if lp64 else []) + [os.path.join(ROOT, "tests", "c_caller.c"), "-L" + os.path.dirname(lib),
                                               "-lvecjac_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe] + (["gpu"] if torch.cuda.is_available() else []), capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok %d" % (32 if lp64 else 64), r.stdout + r.stderr
