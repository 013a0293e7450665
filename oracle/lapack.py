"""LAPACK xGESVJ as a second oracle for the one-sided Jacobi SVD (test infrastructure).

xGESVJ (Drmac and Veselic's one-sided Jacobi SVD, LAPACK 3.2+) is an implementation
independent of VecJac and of the restatement in this folder: different pivoting (de Rijk),
different rotations and convergence test, the same kind of relative accuracy. It comes
from the OpenBLAS that numpy bundles (symbols scipy_?gesvj_64_, ILP64), else from another
bundled OpenBLAS or the system LAPACK (?gesvj_, LP64). The tests compare singular values -- of the restatement on CPU and
of the GPU library -- with it; nothing in the library uses it.

`python -m oracle.lapack M N BaseName [kind]` mirrors the reference's LAPACK driver
(src/tdgesvj.c and its z/s/c siblings): it reads BaseName.G, calls xGESVJ('G', 'U', 'V'),
prints the same CSV line ("BaseName",M,N,info,seconds,SCALE,work(2..6)) and writes
BaseName.SL (SCALE * SVA in the `wide` type, binary128; VJ_WIDE=l for x87), .VL and .UL.
"""
import ctypes as C
import glob
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_LIB = None


def _find():
    """(CDLL, symbol prefix, symbol suffix, integer type) of a LAPACK with xGESVJ, or None:
    the OpenBLAS that numpy or scipy bundles (scipy-openblas or older openblas builds,
    ILP64 or LP64), else the system LAPACK."""
    import ctypes.util
    libs = []
    for mod, sub in (("numpy", "numpy.libs"), ("scipy", "scipy.libs")):
        try:
            m = __import__(mod)
            d = os.path.join(os.path.dirname(os.path.dirname(m.__file__)), sub)
            libs += sorted(glob.glob(os.path.join(d, "lib*openblas*.so*")))
        except Exception:
            pass
    sysl = ctypes.util.find_library("lapack")
    if sysl:
        libs.append(sysl)
    names = (("scipy_", "_64_", C.c_int64), ("", "_64_", C.c_int64), ("scipy_", "_", C.c_int32), ("", "_", C.c_int32))
    for path in libs:
        try:
            lib = C.CDLL(path)
        except OSError:
            continue
        for pre, suf, it in names:
            if hasattr(lib, pre + "dgesvj" + suf):
                return lib, pre, suf, it
    return None


def available():
    global _LIB
    if _LIB is None:
        _LIB = _find() or False
    return bool(_LIB)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def gesvj(kind, A):
    """xGESVJ('G', 'U', 'V') of the (m, n) matrix A, m >= n, kind in 'dzsc'.

    Returns (info, sigma, U, V, stats, sva): sigma = SCALE * SVA rounded to float64
    (descending, as xGESVJ sorts them), U (m, n) and V (n, n) in A's precision, stats =
    the six values of WORK/RWORK(1:6) (SCALE, nonzero sigmas, sigmas above underflow,
    sweeps, max |cos| and max |sin| of the last sweep), sva = SVA as returned."""
    if not available():
        raise RuntimeError("no LAPACK with xGESVJ found")
    lib, pre, suf, I = _LIB
    real = np.float64 if kind in "dz" else np.float32
    cplx = kind in "zc"
    dt = (np.complex128 if kind == "z" else np.complex64) if cplx else real
    m, n = A.shape
    G = np.asfortranarray(np.array(A, dtype=dt))
    sva = np.zeros(n, real)
    V = np.zeros((n, n), dt, order="F")
    info = I(0)
    mi, ni = I(m), I(n)
    hidden = (C.c_size_t(1), C.c_size_t(1), C.c_size_t(1))
    f = getattr(lib, "%s%sgesvj%s" % (pre, kind, suf))
    jobs = (C.c_char_p(b"G"), C.c_char_p(b"U"), C.c_char_p(b"V"))
    if not cplx:
        lwork = max(6, m + n)
        work = np.zeros(lwork, real)
        f(*jobs, C.byref(mi), C.byref(ni), _ptr(G), C.byref(mi), _ptr(sva), C.byref(ni), _ptr(V), C.byref(ni),
          _ptr(work), C.byref(I(lwork)), C.byref(info), *hidden)
        stats = work[:6].astype(np.float64)
    else:
        lwork, lrwork = m + n, max(6, n)
        cwork = np.zeros(lwork, dt)
        rwork = np.zeros(lrwork, real)
        f(*jobs, C.byref(mi), C.byref(ni), _ptr(G), C.byref(mi), _ptr(sva), C.byref(ni), _ptr(V), C.byref(ni),
          _ptr(cwork), C.byref(I(lwork)), _ptr(rwork), C.byref(I(lrwork)), C.byref(info), *hidden)
        stats = rwork[:6].astype(np.float64)
    sigma = sva.astype(np.float64) * stats[0]
    return int(info.value), sigma, G, V, stats, sva


def main(argv):
    """The reference's LAPACK driver over files (src/tdgesvj.c)."""
    sys.path.insert(0, ROOT)
    from fractions import Fraction
    from vecjac_gb300 import mtxio
    if len(argv) not in (4, 5):
        print("%s M N BaseName [kind]" % argv[0], file=sys.stderr)
        return 1
    try:
        m, n = int(argv[1], 0), int(argv[2], 0)
    except ValueError:
        m = n = 0
    bn, kind = argv[3], (argv[4] if len(argv) == 5 else "d")
    if not m or not n or not bn or kind not in "dzsc" or len(kind) != 1:
        print("%s M N BaseName [kind]" % argv[0], file=sys.stderr)
        return 1
    real = np.float64 if kind in "dz" else np.float32
    dt = (np.complex128 if kind == "z" else np.complex64) if kind in "zc" else real
    G = mtxio.read_matrix(bn + ".G", m, n, dt)
    t0 = time.perf_counter()
    info, _, U, V, st, sva = gesvj(kind, G)
    t = time.perf_counter() - t0
    print('"%s",%4d,%4d,%1d,%15.9f,%#.17e,%4d,%4d,%3d,%#.17e,%#.17e' % (bn, m, n, info, t, st[0], int(st[1]),
                                                                        int(st[2]), int(st[3]), st[4], st[5]))
    # SCALE * SVA in the wide type (exact in binary128, rounded to nearest in x87)
    fmt = "l" if os.environ.get("VJ_WIDE") == "l" else "q"
    scale = Fraction(float(st[0]))
    mtxio.write_wide(bn + ".SL", [Fraction(float(v)) * scale for v in sva], fmt)
    mtxio.write_matrix(bn + ".VL", V)
    mtxio.write_matrix(bn + ".UL", U)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
