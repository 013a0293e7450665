"""ctypes mirror of the library's C ABI (include/vecjac_gb300.h).

Names, argument order and return codes follow the reference's entry points:
``bjac2(kind, n, ...)`` calls ``dbjac2_``/``zbjac2_``/``sbjac2_``/``cbjac2_`` (or the masked
``?bjac2i`` with ``internal=True``), ``vjsvd(kind, ...)`` calls ``?vjsvd_``, ``pjs`` calls
``pjs``. Host forms take numpy arrays; ``*_dev`` forms take CUDA tensors (anything with
``data_ptr()``) and an optional CUDA stream handle.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

VJ_ERR_NO_GPU = -100001
VJ_ERR_CUDA = -100002
VJ_ERR_NOMEM = -100003
VJ_ERR_ARG = -100004

_P = C.c_void_p
_ll = C.c_longlong
_ull = C.c_ulonglong


def lib_path():
    return os.path.join(HERE, "_build", "libvecjac_gb300.so")


def lib():
    """Load libvecjac_gb300.so (build it first with vecjac_gb300.build.build())."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError("libvecjac_gb300.so is not built: run python -m vecjac_gb300.build")
        lib_ = C.CDLL(path)
        if lib_.vj_abi_int_bits() != 64:
            raise RuntimeError("%s is an LP64 build; this module binds the ILP64 (default) build" % path)
        _LIB = lib_
        for name in ("dbjac2_", "zbjac2_", "sbjac2_", "cbjac2_", "dbjac2i", "zbjac2i", "sbjac2i", "cbjac2i",
                     "vj_dbjac2_dev", "vj_zbjac2_dev", "vj_sbjac2_dev", "vj_cbjac2_dev", "dvjsvd_", "zvjsvd_",
                     "svjsvd_", "cvjsvd_", "vj_dvjsvd_dev", "vj_zvjsvd_dev", "vj_svjsvd_dev", "vj_cvjsvd_dev",
                     "vj_pjs_dev", "vj_dvjsvd_mixed_dev", "vj_zvjsvd_mixed_dev",
                     "vj_ssvd_adjoint_batch_dev", "vj_dsvd_adjoint_batch_dev", "vj_dvjsvd_batch_dev",
                     "vj_svjsvd_batch_dev", "vj_dvjsvd_batch_tuned_dev", "vj_svjsvd_batch_tuned_dev",
                     "vj_last_mixed_phases", "zsplit_", "zmerge_", "csplit_", "cmerge_",
                     "vj_zsplit_dev", "vj_zmerge_dev", "vj_csplit_dev", "vj_cmerge_dev"):
            if hasattr(_LIB, name):
                getattr(_LIB, name).restype = _ll
        if hasattr(_LIB, "pjs"):
            _LIB.pjs.restype = C.POINTER(C.c_uint)
        _LIB.vj_version.restype = C.c_char_p
    return _LIB


def _p(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(_P)


def _dtype(kind):
    return np.float64 if kind in "dz" else np.float32


def bjac2(kind, n, a11, a22, a21, a21i=None, c=None, at=None, sat=None, l1=None, l2=None, p=None,
          internal=False):
    """Host call of ?bjac2_ (or ?bjac2i). Outputs are allocated when not given.

    Returns (ret, c, at, [sat,] l1, l2, p) like the reference's output arguments."""
    L = lib()
    dt = _dtype(kind)
    nn = abs(int(n))
    lanes = 8 if kind in "dz" else 16
    c = np.empty(nn, dt) if c is None else c
    at = np.empty(nn, dt) if at is None else at
    l1 = np.empty(nn, dt) if l1 is None else l1
    l2 = np.empty(nn, dt) if l2 is None else l2
    p = np.zeros(max(1, nn // lanes), np.uint32) if p is None else p
    nref = _ll(int(n))
    f = getattr(L, kind + ("bjac2i" if internal else "bjac2_"))
    if kind in "zc":
        sat = np.empty(nn, dt) if sat is None else sat
        r = f(C.byref(nref), _p(a11), _p(a22), _p(a21), _p(a21i), _p(c), _p(at), _p(sat), _p(l1), _p(l2), _p(p))
        return r, c, at, sat, l1, l2, p
    r = f(C.byref(nref), _p(a11), _p(a22), _p(a21), _p(c), _p(at), _p(l1), _p(l2), _p(p))
    return r, c, at, l1, l2, p


def bjac2_dev(kind, n, a11, a22, a21, a21i, c, at, sat, l1, l2, p, internal=False, stream=None):
    """Device call on CUDA tensors; asynchronous on ``stream`` (an int handle or None)."""
    L = lib()
    f = getattr(L, "vj_%sbjac2_dev" % kind)
    s = C.c_void_p(stream) if stream else None
    if kind in "zc":
        return f(_ll(int(n)), C.c_int(1 if internal else 0), _p(a11), _p(a22), _p(a21), _p(a21i), _p(c), _p(at),
                 _p(sat), _p(l1), _p(l2), _p(p), s)
    return f(_ll(int(n)), C.c_int(1 if internal else 0), _p(a11), _p(a22), _p(a21), _p(c), _p(at), _p(l1), _p(l2),
             _p(p), s)


def aligned(shape, dtype, order="F", align=64):
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    buf = np.zeros(count * dtype.itemsize + align, np.uint8)
    off = (-buf.ctypes.data) % align
    return buf[off:off + count * dtype.itemsize].view(dtype).reshape(shape, order=order)


def vjsvd(kind, G, js, stp, swp=999, V=None, Gi=None, Vi=None, eS=None, fS=None, work=None, iwork=None):
    """Host call of ?vjsvd_ on Fortran-ordered, 64-byte aligned copies of the inputs.

    Returns (ret, U, V, eS, fS[, Ui, Vi]); sigma_j = fS[j] * 2**eS[j]."""
    L = lib()
    dt = _dtype(kind)
    m, n = G.shape
    Gc = aligned((m, n), dt)
    Gc[...] = G
    preset = V is not None
    Vc = aligned((n, n), dt)
    if preset:
        Vc[...] = V
    eS = aligned(n, dt, "C") if eS is None else eS
    fS = aligned(n, dt, "C") if fS is None else fS
    work = aligned(8 * n + 64, dt, "C") if work is None else work
    iwork = aligned(max(2, n), np.uint32, "C") if iwork is None else iwork
    iwork[0] = 1 if preset else 0
    js = np.ascontiguousarray(js, np.uint32)
    m_, n_, ld_g, ld_v = _ull(m), _ull(n), _ull(m), _ull(n)
    stp_, swp_ = C.c_uint(int(stp)), C.c_uint(int(swp))
    f = getattr(L, kind + "vjsvd_")
    if kind in "zc":
        Gic = aligned((m, n), dt)
        Gic[...] = Gi
        Vic = aligned((n, n), dt)
        if preset:
            Vic[...] = Vi
        r = f(C.byref(m_), C.byref(n_), _p(Gc), C.byref(ld_g), _p(Gic), C.byref(ld_g), _p(Vc), C.byref(ld_v),
              _p(Vic), C.byref(ld_v), _p(eS), _p(fS), _p(js), C.byref(stp_), C.byref(swp_), _p(work), _p(iwork))
        return r, Gc, Vc, eS, fS, Gic, Vic
    r = f(C.byref(m_), C.byref(n_), _p(Gc), C.byref(ld_g), _p(Vc), C.byref(ld_v), _p(eS), _p(fS), _p(js),
          C.byref(stp_), C.byref(swp_), _p(work), _p(iwork))
    return r, Gc, Vc, eS, fS


def vjsvd_dev(kind, m, n, G, ldG, V, ldV, eS, fS, js, stp, swp=999, preset=False, Gi=None, ldGi=None, Vi=None,
              ldVi=None, stream=None):
    """Device call of the SVD on CUDA tensors (column-major storage, leading dimensions given)."""
    L = lib()
    f = getattr(L, "vj_%svjsvd_dev" % kind)
    s = C.c_void_p(stream) if stream else None
    if kind in "zc":
        return f(_ull(m), _ull(n), _p(G), _ull(ldG), _p(Gi), _ull(ldGi), _p(V), _ull(ldV), _p(Vi), _ull(ldVi),
                 _p(eS), _p(fS), _p(js), C.c_uint(int(stp)), C.c_uint(int(swp)), C.c_int(int(preset)), s)
    return f(_ull(m), _ull(n), _p(G), _ull(ldG), _p(V), _ull(ldV), _p(eS), _p(fS), _p(js), C.c_uint(int(stp)),
             C.c_uint(int(swp)), C.c_int(int(preset)), s)


def vjsvd_mixed_dev(kind, m, n, G, ldG, V, ldV, eS, fS, js, stp, swp=999, Gi=None, ldGi=None, Vi=None, ldVi=None,
                    stream=None, stages=0):
    """Mixed-precision device SVD of FP64 data (kind "d" or "z"): `stages` (0: 2) rounds of
    FP32 sweeps with FP64 re-orthogonalisation, plain-dot FP64 sweeps, then the reference's
    FP64 sweeps with V preset. Returns (finishing sweeps or error code, FP32 sweeps,
    plain-dot FP64 sweeps)."""
    if kind not in "dz":
        raise ValueError("the mixed-precision SVD takes FP64 data (kind d or z)")
    L = lib()
    f = getattr(L, "vj_%svjsvd_mixed_dev" % kind)
    s = C.c_void_p(stream) if stream else None
    pre = (C.c_uint * 2)()
    if kind == "z":
        r = f(_ull(m), _ull(n), _p(G), _ull(ldG), _p(Gi), _ull(ldGi), _p(V), _ull(ldV), _p(Vi), _ull(ldVi),
              _p(eS), _p(fS), _p(js), C.c_uint(int(stp)), C.c_uint(int(swp)), C.c_uint(int(stages)), pre, s)
    else:
        r = f(_ull(m), _ull(n), _p(G), _ull(ldG), _p(V), _ull(ldV), _p(eS), _p(fS), _p(js), C.c_uint(int(stp)),
              C.c_uint(int(swp)), C.c_uint(int(stages)), pre, s)
    return r, pre[0], pre[1]


def split(kind, A, Ar=None, Ai=None):
    """Host call of zsplit_ (kind "z") or csplit_ ("c") on a Fortran-ordered complex matrix.
    Returns (ret, Ar, Ai), the planes Fortran-ordered with leading dimension m."""
    L = lib()
    dt = _dtype(kind)
    A = np.asfortranarray(A, np.complex128 if kind == "z" else np.complex64)
    m, n = A.shape
    Ar = np.empty((m, n), dt, order="F") if Ar is None else Ar
    Ai = np.empty((m, n), dt, order="F") if Ai is None else Ai
    mm, nn = _ull(m), _ull(n)
    r = getattr(L, kind + "split_")(C.byref(mm), C.byref(nn), _p(A), C.byref(mm), _p(Ar), C.byref(mm), _p(Ai),
                                    C.byref(mm))
    return r, Ar, Ai


def merge(kind, Ar, Ai, A=None):
    """Host call of zmerge_ / cmerge_: two Fortran-ordered planes into an interleaved complex
    matrix. Returns (ret, A)."""
    L = lib()
    dt = _dtype(kind)
    Ar = np.asfortranarray(Ar, dt)
    Ai = np.asfortranarray(Ai, dt)
    m, n = Ar.shape
    A = np.empty((m, n), np.complex128 if kind == "z" else np.complex64, order="F") if A is None else A
    mm, nn = _ull(m), _ull(n)
    r = getattr(L, kind + "merge_")(C.byref(mm), C.byref(nn), _p(Ar), C.byref(mm), _p(Ai), C.byref(mm), _p(A),
                                    C.byref(mm))
    return r, A


def split_dev(kind, m, n, A, ldA, Ar, ldAr, Ai, ldAi, stream=None):
    """vj_zsplit_dev / vj_csplit_dev on CUDA tensors (A interleaved, ldA in complex elements)."""
    s = C.c_void_p(stream) if stream else None
    return getattr(lib(), "vj_%ssplit_dev" % kind)(_ull(m), _ull(n), _p(A), _ull(ldA), _p(Ar), _ull(ldAr), _p(Ai),
                                                   _ull(ldAi), s)


def merge_dev(kind, m, n, Ar, ldAr, Ai, ldAi, A, ldA, stream=None):
    """vj_zmerge_dev / vj_cmerge_dev on CUDA tensors."""
    s = C.c_void_p(stream) if stream else None
    return getattr(lib(), "vj_%smerge_dev" % kind)(_ull(m), _ull(n), _p(Ar), _ull(ldAr), _p(Ai), _ull(ldAi), _p(A),
                                                   _ull(ldA), s)


def pjs(sid, n):
    """Pivot table (stp x n uint32) of strategy id 2 or 4, generated on the GPU; (None, 0) on error."""
    L = lib()
    stp = C.c_uint(0)
    t = L.pjs(C.c_long(int(sid)), C.c_uint(int(n)), C.byref(stp))
    if not t:
        return None, 0
    arr = np.ctypeslib.as_array(t, shape=(stp.value * int(n),)).copy().reshape(stp.value, int(n))
    C.CDLL(None).free(C.cast(t, C.c_void_p))
    return arr, stp.value


def pjs_dev(sid, n, table, stream=None):
    L = lib()
    s = C.c_void_p(stream) if stream else None
    return L.vj_pjs_dev(C.c_long(int(sid)), C.c_uint(int(n)), _p(table), s)


class _Trace(C.Structure):
    _fields_ = [("sweeps", C.c_uint), ("rotations", C.c_ulonglong * 64), ("phase_cycles", C.c_ulonglong * 8)]


PHASES = ("control", "staging", "dots", "2x2", "rotations", "norms")


def last_mixed_phases():
    """Phase times (ms) of the last mixed-precision SVD: FP32 sweeps, orthonormalisation + GEMMs,
    plain FP64 sweeps + sort, the reference's finishing sweeps; the FP32 kernel launches and
    whether the FP32 stages ran as block sweeps on the tensor cores."""
    out = (C.c_double * 6)()
    lib().vj_last_mixed_phases(out)
    return {"fp32_ms": out[0], "gemm_ms": out[1], "fp64_plain_ms": out[2], "finish_ms": out[3],
            "fp32_launches": int(out[4]), "fp32_block_sweeps": bool(out[5])}


def last_trace():
    """Statistics of the last host-API SVD: transformed pairs per sweep and, with VJ_TRACE=1,
    SM cycles of one CTA per step phase (summed over all steps)."""
    t = _Trace()
    lib().vj_last_trace(C.byref(t))
    return {"sweeps": t.sweeps, "rotations": list(t.rotations[:min(t.sweeps, 64)]),
            "phase_cycles": dict(zip(PHASES, list(t.phase_cycles[:len(PHASES)])))}
