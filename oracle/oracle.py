"""TEST INFRASTRUCTURE ONLY -- ctypes bindings of the CPU oracle.

Two libraries are bound here:

* ``libvjo.so`` (``oracle/_build``): the portable C restatement of VecJac's hot path
  (``oracle/vjo.c``). It builds on any architecture and is the checker for the GPU
  library's results in ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
  baseline.
* ``libvjref.so`` (``oracle/_ref``): VecJac itself, compiled from its own sources on an
  x86-64 host with AVX-512 (``make -C oracle ref``). It exists only where the reference
  checkout is present; it pins the restatement (``tests/golden/make_golden.py``).

Nothing in the product imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
VJO_PATH = os.path.join(HERE, "_build", "libvjo.so")
REF_PATH = os.path.join(HERE, "_ref", "libvjref.so")

_P = C.c_void_p
_ll = C.c_longlong
_ull = C.c_ulonglong


def build(ref=False):
    """Compile the restatement (and the reference when ``ref`` is set)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def aligned(shape, dtype, order="C", align=64):
    """Zeroed array whose data starts on an ``align``-byte boundary (the reference's
    AVX-512 code uses aligned loads and stores)."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    buf = np.zeros(count * dtype.itemsize + align, np.uint8)
    off = (-buf.ctypes.data) % align
    a = buf[off:off + count * dtype.itemsize].view(dtype)
    return a.reshape(shape, order=order)


def acopy(x, dtype=None, order="C"):
    x = np.asarray(x, dtype=dtype)
    a = aligned(x.shape, x.dtype, order=order)
    a[...] = x
    return a


class _Lib:
    """Common calling code for the two libraries (same symbols, different prefixes)."""

    def __init__(self, path, prefix):
        self.lib = C.CDLL(path)
        self.prefix = prefix

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # ----- batched 2x2 -----
    def bjac2(self, kind, n, a11, a22, a21, a21i=None, internal=False, p=None):
        """kind in 'dszc'; n signed like the reference. Returns (ret, outputs...)."""
        dt = np.float64 if kind in "dz" else np.float32
        lanes = 8 if kind in "dz" else 16
        nn = abs(n)
        a11, a22, a21 = acopy(a11, dt), acopy(a22, dt), acopy(a21, dt)
        a21i = None if a21i is None else acopy(a21i, dt)
        c = aligned(nn, dt)
        at = aligned(nn, dt)
        l1 = aligned(nn, dt)
        l2 = aligned(nn, dt)
        p = aligned(max(1, nn // lanes), np.uint32) if p is None else acopy(p, np.uint32)
        nref = _ll(n)
        name = kind + "bjac2" + ("i" if internal else "_")
        f = self.fn(name)
        f.restype = _ll
        if kind in "zc":
            sat = aligned(nn, dt)
            r = f(C.byref(nref), _ptr(a11), _ptr(a22), _ptr(a21), _ptr(a21i), _ptr(c), _ptr(at), _ptr(sat),
                  _ptr(l1), _ptr(l2), _ptr(p))
            return r, c, at, sat, l1, l2, p
        r = f(C.byref(nref), _ptr(a11), _ptr(a22), _ptr(a21), _ptr(c), _ptr(at), _ptr(l1), _ptr(l2), _ptr(p))
        return r, c, at, l1, l2, p

    # ----- SVD -----
    def vjsvd(self, kind, G, js, stp, swp=999, V=None, Gi=None, Vi=None):
        """Run ?vjsvd_ in place on Fortran-ordered copies. Returns (ret, G, V, eS, fS[, Gi, Vi])."""
        dt = np.float64 if kind in "dz" else np.float32
        m, n = G.shape
        G = acopy(G, dt, order="F")
        preset = V is not None
        V = acopy(V, dt, order="F") if preset else aligned((n, n), dt, order="F")
        eS = aligned(n, dt)
        fS = aligned(n, dt)
        work = aligned(16 * n + 64, dt)
        iwork = aligned(max(2, n), np.uint32)
        iwork[0] = 1 if preset else 0
        js = np.ascontiguousarray(js, np.uint32)
        m_, n_, ldG, ldV = _ull(m), _ull(n), _ull(m), _ull(n)
        stp_, swp_ = C.c_uint(stp), C.c_uint(swp)
        f = self.fn(kind + "vjsvd_")
        f.restype = _ll
        if kind in "zc":
            Gi = acopy(Gi, dt, order="F")
            Vi = acopy(Vi, dt, order="F") if preset else aligned((n, n), dt, order="F")
            r = f(C.byref(m_), C.byref(n_), _ptr(G), C.byref(ldG), _ptr(Gi), C.byref(ldG), _ptr(V), C.byref(ldV),
                  _ptr(Vi), C.byref(ldV), _ptr(eS), _ptr(fS), _ptr(js), C.byref(stp_), C.byref(swp_), _ptr(work),
                  _ptr(iwork))
            return r, G, V, eS, fS, Gi, Vi
        r = f(C.byref(m_), C.byref(n_), _ptr(G), C.byref(ldG), _ptr(V), C.byref(ldV), _ptr(eS), _ptr(fS),
              _ptr(js), C.byref(stp_), C.byref(swp_), _ptr(work), _ptr(iwork))
        return r, G, V, eS, fS


    # ----- interleaved <-> split complex -----
    def split(self, kind, A):
        """?split_ of a complex matrix (kind 'z' or 'c'). Returns (ret, Ar, Ai)."""
        dt = np.float64 if kind == "z" else np.float32
        m, n = A.shape
        Ac = acopy(A, np.complex128 if kind == "z" else np.complex64, order="F")
        Ar = aligned((m, n), dt, order="F")
        Ai = aligned((m, n), dt, order="F")
        f = self.fn(kind + "split_")
        f.restype = _ll
        mm, nn = _ull(m), _ull(n)
        r = f(C.byref(mm), C.byref(nn), _ptr(Ac), C.byref(mm), _ptr(Ar), C.byref(mm), _ptr(Ai), C.byref(mm))
        return r, Ar, Ai

    def merge(self, kind, Ar, Ai):
        """?merge_ of two planes (kind 'z' or 'c'). Returns (ret, A)."""
        dt = np.float64 if kind == "z" else np.float32
        m, n = Ar.shape
        Arc, Aic = acopy(Ar, dt, order="F"), acopy(Ai, dt, order="F")
        A = aligned((m, n), np.complex128 if kind == "z" else np.complex64, order="F")
        f = self.fn(kind + "merge_")
        f.restype = _ll
        mm, nn = _ull(m), _ull(n)
        r = f(C.byref(mm), C.byref(nn), _ptr(Arc), C.byref(mm), _ptr(Aic), C.byref(mm), _ptr(A), C.byref(mm))
        return r, A


class Restatement(_Lib):
    def __init__(self):
        if not os.path.exists(VJO_PATH):
            build()
        super().__init__(VJO_PATH, "vjo_")
        self.lib.vjo_pjs.restype = C.POINTER(C.c_uint)
        self.lib.vjo_dnorm.restype = C.c_double
        self.lib.vjo_snorm.restype = C.c_float
        self.lib.vjo_last_swt.restype = C.c_uint

    def last_swt(self):
        """Transformed pairs per sweep of the last vjsvd call (first 64 sweeps)."""
        out = (C.c_ulonglong * 64)()
        k = self.lib.vjo_last_swt(out, C.c_uint(64))
        return list(out[:min(k, 64)])

    def pjs(self, sid, n):
        stp = C.c_uint(0)
        t = self.lib.vjo_pjs(C.c_long(sid), C.c_uint(n), C.byref(stp))
        if not t:
            return None, 0
        arr = np.ctypeslib.as_array(t, shape=(stp.value * n,)).copy().reshape(stp.value, n)
        self.lib.vjo_free(C.cast(t, C.c_void_p))
        return arr, stp.value

    def nrm2(self, x):
        x = np.ascontiguousarray(x)
        if x.dtype == np.float64:
            return self.lib.vjo_dnorm(_ll(x.size), _ptr(x))
        return self.lib.vjo_snorm(_ll(x.size), _ptr(x))


class Reference(_Lib):
    """VecJac compiled from source; mode 0 = project norm, mode 1 = OpenBLAS + libm."""

    def __init__(self):
        super().__init__(REF_PATH, "")
        self.lib.vjref_set_blas.argtypes = [C.c_char_p]
        blas = openblas_path()
        self.has_blas = bool(blas) and self.lib.vjref_set_blas(blas.encode()) == 0

    def mode(self, m):
        if self.lib.vjref_set_mode(C.c_int(m)) != 0:
            raise RuntimeError("OpenBLAS norm unavailable")


def openblas_path():
    try:
        import numpy
        d = os.path.join(os.path.dirname(os.path.dirname(numpy.__file__)), "numpy.libs")
        for f in sorted(os.listdir(d)):
            if f.startswith("libscipy_openblas64_"):
                return os.path.join(d, f)
    except OSError:
        pass
    return None


def reference_available():
    return os.path.exists(REF_PATH)
