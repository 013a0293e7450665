"""Generate the golden fixtures of tests/golden/ by running VecJac itself.

The reference is compiled from its own sources (``make -C oracle ref``; x86-64 with
AVX-512 only, so this script runs on the development host, never on the GPU host) and
called through ctypes. Mode 0 routes the reference's BLAS xNRM2 and libm hypot to the
project's portable norm (oracle/vjo_nrm2.h), which makes every output reproducible bit
for bit by the C restatement and by the GPU library; mode 1 keeps the stock OpenBLAS
norm and libm hypot, whose singular values are stored for tolerance checks.

    python tests/golden/make_golden.py [--new | --split]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vecjac_gb300 import workloads as W  # noqa: E402


def special2x2(kind, n, seed):
    """2x2 inputs with infinities and NaNs among the special finite values"""
    rng = np.random.default_rng(seed)
    dt = np.float64 if kind in "dz" else np.float32
    fi = np.finfo(dt)
    vals = np.array([0.0, -0.0, 1.0, -2.0, fi.max, -fi.max, fi.tiny, fi.smallest_subnormal, -fi.smallest_subnormal,
                     np.inf, -np.inf, np.nan, 3e-300 if dt == np.float64 else 3e-40, 5.0], dt)
    return [rng.choice(vals, n).astype(dt) for _ in range(4 if kind in "zc" else 3)]


def bjac2_special_fixtures(ref):
    for kind in "dszc":
        ins = special2x2(kind, 1024, 4)
        out = {"a11": ins[0], "a22": ins[1], "a21": ins[2]}
        if kind in "zc":
            out["a21i"] = ins[3]
        names = ["c", "at", "sat", "l1", "l2", "p"] if kind in "zc" else ["c", "at", "l1", "l2", "p"]
        for tag, sgn in (("sin", -1), ("tan", 1)):
            r = ref.bjac2(kind, sgn * 1024, *ins)
            for name, arr in zip(names, r[1:]):
                out[f"{tag}_{name}"] = np.array(arr)
        np.savez_compressed(os.path.join(HERE, f"bjac2_{kind}_special.npz"), **out)


def bjac2_fixtures(ref):
    for kind in "dszc":
        lanes = 8 if kind in "dz" else 16
        rnd = W.pairs2x2(kind, 1536, seed=11 + ord(kind))
        edg = W.edge2x2(kind, 512, seed=23 + ord(kind))
        ins = [np.concatenate([a, b]) for a, b in zip(rnd, edg)]
        n = ins[0].size
        rng = np.random.default_rng(5)
        pin = (rng.integers(0, 3, n // lanes).astype(np.uint32) * np.uint32(0x10001 if lanes == 16 else 0x101))
        out = {"a11": ins[0], "a22": ins[1], "a21": ins[2], "p_in": pin}
        if kind in "zc":
            out["a21i"] = ins[3]
        names = ["c", "at", "sat", "l1", "l2", "p"] if kind in "zc" else ["c", "at", "l1", "l2", "p"]
        for tag, sgn, internal in (("sin", -1, False), ("tan", 1, False), ("isec", -1, True), ("itan", 1, True)):
            r = ref.bjac2(kind, sgn * n, *ins, internal=internal, p=(pin.copy() if internal else None))
            assert r[0] >= 0, (kind, tag, r[0])
            for name, arr in zip(names, r[1:]):
                out[f"{tag}_{name}"] = np.array(arr)
        np.savez_compressed(os.path.join(HERE, f"bjac2_{kind}.npz"), **out)


def svd_cases():
    """(name, kind, G, Gi, V, Vi, strategy, swp)"""
    cases = []
    A, _ = W.svd_matrix(64, 32, seed=101)
    cases.append(("d_64x32", "d", A, None, None, None, 2, 999))
    A, _ = W.svd_matrix(48, 16, seed=102, lo=-12.0)
    cases.append(("d_48x16_k1e12", "d", A, None, None, None, 4, 999))
    cases.append(("d_graded16", "d", W.graded16(), None, None, None, 2, 999))
    A, _ = W.svd_matrix(32, 32, seed=103)
    cases.append(("d_32x32_swp2", "d", A, None, None, None, 2, 2))
    A, _ = W.svd_matrix(32, 16, seed=104)
    rng = np.random.default_rng(104)
    V0 = W.haar(16, rng) * 3.0
    cases.append(("d_32x16_presetV", "d", A, None, V0, None, 2, 999))
    A, _ = W.svd_matrix(16, 16, seed=105)
    A[:, 5] = 0.0
    cases.append(("d_16x16_zerocol", "d", A, None, None, None, 2, 999))
    A, _ = W.svd_matrix(64, 64, seed=106)
    cases.append(("s_64x64", "s", A, None, None, None, 2, 999))
    A, _ = W.svd_matrix(48, 32, seed=107, complex_=True)
    cases.append(("z_48x32", "z", A.real, A.imag, None, None, 2, 999))
    A, _ = W.svd_matrix(32, 16, seed=108, complex_=True)
    rng = np.random.default_rng(108)
    V0 = W.haar(16, rng, True)
    cases.append(("z_32x16_presetV", "z", A.real, A.imag, V0.real, V0.imag, 4, 999))
    A, _ = W.svd_matrix(64, 32, seed=109, complex_=True)
    cases.append(("c_64x32", "c", A.real, A.imag, None, None, 2, 999))
    # rescaling, shear and rank paths in the other precisions, a sweep cap in FP32, a
    # preset V in FP32 complex, and a larger FP64 case
    rng = np.random.default_rng(110)
    ph = rng.uniform(0, 2 * np.pi, (16, 16))
    g = W.graded16()
    cases.append(("z_graded16", "z", g * np.cos(ph), g * np.sin(ph), None, None, 2, 999))
    cases.append(("s_graded32", "s", W.graded32_f32(), None, None, None, 2, 999))
    A, _ = W.svd_matrix(16, 16, seed=111, complex_=True)
    A[:, 9] = 0.0
    cases.append(("z_16x16_zerocol", "z", A.real, A.imag, None, None, 4, 999))
    A, _ = W.svd_matrix(32, 32, seed=112, complex_=True)
    rng = np.random.default_rng(112)
    V0 = W.haar(32, rng, True) * 0.5
    cases.append(("c_32x32_presetV", "c", A.real, A.imag, V0.real, V0.imag, 4, 999))
    A, _ = W.svd_matrix(64, 32, seed=113)
    cases.append(("s_64x32_swp1", "s", A, None, None, None, 4, 1))
    A, _ = W.svd_matrix(128, 64, seed=114, lo=-8.0)
    cases.append(("d_128x64", "d", A, None, None, None, 4, 999))
    return cases


def svd_fixtures(ref, rst, only_new=False):
    for name, kind, G, Gi, V, Vi, sid, swp in svd_cases():
        if only_new and os.path.exists(os.path.join(HERE, f"svd_{name}.npz")):
            continue
        m, n = G.shape
        js, stp = rst.pjs(sid, n)
        kw = dict(js=js, stp=stp, swp=swp, V=V)
        if kind in "zc":
            kw.update(Gi=Gi, Vi=Vi)
        ref.mode(0)
        r = ref.vjsvd(kind, G, **kw)
        out = {"G": G, "js": js, "stp": np.uint32(stp), "swp": np.uint32(swp), "sid": np.int32(sid),
               "ret": np.int64(r[0]), "U": r[1], "V": r[2], "eS": r[3], "fS": r[4]}
        if V is not None:
            out["V0"] = V
        if kind in "zc":
            out["Gi"] = Gi
            out["Ui"] = r[5]
            out["Vi"] = r[6]
            if Vi is not None:
                out["Vi0"] = Vi
        if ref.has_blas:
            ref.mode(1)
            rb = ref.vjsvd(kind, G, **kw)
            out["blas_ret"] = np.int64(rb[0])
            out["blas_eS"] = rb[3]
            out["blas_fS"] = rb[4]
            ref.mode(0)
        np.savez_compressed(os.path.join(HERE, f"svd_{name}.npz"), **out)
        print(name, "sweeps", r[0], "(stock BLAS norm:", out.get("blas_ret"), ")")


def split_matrix(kind, m, n, seed):
    """real and imaginary planes of an m x n complex matrix with special values (signed
    zeros, infinities, a NaN with a payload) among random ones"""
    rng = np.random.default_rng(seed)
    dt = np.float64 if kind == "z" else np.float32
    re, im = rng.standard_normal((m, n)).astype(dt), rng.standard_normal((m, n)).astype(dt)
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan], dt)
    re.flat[::7] = rng.choice(sp, re.flat[::7].size)
    im.flat[3::11] = rng.choice(sp, im.flat[3::11].size)
    nanp = np.array([0x7ff4000000000123 if kind == "z" else 0x7fa00123], np.uint64 if kind == "z" else np.uint32)
    re.flat[5] = nanp.view(dt)[0]
    return re, im


def split_fixtures(ref):
    """zsplit_/zmerge_ and csplit_/cmerge_ of the compiled reference"""
    out = {}
    for kind in "zc":
        m, n = (24, 7) if kind == "z" else (48, 5)
        re, im = split_matrix(kind, m, n, 31 + ord(kind))
        # the interleaved input assembled from the planes' bits (complex arithmetic would not
        # keep the NaN payloads)
        Ai = np.empty((m, n), np.complex128 if kind == "z" else np.complex64)
        Ai.real, Ai.imag = re, im
        r, Ar, Aim = ref.split(kind, Ai)
        q, B = ref.merge(kind, re, im)
        out.update({f"{kind}_A": Ai, f"{kind}_re": re, f"{kind}_im": im, f"{kind}_split_ret": r,
                    f"{kind}_Ar": np.array(Ar), f"{kind}_Ai": np.array(Aim), f"{kind}_merge_ret": q,
                    f"{kind}_B": np.array(B)})
    np.savez_compressed(os.path.join(HERE, "split_merge.npz"), **out)


def main():
    """All fixtures; with --new only the SVD fixtures whose files do not exist yet."""
    O.build(ref=True)
    ref = O.Reference()
    rst = O.Restatement()
    if "--new" in sys.argv[1:]:
        svd_fixtures(ref, rst, only_new=True)
        return
    if "--split" in sys.argv[1:]:
        split_fixtures(ref)
        return
    split_fixtures(ref)
    bjac2_fixtures(ref)
    bjac2_special_fixtures(ref)
    svd_fixtures(ref, rst)


if __name__ == "__main__":
    main()
