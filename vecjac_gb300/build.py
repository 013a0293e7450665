"""Build libvecjac_gb300.so for sm_103a with nvcc, in-tree (vecjac_gb300/_build/).

Every translation unit under csrc/ is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo --fmad=false`` (no implicit
multiply-add contraction: the kernels reproduce the reference's rounding op by op)
and linked against the CUDA runtime and cuBLAS (the plain FP64 GEMMs of the mixed-precision
SVD) -- PyTorch is not a dependency of the library.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvecjac_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-I" + os.path.join(os.path.dirname(HERE), "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _compile(src, extra, out=OUT):
    obj = os.path.join(out, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(p) for p in [src] + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(CSRC, "*.h")) + [os.path.join(os.path.dirname(HERE), "include",
                                                                    "vecjac_gb300.h"), __file__]):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


LP64_OUT = os.path.join(HERE, "_build_lp64")


def build(verbose=False, extra=(), lp64=False, out_dir=None):
    """Compile and link the library; returns its path. lp64=True builds the flavour with
    32-bit Fortran integers (-DVJ_LP64, the reference's ABI=lp64) into _build_lp64/ (or
    out_dir); the default is ILP64 in _build/, the build the Python API binds."""
    out = out_dir or (LP64_OUT if lp64 else OUT)
    lib = os.path.join(out, "libvecjac_gb300.so")
    extra = list(extra) + (["-DVJ_LP64"] if lp64 else [])
    os.makedirs(out, exist_ok=True)
    # objects built with other flags are not reused: a stamp records the flags of a folder
    stamp, flags = os.path.join(out, "flags"), " ".join([nvcc()] + ARCH + FLAGS + extra)
    old = open(stamp).read() if os.path.exists(stamp) else None
    if old != flags:
        for f in glob.glob(os.path.join(out, "*.o")) + [lib]:
            if os.path.exists(f):
                os.remove(f)
        with open(stamp, "w") as f:
            f.write(flags)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, out), srcs))
    if os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in objs):
        return lib
    cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", lib)
    return lib


CLI_KINDS = "dzsc"
# the command-line drivers: source and executable name pattern (kind in 'dzsc')
CLI_PROGRAMS = (("tvjsvd.cpp", "t%svjsvd.exe"), ("tbjac2.cpp", "t%sbjac2.exe"))


def cli_path(kind, program="t%svjsvd.exe"):
    """A command-line driver's path, e.g. t<kind>vjsvd.exe or t<kind>bjac2.exe."""
    return os.path.join(OUT, program % kind)


def _cuda_libdir():
    import shutil
    nv = nvcc()
    nv = nv if os.path.isabs(nv) else (shutil.which(nv) or "/usr/local/cuda/bin/nvcc")
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "lib64")


def build_cli(verbose=False, lib=None, out_dir=None, extra_sources=(), link_lib=True, programs=CLI_PROGRAMS,
              extra_flags=()):
    """Compile each command-line driver (csrc/tvjsvd.cpp: t?vjsvd.exe, csrc/tbjac2.cpp:
    t?bjac2.exe) once per precision next to the library (host C++ only, linked against
    libvecjac_gb300.so with an rpath to it and to the CUDA runtime). Returns the
    executables in the order of `programs` x CLI_KINDS. Tests build the same sources
    against a stand-in library through extra_sources/extra_flags/link_lib."""
    import shutil
    hdr = os.path.join(os.path.dirname(HERE), "include", "vecjac_gb300.h")
    out_dir = out_dir or OUT
    os.makedirs(out_dir, exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    base = [cxx] if cxx else [nvcc(), "-x", "c++"]
    # linker options: -Wl for a C++ driver, -Xlinker for nvcc
    lk = (lambda o: ["-Wl," + o]) if cxx else (lambda o: ["-Xlinker", o])
    def one(job):
        (srcname, pattern), kind = job
        src = os.path.join(CSRC, srcname)
        deps = [src, hdr, __file__] + list(extra_sources) + ([lib or LIB] if link_lib else [])
        exe = os.path.join(out_dir, pattern % kind)
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps):
            return exe
        cmd = base + ["-O2", "-std=c++17", "-DVJ_CLI_KIND='%s'" % kind, "-I" + os.path.dirname(hdr), src]
        cmd += list(extra_sources) + list(extra_flags)
        if link_lib:
            ld = os.path.dirname(lib or LIB)
            here = "$ORIGIN" if os.path.realpath(ld) == os.path.realpath(out_dir) else ld
            cmd += ["-L" + ld, "-lvecjac_gb300"] + lk("--disable-new-dtags") + lk("-rpath=" + here) + \
                lk("-rpath=" + _cuda_libdir())
        cmd += ["-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compiling the command-line driver failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return exe

    jobs = [(prog, kind) for prog in programs for kind in CLI_KINDS]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        exes = list(ex.map(one, jobs))
    if verbose:
        print("built", " ".join(os.path.basename(e) for e in exes))
    return exes


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--lp64" in args:
        build(verbose=True, extra=[a for a in args if a != "--lp64"], lp64=True)
    else:
        build(verbose=True, extra=args)
        build_cli(verbose=True)
