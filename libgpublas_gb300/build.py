"""Build recipe for libgbxblas.so (sm_103a only).

Compiles every CUDA translation unit with nvcc and every C file with gcc,
in parallel, and links one shared library in-tree:

    libgpublas_gb300/libgbxblas.so           the BLAS library (csrc/)
    libgpublas_gb300/libgbxblas_preload.so   the same plus the allocation
                                             interposer (csrc/preload_*.c)
    libgpublas_gb300/libgbxdiag.so           diagnostics for benchmarks and
                                             failure-path tests (csrc_diag/),
                                             linked against libgbxblas.so

The build is skipped when a stamp of all sources, headers and flags matches
the last successful build.  No cmake, no torch extension machinery: the
library is a plain C ABI that Fortran programs load with LD_PRELOAD.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
CSRC_DIAG = os.path.join(HERE, "csrc_diag")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbxblas.so")
PRELOAD_LIB = os.path.join(HERE, "libgbxblas_preload.so")
DIAG_LIB = os.path.join(HERE, "libgbxdiag.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbxblas")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    c = sorted(glob.glob(os.path.join(CSRC, "*.c")))   # includes preload_*.c
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                 glob.glob(os.path.join(ROOT, "include", "*.h")))
    return cu, c, hdr


def _diag_sources():
    return sorted(glob.glob(os.path.join(CSRC_DIAG, "*.cu")))


def _stamp(files, extra):
    h = hashlib.sha256()
    for f in files:
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_library(force: bool = False, verbose: bool = False) -> str:
    cu, c, hdr = _sources()
    dcu = _diag_sources()
    nvcc = _nvcc()
    stamp = _stamp(cu + c + hdr + dcu, NVCC_FLAGS + CC_FLAGS + [nvcc])
    stamp_file = os.path.join(BUILD, "stamp")
    if (not force and all(os.path.exists(p) for p in (LIB, PRELOAD_LIB, DIAG_LIB))
            and os.path.exists(stamp_file) and open(stamp_file).read() == stamp):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs.append(([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj], obj))
    for src in c:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs.append((["gcc"] + CC_FLAGS + ["-c", src, "-o", obj], obj))
    diag_objs = []
    for src in dcu:
        obj = os.path.join(BUILD, "diag_" + os.path.basename(src) + ".o")
        jobs.append(([nvcc] + NVCC_FLAGS + ["-I" + CSRC, "-c", src, "-o", obj], obj))
        diag_objs.append(obj)
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [j[1] for j in jobs if j[1] not in diag_objs]
    # libgbxblas.so: the BLAS library; libgbxblas_preload.so: the same plus
    # the malloc/free interposer (preload_*.c), for LD_PRELOAD use.
    core = [o for o in objs if not os.path.basename(o).startswith("preload_")]
    for out, parts in ((LIB, core), (PRELOAD_LIB, objs)):
        tmp = out + ".tmp%d" % os.getpid()
        # executing the library prints its options (csrc/so_entry.c)
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + parts +
             ["-Xlinker", "-e", "-Xlinker", "gbx_so_entry", "-lpthread", "-ldl"])
        os.replace(tmp, out)
    # libgbxdiag.so: benchmark and failure-path diagnostics, resolved against
    # libgbxblas.so next to it
    tmp = DIAG_LIB + ".tmp%d" % os.getpid()
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + diag_objs +
         ["-L" + HERE, "-lgbxblas", "-Xlinker", "-rpath=$ORIGIN", "-lpthread"])
    os.replace(tmp, DIAG_LIB)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
