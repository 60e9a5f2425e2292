"""Build libves.so (sm_103a) in this directory.

    python build.py            # compile if any source is newer than the library
    python build.py --force
    python build.py --variant bc   # libves_bc.so: the bounds-checked build (-DVES_BOUNDS_CHECK)

The library is compiled with nvcc for sm_103a only; each translation unit is
compiled in parallel and linked into one shared object.  No CMake.
"""
import argparse
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libves.so")
OBJDIR = os.path.join(HERE, "_build")

SOURCES = ["ves_kernels.cu", "ves_mixed.cu", "ves_extras.cu", "ves_varsize.cu", "ves_noalloc.cu", "ves_shiftnet.cu",
           "ves_api.cu", "ves_dropin_cxx.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
EXTRA = {}  # per-source extra nvcc flags


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


VARIANTS = {"": ("libves.so", "_build", []), "bc": ("libves_bc.so", "_build_bc", ["-DVES_BOUNDS_CHECK"])}


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "ves.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, variant=""):
    libname, objname, vflags = VARIANTS[variant]
    lib, objdir = os.path.join(HERE, libname), os.path.join(HERE, objname)
    if not force and not _stale(lib):
        return lib
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(objdir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + ARCH + FLAGS + vflags + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--variant", default="", choices=sorted(VARIANTS))
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, variant=a.variant))
