"""ctypes loader for the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker or the timed CPU reference --
never by the product.

  restatement()  -> libves_oracle.so, the C restatement of the reference path
                    (ves_oracle.c), built by `make -C oracle`.
  reference()    -> _ref/libref.so, the unmodified reference sources compiled
                    through ref_harness.cpp (`make -C oracle ref`); only
                    available where the reference checkout exists (None otherwise).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libves_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_int, _dbl = ctypes.c_int, ctypes.c_double

_ORACLE_SIGS = {
    "vo_set_threads": (None, [_int]),
    "vo_get_threads": (_int, []),
    "vo_zgehrd": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "vo_zunghr": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "vo_clear_below_subdiag": (None, [_int, _int, _int, _D, _D]),
    "vo_zlahqr": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D, _I]),
    "vo_ztrevc": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "vo_zgemv": (None, [_int, _int, _int, _int, _D, _D, _D, _D, _dbl, _dbl, _D, _D]),
    "vo_backsubstitution": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "vo_eigensolver": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D, _I]),
}
_REF_SIGS = {
    "ref_set_threads": (None, [_int]),
    "ref_call_zgehrd": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_call_zunghr": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_hessenberg": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_zgehrd_zw": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_zunghr_zw": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_hessenberg_zw": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_call_zlahqr_new": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D]),
    "ref_call_ztrevc": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_call_zgemv": (None, [_int, _int, _int, _int, _D, _D, _D, _D, _D, _D, _dbl, _dbl]),
    "ref_call_backsubstitution": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "ref_eigensolver_shipped": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D]),
    "ref_eigensolver_cleared": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D]),
    "ref_repMatrixSoA": (None, [_int, _int, _int, _D, _D]),
    "ref_repVectorSoA": (None, [_int, _int, _int, _D, _D]),
    "ref_rearrangeMatrices": (None, [_int, _int, _int, _D, _D]),
    "ref_arrangeMatricesAoS": (None, [_int, _int, _int, _D, _D]),
}

_cache = {}


def build(ref=True):
    """Compile the restatement (and the reference harness when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref and os.path.exists(os.path.join(reference_dir(), "utils.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + reference_dir()], check=True)


def reference_dir():
    """The reference checkout: $VES_REFERENCE_DIR, else a directory named
    "reference" beside the repository (absent on machines without it)."""
    return os.environ.get("VES_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _load(path, sigs):
    L = ctypes.CDLL(path)
    for k, (res, args) in sigs.items():
        f = getattr(L, k)
        f.restype = res
        f.argtypes = args
    return L


def restatement():
    if "o" not in _cache:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        _cache["o"] = _load(ORACLE_SO, _ORACLE_SIGS)
    return _cache["o"]


def reference():
    """The compiled reference, or None where it is not available."""
    if "r" not in _cache:
        _cache["r"] = _load(REF_SO, _REF_SIGS) if os.path.exists(REF_SO) else None
    return _cache["r"]


def ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I)


def eigensolve(rA, iA, dim, thread_cnt, lib=None, threads=0):
    """Run the full path on SoA planes (copies; inputs untouched).
    Returns (rE, iE, rV, iV, rT, iT, sweeps) with sweeps None for the reference."""
    N = rA.size // (dim * dim)
    bc = N // thread_cnt
    rA = rA.copy(); iA = iA.copy()
    rV = np.zeros_like(rA); iV = np.zeros_like(iA)
    rE = np.zeros(N * dim); iE = np.zeros(N * dim)
    if lib is None or lib == "restatement":
        L = restatement()
        L.vo_set_threads(threads)
        sw = np.zeros(N, dtype=np.int32)
        L.vo_eigensolver(dim, bc, thread_cnt, ptr(rA), ptr(iA), ptr(rE), ptr(iE), ptr(rV), ptr(iV), iptr(sw))
        return rE, iE, rV, iV, rA, iA, sw
    R = reference()
    if R is None:
        raise RuntimeError("reference build not available")
    if threads:
        R.ref_set_threads(threads)
    fn = R.ref_eigensolver_cleared if lib == "reference" else R.ref_eigensolver_shipped
    fn(dim, bc, thread_cnt, ptr(rA), ptr(iA), ptr(rE), ptr(iE), ptr(rV), ptr(iV))
    return rE, iE, rV, iV, rA, iA, None
