"""ctypes binding of libves.so (include/ves.h) plus layout helpers.

This module is the host-side mirror of the reference's C++ host API
(utils.h:37-65): every drop-in entry point of the library is reachable here
with NumPy float64 arrays in the reference's structure-of-arrays (SoA)
layout, and the native device API (ves_eigensolve & co.) with torch CUDA
tensors.  There is no CPU fallback: without the compiled library or a GPU
every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# VES_LIBRARY selects another build of the library (the bounds-checked
# libves_bc.so that build.py makes with variant="bc")
LIBPATH = os.environ.get("VES_LIBRARY") or os.path.join(HERE, "libves.so")

VES_STATUS_ITCAP = 1
VES_STATUS_NONFINITE = 2
VES_STATUS_SHIFT_FALLBACK = 4
VES_STATUS_REFINE_FALLBACK = 8
VES_STATUS_BAD_DIM = 16
VES_PREC_FP64 = 0
VES_PREC_FP32_REFINE = 1
VNORM_REFERENCE, VNORM_MAX, VNORM_TWO = 0, 1, 2

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p
_int, _dbl, _bool, _size = ctypes.c_int, ctypes.c_double, ctypes.c_bool, ctypes.c_size_t


class VesError(RuntimeError):
    pass


class ShiftNetConfig(ctypes.Structure):
    _fields_ = [("dim", _int), ("n_params", _int), ("hidden", _int), ("layers", _int), ("fourier", _int),
                ("loss", _int), ("delta", ctypes.c_float), ("seed", ctypes.c_ulonglong), ("subdiag", _int)]


VES_SHIFTNET_LOSS_CHAMFER, VES_SHIFTNET_LOSS_ROBUST = 0, 1


class Options(ctypes.Structure):
    _fields_ = [("precision", _int), ("max_its", _int), ("vnorm", _int), ("refine_steps", _int),
                ("refine_tol", _dbl), ("want_vectors", _int), ("blocks_per_sm", _int), ("varsize_order", _int),
                ("shift_sweeps", _int), ("shift_gate", ctypes.c_float), ("shift_polish", _int),
                ("work_counts", _VP)]


VES_WORK_RES64, VES_WORK_CORR32, VES_WORK_RESFF, VES_WORK_POLISH, VES_WORK_COUNTS = 0, 1, 2, 3, 4


# exported symbol -> (restype, argtypes); every name declared in include/ves.h
SIGNATURES = {
    "eigensolver": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D]),
    "hessenberg": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "call_zgehrd": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "call_zunghr": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "call_zlahqr_new": (None, [_int, _int, _int, _D, _D, _D, _D, _D, _D]),
    "call_ztrevc": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "call_zgemv": (None, [_bool, _int, _int, _int, _D, _D, _D, _D, _D, _D, _dbl, _dbl]),
    "call_backsubstitution": (None, [_int, _int, _int, _D, _D, _D, _D]),
    "repMatrixSoA": (None, [_int, _int, _int, _D, _D]),
    "repVectorSoA": (None, [_int, _int, _int, _D, _D]),
    "rearrangeMatrices": (None, [_int, _int, _int, _D, _D]),
    "arrangeMatricesAoS": (None, [_int, _int, _int, _D, _D]),
    "ves_default_options": (None, [ctypes.POINTER(Options)]),
    "ves_eigensolve_workspace_size": (_size, [_int, _int, _int, ctypes.POINTER(Options)]),
    "ves_eigensolve": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                              ctypes.POINTER(Options), _VP, _size, _VP]),
    "ves_zgehrd": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP]),
    "ves_zunghr": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP]),
    "ves_hessenberg": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "ves_zlahqr": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _int, _VP]),
    "ves_ztrevc": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "ves_zgemv": (_int, [_bool, _int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _dbl, _dbl, _VP]),
    "ves_backsubstitution": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP]),
    "ves_fp64_fma_rate": (_int, [_D, _VP]),
    "ves_fp32_fma_rate": (_int, [_D, _VP]),
    "ves_polyroots_workspace_size": (_size, [_int, _int, _int]),
    "ves_eigensolve_varsize_workspace_size": (_size, [ctypes.c_longlong, _int, ctypes.POINTER(Options)]),
    "ves_eigensolve_varsize": (_int, [ctypes.c_longlong, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                      ctypes.POINTER(Options), _VP, _size, _VP]),
    "ves_graph_capture_varsize": (_int, [ctypes.POINTER(_VP), ctypes.c_longlong, _int, _VP, _VP, _VP, _VP, _VP, _VP,
                                         _VP, _VP, _VP, ctypes.POINTER(Options), _VP, _size]),
    "ves_graph_launch": (_int, [_VP, _VP]),
    "ves_eigensolve_shifts_workspace_size": (_size, [_int, _int, _int, ctypes.POINTER(Options)]),
    "ves_eigensolve_shifts": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                     ctypes.POINTER(Options), _VP, _size, _VP]),
    "ves_shiftnet_create": (_int, [ctypes.POINTER(_VP), _int, _int, _int, ctypes.c_ulonglong]),
    "ves_shiftnet_default_config": (None, [ctypes.POINTER(ShiftNetConfig)]),
    "ves_shiftnet_create_config": (_int, [ctypes.POINTER(_VP), ctypes.POINTER(ShiftNetConfig)]),
    "ves_shiftnet_destroy": (None, [_VP]),
    "ves_shiftnet_train": (_int, [_VP, ctypes.c_longlong, _int, _VP, _VP, _VP, _VP, _VP, _int, _int,
                                  ctypes.c_float, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_float), _VP]),
    "ves_shiftnet_predict_workspace_size": (_size, [_VP, ctypes.c_longlong]),
    "ves_shiftnet_param_count": (_size, [_VP]),
    "ves_shiftnet_gradient": (_int, [_VP, ctypes.c_longlong, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "ves_shiftnet_predict": (_int, [_VP, ctypes.c_longlong, _int, _VP, _VP, _VP, _VP, _VP, _VP, _size, _VP]),
    "ves_shiftnet_save": (_int, [_VP, ctypes.c_char_p]),
    "ves_shiftnet_load": (_int, [ctypes.POINTER(_VP), ctypes.c_char_p]),
    "ves_gemm_bf16": (_int, [_int, _int, _int, _VP, _int, _VP, _int, _VP, _int, _VP, _VP, _int, _VP, _VP]),
    "ves_graph_destroy": (None, [_VP]),
    "ves_polyroots": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _size, _VP]),
    "ves_soa_from_complex": (_int, [_int, _int, _int, _VP, _int, _VP, _VP, _VP]),
    "ves_complex_from_soa": (_int, [_int, _int, _int, _VP, _VP, _int, _VP, _VP]),
    "ves_soa_vec_from_complex": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP]),
    "ves_complex_from_soa_vec": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP]),
    "ves_eigensolve_noalloc": (_int, [_int, _int, _int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "ves_partition_blocks": (_int, [_int, _int, _int, ctypes.POINTER(_int), ctypes.POINTER(_int)]),
    "ves_bounds_violations": (_int, [ctypes.POINTER(ctypes.c_ulonglong), _int]),
    "ves_last_error": (ctypes.c_char_p, []),
    "ves_release": (None, []),
    "ves_version": (_int, []),
}

_lib = None


def lib():
    """Load libves.so (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH) or os.environ.get("VES_AUTOBUILD", "1") == "1":
        try:
            import build as _build  # noqa: E402  (sibling module)
        except ImportError:
            _build = None
        if _build is not None:
            try:
                _build.build()
            except Exception as e:  # a stale-but-present library is still usable
                if not os.path.exists(LIBPATH):
                    raise VesError("libves.so is missing and could not be built: %s" % e)
    if not os.path.exists(LIBPATH):
        raise VesError("libves.so not found at %s (run build.py)" % LIBPATH)
    L = ctypes.CDLL(LIBPATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error():
    return lib().ves_last_error().decode()


def _check(rc, what):
    if rc != 0:
        raise VesError("%s failed (%d): %s" % (what, rc, last_error()))


def _dropin_check(what):
    msg = last_error()
    if msg:
        raise VesError("%s failed: %s" % (what, msg))


def default_options(**kw):
    o = Options()
    lib().ves_default_options(ctypes.byref(o))
    for k, v in kw.items():
        # work_counts: a device tensor of VES_WORK_COUNTS uint64/int64 counters (or a raw pointer)
        if k == "work_counts" and hasattr(v, "data_ptr"):
            v = v.data_ptr()
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------------------
# SoA layout helpers (reference utils.cpp:85-157), vectorised in NumPy.
# ---------------------------------------------------------------------------
def soa_from_complex(A, thread_cnt):
    """(N, n, n) complex -> (re, im) flat float64 planes in the SoA layout."""
    A = np.asarray(A)
    N, n, _ = A.shape
    if N % thread_cnt:
        raise ValueError("N=%d is not a multiple of thread_cnt=%d" % (N, thread_cnt))
    bc = N // thread_cnt
    # element (i, j) of matrix b*tc + t at b*tc*n*n + (i + j*n)*tc + t
    s = A.reshape(bc, thread_cnt, n, n).transpose(0, 3, 2, 1)  # b, j, i, t
    return (np.ascontiguousarray(s.real, dtype=np.float64).reshape(-1),
            np.ascontiguousarray(s.imag, dtype=np.float64).reshape(-1))


def complex_from_soa(re, im, dim, thread_cnt):
    re = np.asarray(re).reshape(-1, dim, dim, thread_cnt)  # b, j, i, t
    im = np.asarray(im).reshape(-1, dim, dim, thread_cnt)
    z = (re + 1j * im).transpose(0, 3, 2, 1)  # b, t, i, j
    return z.reshape(-1, dim, dim)


def soa_vec_from_complex(v, thread_cnt):
    v = np.asarray(v)
    N, n = v.shape
    bc = N // thread_cnt
    s = v.reshape(bc, thread_cnt, n).transpose(0, 2, 1)
    return (np.ascontiguousarray(s.real, dtype=np.float64).reshape(-1),
            np.ascontiguousarray(s.imag, dtype=np.float64).reshape(-1))


def complex_vec_from_soa(re, im, dim, thread_cnt):
    re = np.asarray(re).reshape(-1, dim, thread_cnt)
    im = np.asarray(im).reshape(-1, dim, thread_cnt)
    return (re + 1j * im).transpose(0, 2, 1).reshape(-1, dim)


# ---------------------------------------------------------------------------
# Drop-in calls on NumPy arrays (host pointers, synchronous).
# ---------------------------------------------------------------------------
def _p(a, name, n):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.ndim != 1 or not a.flags.c_contiguous:
        raise ValueError("%s must be a contiguous 1-D float64 array" % name)
    if not a.flags.writeable:
        raise ValueError("%s must be writeable" % name)
    if a.size < n:
        raise ValueError("%s has %d elements, %d needed" % (name, a.size, n))
    return a.ctypes.data_as(_D)


def _sizes(dim, block_cnt, thread_cnt):
    N = int(block_cnt) * int(thread_cnt)
    return N * dim * dim, N * dim


def eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().eigensolver(dim, block_cnt, thread_cnt, _p(rA, "rA", nm), _p(iA, "iA", nm), _p(rE, "rE", nv),
                      _p(iE, "iE", nv), _p(rV, "rV", nm), _p(iV, "iV", nm))
    _dropin_check("eigensolver")


def hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ):
    nm, _ = _sizes(dim, block_cnt, thread_cnt)
    lib().hessenberg(dim, block_cnt, thread_cnt, _p(rA, "rA", nm), _p(iA, "iA", nm), _p(rQ, "rQ", nm),
                     _p(iQ, "iQ", nm))
    _dropin_check("hessenberg")


def call_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().call_zgehrd(dim, block_cnt, thread_cnt, _p(rA, "rA", nm), _p(iA, "iA", nm), _p(rtau, "rtau", nv),
                      _p(itau, "itau", nv))
    _dropin_check("call_zgehrd")


def call_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().call_zunghr(dim, block_cnt, thread_cnt, _p(rA, "rA", nm), _p(iA, "iA", nm), _p(rtau, "rtau", nv),
                      _p(itau, "itau", nv))
    _dropin_check("call_zunghr")


def call_zlahqr_new(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().call_zlahqr_new(dim, block_cnt, thread_cnt, _p(rE, "rE", nv), _p(iE, "iE", nv), _p(rM, "rM", nm),
                          _p(iM, "iM", nm), _p(rS, "rS", nm), _p(iS, "iS", nm))
    _dropin_check("call_zlahqr_new")


def call_ztrevc(dim, block_cnt, thread_cnt, rT, iT, rR, iR):
    nm, _ = _sizes(dim, block_cnt, thread_cnt)
    lib().call_ztrevc(dim, block_cnt, thread_cnt, _p(rT, "rT", nm), _p(iT, "iT", nm), _p(rR, "rR", nm),
                      _p(iR, "iR", nm))
    _dropin_check("call_ztrevc")


def call_zgemv(hermitian, dim, block_cnt, thread_cnt, rM, iM, rx, ix, ry, iy, rbeta, ibeta):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().call_zgemv(bool(hermitian), dim, block_cnt, thread_cnt, _p(rM, "rM", nm), _p(iM, "iM", nm),
                     _p(rx, "rx", nv), _p(ix, "ix", nv), _p(ry, "ry", nv), _p(iy, "iy", nv), float(rbeta),
                     float(ibeta))
    _dropin_check("call_zgemv")


def call_backsubstitution(dim, block_cnt, thread_cnt, rT, iT, rb, ib):
    nm, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().call_backsubstitution(dim, block_cnt, thread_cnt, _p(rT, "rT", nm), _p(iT, "iT", nm), _p(rb, "rb", nv),
                                _p(ib, "ib", nv))
    _dropin_check("call_backsubstitution")


def repMatrixSoA(dim, block_cnt, thread_cnt, matrix, out):
    nm, _ = _sizes(dim, block_cnt, thread_cnt)
    lib().repMatrixSoA(dim, block_cnt, thread_cnt, _p(matrix, "matrix", dim * dim), _p(out, "out", nm))


def repVectorSoA(dim, block_cnt, thread_cnt, vec, out):
    _, nv = _sizes(dim, block_cnt, thread_cnt)
    lib().repVectorSoA(dim, block_cnt, thread_cnt, _p(vec, "vec", dim), _p(out, "out", nv))


def rearrangeMatrices(dim, block_cnt, thread_cnt, inp, out):
    nm, _ = _sizes(dim, block_cnt, thread_cnt)
    lib().rearrangeMatrices(dim, block_cnt, thread_cnt, _p(inp, "in", nm), _p(out, "out", nm))


def arrangeMatricesAoS(dim, block_cnt, thread_cnt, inp, out):
    nm, _ = _sizes(dim, block_cnt, thread_cnt)
    lib().arrangeMatricesAoS(dim, block_cnt, thread_cnt, _p(inp, "in", nm), _p(out, "out", nm))


# ---------------------------------------------------------------------------
# Native device API on torch CUDA tensors.
# ---------------------------------------------------------------------------
def _dp(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream_ptr(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Workspace:
    """A device workspace for ves_eigensolve held by the caller."""

    def __init__(self, dim, block_cnt, thread_cnt, options=None, device=None):
        import torch
        o = options if options is not None else default_options()
        self.nbytes = int(lib().ves_eigensolve_workspace_size(dim, block_cnt, thread_cnt, ctypes.byref(o)))
        self.buf = torch.empty(max(self.nbytes, 1) + 256, dtype=torch.uint8, device=device or "cuda")
        base = self.buf.data_ptr()
        self.ptr = (base + 255) // 256 * 256


def eigensolve(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV, rT=None, iT=None, status=None, sweeps=None,
               options=None, workspace=None, stream=None):
    """ves_eigensolve on torch CUDA tensors (asynchronous on `stream`)."""
    o = options if options is not None else default_options()
    ws_ptr, ws_n = (None, 0) if workspace is None else (ctypes.c_void_p(workspace.ptr), workspace.nbytes)
    rc = lib().ves_eigensolve(dim, block_cnt, thread_cnt, _dp(rA), _dp(iA), _dp(rE), _dp(iE), _dp(rV), _dp(iV),
                              _dp(rT), _dp(iT), _dp(status), _dp(sweeps), ctypes.byref(o), ws_ptr, ws_n,
                              _stream_ptr(stream))
    _check(rc, "ves_eigensolve")


class DeviceBuffer:
    """A 256-byte aligned device allocation (torch uint8 storage)."""

    def __init__(self, nbytes, device=None):
        import torch
        self.nbytes = int(nbytes)
        self.buf = torch.empty(max(self.nbytes, 1) + 256, dtype=torch.uint8, device=device or "cuda")
        self.ptr = (self.buf.data_ptr() + 255) // 256 * 256


def varsize_workspace(count, max_dim, options=None):
    o = options if options is not None else default_options()
    return DeviceBuffer(lib().ves_eigensolve_varsize_workspace_size(count, max_dim, ctypes.byref(o)))


def eigensolve_varsize(count, max_dim, dims, rA, iA, rE, iE, rV, iV, status=None, sweeps=None, options=None,
                       workspace=None, stream=None):
    """ves_eigensolve_varsize on torch CUDA tensors (packed mixed-size layout)."""
    o = options if options is not None else default_options()
    ws_ptr, ws_n = (None, 0) if workspace is None else (ctypes.c_void_p(workspace.ptr), workspace.nbytes)
    _check(lib().ves_eigensolve_varsize(count, max_dim, _dp(dims), _dp(rA), _dp(iA), _dp(rE), _dp(iE), _dp(rV),
                                        _dp(iV), _dp(status), _dp(sweeps), ctypes.byref(o), ws_ptr, ws_n,
                                        _stream_ptr(stream)), "ves_eigensolve_varsize")


class VarsizeGraph:
    """A captured CUDA graph of one mixed-size solve; replay with launch()."""

    def __init__(self, count, max_dim, dims, rA, iA, rE, iE, rV, iV, status=None, sweeps=None, options=None,
                 workspace=None):
        o = options if options is not None else default_options()
        self.workspace = workspace if workspace is not None else varsize_workspace(count, max_dim, o)
        self.handle = _VP()
        self._keep = (dims, rA, iA, rE, iE, rV, iV, status, sweeps)
        _check(lib().ves_graph_capture_varsize(ctypes.byref(self.handle), count, max_dim, _dp(dims), _dp(rA),
                                               _dp(iA), _dp(rE), _dp(iE), _dp(rV), _dp(iV), _dp(status),
                                               _dp(sweeps), ctypes.byref(o), ctypes.c_void_p(self.workspace.ptr),
                                               self.workspace.nbytes), "ves_graph_capture_varsize")

    def launch(self, stream=None):
        _check(lib().ves_graph_launch(self.handle, _stream_ptr(stream)), "ves_graph_launch")

    def __del__(self):
        try:
            if self.handle:
                lib().ves_graph_destroy(self.handle)
        except Exception:
            pass


def eigensolve_shifts(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV, rS, iS, status=None, sweeps=None,
                      fallbacks=None, options=None, workspace=None, stream=None):
    """ves_eigensolve_shifts on torch CUDA tensors (predicted shifts rS, iS)."""
    o = options if options is not None else default_options()
    ws_ptr, ws_n = (None, 0) if workspace is None else (ctypes.c_void_p(workspace.ptr), workspace.nbytes)
    _check(lib().ves_eigensolve_shifts(dim, block_cnt, thread_cnt, _dp(rA), _dp(iA), _dp(rE), _dp(iE), _dp(rV),
                                       _dp(iV), _dp(rS), _dp(iS), _dp(status), _dp(sweeps), _dp(fallbacks),
                                       ctypes.byref(o), ws_ptr, ws_n, _stream_ptr(stream)), "ves_eigensolve_shifts")


def shifts_workspace(dim, block_cnt, thread_cnt, options=None):
    """A device workspace for ves_eigensolve_shifts with these options."""
    o = options if options is not None else default_options()
    return DeviceBuffer(lib().ves_eigensolve_shifts_workspace_size(dim, block_cnt, thread_cnt, ctypes.byref(o)))


class ShiftNet:
    """The learned-shift network (ves_shiftnet_*): features -> predicted eigenvalues."""

    def __init__(self, dim=None, n_params=0, hidden=256, seed=0, path=None, **config):
        """config: layers, fourier, loss, delta (ves_shiftnet_config fields)."""
        self.handle = _VP()
        if path is not None:
            _check(lib().ves_shiftnet_load(ctypes.byref(self.handle), path.encode()), "ves_shiftnet_load")
        else:
            c = ShiftNetConfig()
            lib().ves_shiftnet_default_config(ctypes.byref(c))
            c.dim, c.n_params, c.hidden, c.seed = dim, n_params, hidden, seed
            for k, v in config.items():
                setattr(c, k, v)
            _check(lib().ves_shiftnet_create_config(ctypes.byref(self.handle), ctypes.byref(c)),
                   "ves_shiftnet_create_config")

    def train(self, count, thread_cnt, params, rA, iA, rE, iE, epochs=20, batch=1024, lr=1e-3, seed=0, stream=None):
        losses = (ctypes.c_float * max(epochs, 1))()
        _check(lib().ves_shiftnet_train(self.handle, count, thread_cnt, _dp(params), _dp(rA), _dp(iA), _dp(rE),
                                        _dp(iE), epochs, batch, lr, seed, losses, _stream_ptr(stream)),
               "ves_shiftnet_train")
        return list(losses)[:epochs]

    def gradient(self, count, thread_cnt, params, rA, iA, rE, iE, stream=None):
        """(grad, loss): the loss and parameter gradients of one batch of all
        `count` matrices (device tensors; grad in checkpoint order)."""
        import torch
        grad = torch.empty(int(lib().ves_shiftnet_param_count(self.handle)), dtype=torch.float32, device=rA.device)
        loss = torch.zeros(1, dtype=torch.float32, device=rA.device)
        _check(lib().ves_shiftnet_gradient(self.handle, count, thread_cnt, _dp(params), _dp(rA), _dp(iA), _dp(rE),
                                           _dp(iE), _dp(grad), _dp(loss), _stream_ptr(stream)),
               "ves_shiftnet_gradient")
        return grad, loss

    def predict_workspace(self, count):
        return DeviceBuffer(lib().ves_shiftnet_predict_workspace_size(self.handle, count))

    def predict_into(self, count, thread_cnt, params, rA, iA, rS, iS, workspace, stream=None):
        """Inference into rS, iS with a caller-held workspace (predict_workspace)."""
        _check(lib().ves_shiftnet_predict(self.handle, count, thread_cnt, _dp(params), _dp(rA), _dp(iA), _dp(rS),
                                          _dp(iS), ctypes.c_void_p(workspace.ptr), workspace.nbytes,
                                          _stream_ptr(stream)), "ves_shiftnet_predict")

    def predict(self, count, thread_cnt, params, rA, iA, rS, iS, stream=None):
        ws = self.predict_workspace(count)
        self.predict_into(count, thread_cnt, params, rA, iA, rS, iS, ws, stream)
        return ws

    def save(self, path):
        _check(lib().ves_shiftnet_save(self.handle, path.encode()), "ves_shiftnet_save")

    def __del__(self):
        try:
            if self.handle:
                lib().ves_shiftnet_destroy(self.handle)
        except Exception:
            pass


def gemm_bf16(A, Bt, bias=None, act=0, out_bf16=True, out_f32=False, err=None, stream=None):
    """C = A @ Bt.T (+ bias, GELU) on the tcgen05 tensor cores; A (M, K) and Bt (N, K)
    contiguous bfloat16 CUDA tensors.  Returns (C_bf16 or None, C_f32 or None)."""
    import torch
    M, K = A.shape
    N = Bt.shape[0]
    C = torch.empty(M, N, dtype=torch.bfloat16, device=A.device) if out_bf16 else None
    Cf = torch.empty(M, N, dtype=torch.float32, device=A.device) if out_f32 else None
    _check(lib().ves_gemm_bf16(M, N, K, _dp(A), A.stride(0), _dp(Bt), Bt.stride(0), _dp(bias), act, _dp(C), _dp(Cf),
                               N, _dp(err), _stream_ptr(stream)), "ves_gemm_bf16")
    return C, Cf


def polyroots(degree, block_cnt, thread_cnt, rC, iC, rR, iR, status=None, stream=None):
    """Roots of SoA-stored polynomials (device tensors), see ves_polyroots."""
    _check(lib().ves_polyroots(degree, block_cnt, thread_cnt, _dp(rC), _dp(iC), _dp(rR), _dp(iR), _dp(status), None, 0,
                               _stream_ptr(stream)), "ves_polyroots")


def soa_from_complex_dev(dim, block_cnt, thread_cnt, z, re, im, row_major=True, stream=None):
    """Device: interleaved complex batch z (e.g. torch complex128 (N, n, n)) -> SoA planes."""
    _check(lib().ves_soa_from_complex(dim, block_cnt, thread_cnt, _dp(z), int(row_major), _dp(re), _dp(im),
                                      _stream_ptr(stream)), "ves_soa_from_complex")


def complex_from_soa_dev(dim, block_cnt, thread_cnt, re, im, z, row_major=True, stream=None):
    _check(lib().ves_complex_from_soa(dim, block_cnt, thread_cnt, _dp(re), _dp(im), int(row_major), _dp(z),
                                      _stream_ptr(stream)), "ves_complex_from_soa")


def soa_vec_from_complex_dev(dim, block_cnt, thread_cnt, z, re, im, stream=None):
    _check(lib().ves_soa_vec_from_complex(dim, block_cnt, thread_cnt, _dp(z), _dp(re), _dp(im), _stream_ptr(stream)),
           "ves_soa_vec_from_complex")


def complex_from_soa_vec_dev(dim, block_cnt, thread_cnt, re, im, z, stream=None):
    _check(lib().ves_complex_from_soa_vec(dim, block_cnt, thread_cnt, _dp(re), _dp(im), _dp(z), _stream_ptr(stream)),
           "ves_complex_from_soa_vec")


def zgehrd_dev(dim, block_cnt, thread_cnt, rA, iA, rtau, itau, stream=None):
    _check(lib().ves_zgehrd(dim, block_cnt, thread_cnt, _dp(rA), _dp(iA), _dp(rtau), _dp(itau), _stream_ptr(stream)),
           "ves_zgehrd")


def zunghr_dev(dim, block_cnt, thread_cnt, rA, iA, rtau, itau, stream=None):
    _check(lib().ves_zunghr(dim, block_cnt, thread_cnt, _dp(rA), _dp(iA), _dp(rtau), _dp(itau), _stream_ptr(stream)),
           "ves_zunghr")


def zlahqr_dev(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS, status=None, max_its=30, stream=None):
    _check(lib().ves_zlahqr(dim, block_cnt, thread_cnt, _dp(rE), _dp(iE), _dp(rM), _dp(iM), _dp(rS), _dp(iS),
                            _dp(status), max_its, _stream_ptr(stream)), "ves_zlahqr")


def fp64_fma_rate(stream=None):
    """Measured FP64 FMA throughput of the current GPU, flop/s."""
    v = ctypes.c_double(0.0)
    _check(lib().ves_fp64_fma_rate(ctypes.byref(v), _stream_ptr(stream)), "ves_fp64_fma_rate")
    return v.value


def partition_blocks(block_cnt, parts, part):
    """(first_block, n_blocks): the contiguous range of whole SoA blocks that
    part `part` of `parts` owns when one batch is split over several GPUs."""
    f, nb = _int(0), _int(0)
    _check(lib().ves_partition_blocks(block_cnt, parts, part, ctypes.byref(f), ctypes.byref(nb)),
           "ves_partition_blocks")
    return f.value, nb.value


def fp32_fma_rate(stream=None):
    """Measured FP32 FMA throughput of the current GPU, flop/s."""
    v = ctypes.c_double(0.0)
    _check(lib().ves_fp32_fma_rate(ctypes.byref(v), _stream_ptr(stream)), "ves_fp32_fma_rate")
    return v.value


def ztrevc_dev(dim, block_cnt, thread_cnt, rT, iT, rR, iR, rwork, iwork, stream=None):
    _check(lib().ves_ztrevc(dim, block_cnt, thread_cnt, _dp(rT), _dp(iT), _dp(rR), _dp(iR), _dp(rwork), _dp(iwork),
                            _stream_ptr(stream)), "ves_ztrevc")
