"""libves.so on a CPU-only machine: it loads, exports every entry point that
include/ves.h declares, its host-side layout helpers agree with the
reference's (utils.cpp:85-157), and its GPU entry points fail loudly -- no
CPU fallback -- when there is no GPU."""
import os
import re

import numpy as np
import pytest

import ves

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ves.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:void|int|size_t|char)\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("eigensolver", "hessenberg", "call_zgehrd", "call_zunghr", "call_zlahqr_new", "call_ztrevc",
                "call_zgemv", "call_backsubstitution", "repMatrixSoA", "repVectorSoA", "rearrangeMatrices",
                "arrangeMatricesAoS"):
        assert ref in names


def test_library_exports_every_declared_symbol():
    L = ves.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the binding knows every one of them
    assert set(declared_functions()) <= set(ves.SIGNATURES)


def test_version():
    assert ves.lib().ves_version() >= 100


def test_default_options_match_the_header():
    """ves_default_options (host code) gives the defaults include/ves.h documents."""
    o = ves.default_options()
    assert o.precision == ves.VES_PREC_FP64
    assert o.max_its == 30
    assert o.refine_steps == 8
    assert o.refine_tol == 5e-14
    assert o.want_vectors == 1
    assert o.blocks_per_sm == 0  # the library's measured launch shape


def _soa_reference(A, tc):
    N, n, _ = A.shape
    out = np.zeros(N * n * n)
    for m in range(N):
        b, t = divmod(m, tc)
        for i in range(n):
            for j in range(n):
                out[b * tc * n * n + (i + j * n) * tc + t] = A[m, i, j]
    return out


@pytest.mark.parametrize("n,bc,tc", [(3, 2, 4), (5, 3, 1), (4, 1, 7)])
def test_host_layout_helpers(n, bc, tc):
    rng = np.random.default_rng(n)
    N = bc * tc
    A = rng.standard_normal((N, n, n))
    aos = np.ascontiguousarray(A.transpose(0, 2, 1)).reshape(-1)  # column-major per matrix
    soa = np.zeros(N * n * n)
    ves.rearrangeMatrices(n, bc, tc, aos, soa)
    np.testing.assert_array_equal(soa, _soa_reference(A, tc))
    back = np.zeros_like(aos)
    ves.arrangeMatricesAoS(n, bc, tc, soa, back)
    np.testing.assert_array_equal(back, aos)
    m = rng.standard_normal(n * n)
    rep = np.zeros(N * n * n)
    ves.repMatrixSoA(n, bc, tc, m, rep)
    M = np.broadcast_to(m.reshape(n, n).T, (N, n, n))
    np.testing.assert_array_equal(rep, _soa_reference(M, tc))
    v = rng.standard_normal(n)
    repv = np.zeros(N * n)
    ves.repVectorSoA(n, bc, tc, v, repv)
    np.testing.assert_array_equal(repv.reshape(bc, n, tc), np.broadcast_to(v[None, :, None], (bc, n, tc)))


def test_numpy_layout_helpers_roundtrip():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((12, 4, 4)) + 1j * rng.standard_normal((12, 4, 4))
    for tc in (1, 3, 4, 12):
        r, i = ves.soa_from_complex(A, tc)
        np.testing.assert_array_equal(r, _soa_reference(A.real, tc))
        np.testing.assert_array_equal(ves.complex_from_soa(r, i, 4, tc), A)
        v = A[:, :, 0]
        vr, vi = ves.soa_vec_from_complex(v, tc)
        np.testing.assert_array_equal(ves.complex_vec_from_soa(vr, vi, 4, tc), v)


def test_argument_checks():
    a = np.zeros(16)
    with pytest.raises(ValueError):
        ves.eigensolver(2, 1, 4, a.astype(np.float32), a, a, a, a, a)
    with pytest.raises(ValueError):
        ves.eigensolver(2, 1, 4, a[:3], a, a, a, a, a)


def test_gpu_entry_points_fail_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    n, bc, tc = 4, 1, 4
    rA = np.ones(n * n * tc); iA = np.zeros_like(rA)
    rE = np.zeros(n * tc); iE = np.zeros_like(rE)
    rV = np.zeros_like(rA); iV = np.zeros_like(rA)
    with pytest.raises(ves.VesError):
        ves.eigensolver(n, bc, tc, rA, iA, rE, iE, rV, iV)
    with pytest.raises(ves.VesError):
        ves.call_zgehrd(n, bc, tc, rA, iA, rE, iE)


def test_python_interface_mirrors_reference_module():
    import python_interface as pi
    # the function names of python_interface.pyx:31-220
    for name in ("my_repMatrix", "arrangeMatrices", "my_zlahqr", "my_backsubs", "my_repVector", "my_ztrevec",
                 "my_zgemv", "my_zgehrd", "my_zunghr", "my_hessenberg", "extractMatrix", "extractVector",
                 "test_backsubs", "test_zgehrd", "test_hessenberg", "test_zgemv", "test_zlahqr",
                 "test_eigenvectors"):
        assert callable(getattr(pi, name))
    m = np.arange(2 * 9 * 4, dtype=float)
    np.testing.assert_array_equal(pi.extractMatrix(3, 4, m), m[::4][:9].reshape(3, 3).T)
    np.testing.assert_array_equal(pi.extractVector(3, 4, m), m[::4][:3])


def test_bounds_query_needs_the_checked_build():
    """ves_bounds_violations counts only in the bounds-checked build
    (libves_bc.so); the normal library says so instead of returning 0."""
    import ctypes
    cnt = ctypes.c_ulonglong(7)
    assert ves.lib().ves_bounds_violations(ctypes.byref(cnt), 0) == -4  # VES_ERR_UNSUPPORTED
    assert cnt.value == 0
