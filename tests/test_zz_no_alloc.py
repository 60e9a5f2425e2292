"""ves_eigensolve_noalloc: the allocation-free entry point, called through the
C ABI, against ves_eigensolve on the same batch.

This entry point exists for callers that may not allocate device memory
(a host whose allocator belongs to someone else, code that may not allocate
after start-up); it runs the FP64 solver in a static device array instead of
a workspace.  Two calls in a row must both match ves_eigensolve, which also
shows that whatever the first call leaves in the shared array does not leak
into the second.  Collected last (file name), so a failure here cannot stop
a -x run before the other tests have run; it also passes on its own in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

import ves

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-12  # |lambda - lambda_ref| / ||A||_F, as in the parity tests
VEC_TOL = 1e-12  # relative eigenvector difference (same scaling convention)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _solve_noalloc(n, bc, tc, dAr, dAi):
    import torch
    N = bc * tc
    dEr = torch.full((N * n,), np.nan, dtype=torch.float64, device="cuda")
    dEi = torch.full_like(dEr, np.nan)
    dVr = torch.full_like(dAr, np.nan)
    dVi = torch.full_like(dAi, np.nan)
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = ves.lib().ves_eigensolve_noalloc(n, bc, tc, _ptr(dAr), _ptr(dAi), _ptr(dEr), _ptr(dEi), _ptr(dVr), _ptr(dVi),
                                          _ptr(st), stream)
    assert rc == 0, ves.last_error()
    torch.cuda.synchronize()
    return dEr.cpu().numpy(), dEi.cpu().numpy(), dVr.cpu().numpy(), dVi.cpu().numpy(), st.cpu().numpy()


def _solve_ref(n, bc, tc, dAr, dAi):
    import torch
    N = bc * tc
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    dVr, dVi = torch.empty_like(dAr), torch.empty_like(dAi)
    st = torch.empty(N, dtype=torch.int32, device="cuda")
    ves.eigensolve(n, bc, tc, dAr, dAi, dEr, dEi, dVr, dVi, status=st)
    torch.cuda.synchronize()
    return dEr.cpu().numpy(), dEi.cpu().numpy(), dVr.cpu().numpy(), dVi.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("n,bc,tc", [(16, 64, 512), (7, 9, 13), (64, 2, 32)])
def test_noalloc_matches_eigensolve_twice(n, bc, tc):
    import torch
    N = bc * tc
    rng = np.random.default_rng(70 + n)
    A = rng.standard_normal((N, n, n)) + 1j * rng.standard_normal((N, n, n))
    rA, iA = ves.soa_from_complex(A, tc)
    dAr, dAi = torch.from_numpy(rA).cuda(), torch.from_numpy(iA).cuda()
    ref = _solve_ref(n, bc, tc, dAr, dAi)
    E_ref = ves.complex_vec_from_soa(ref[0], ref[1], n, tc)
    V_ref = ves.complex_from_soa(ref[2], ref[3], n, tc)
    nA = np.linalg.norm(A, axis=(1, 2))
    for call in range(2):
        out = _solve_noalloc(n, bc, tc, dAr, dAi)
        E = ves.complex_vec_from_soa(out[0], out[1], n, tc)
        V = ves.complex_from_soa(out[2], out[3], n, tc)
        assert (np.abs(E - E_ref).max(axis=1) / nA).max() <= EIG_TOL, call
        dv = np.linalg.norm(V - V_ref, axis=1) / np.linalg.norm(V_ref, axis=1)
        assert dv.max() <= VEC_TOL, call
        np.testing.assert_array_equal(out[4], ref[4])


def test_noalloc_rejects_oversize_dim():
    import torch
    z = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = ves.lib().ves_eigensolve_noalloc(65, 1, 1, _ptr(z), _ptr(z), _ptr(z), _ptr(z), _ptr(z), _ptr(z), None, None)
    assert rc == -1
    assert "VES_NOALLOC_MAX_DIM" in ves.last_error()
