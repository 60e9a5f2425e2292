"""Entry points around the solver path: eigenvalues only, companion-matrix
polynomial roots, and the SoA <-> interleaved-complex device transposes."""
import numpy as np
import pytest

import oracle
from oracle import ptr, iptr
import ves
from gpu_util import run_fused
from parity import match_eigs

pytestmark = pytest.mark.gpu


def cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def run_eigvals(A, tc, max_its=30):
    import torch
    N, n, _ = A.shape
    rA, iA = ves.soa_from_complex(A, tc)
    dAr, dAi = torch.from_numpy(rA).cuda(), torch.from_numpy(iA).cuda()
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    sw = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    opt = ves.default_options(want_vectors=0, max_its=max_its)
    ves.eigensolve(n, N // tc, tc, dAr, dAi, dEr, dEi, None, None, status=st, sweeps=sw, options=opt)
    torch.cuda.synchronize()
    return (ves.complex_vec_from_soa(dEr.cpu().numpy(), dEi.cpu().numpy(), n, tc), st.cpu().numpy(),
            sw.cpu().numpy())


@pytest.mark.parametrize("n,N,tc", [(1, 64, 4), (5, 96, 32), (16, 2048, 512), (32, 256, 32), (13, 77, 7)])
def test_eigvals_only_equals_full_solve(n, N, tc):
    rng = np.random.default_rng(300 + n)
    A = cgauss(rng, (N, n, n))
    E, st, sw = run_eigvals(A, tc)
    full = run_fused(A, tc)
    # same arithmetic on the active block: the same eigenvalues, bit for bit
    np.testing.assert_array_equal(E, full["E"])
    np.testing.assert_array_equal(sw, full["sweeps"])
    assert (st == 0).all()
    _, err, _ = match_eigs(E, np.linalg.eigvals(A))
    assert (err / np.linalg.norm(A, axis=(1, 2))).max() <= 1e-12


def companion_oracle_roots(C):
    """Roots through the oracle's zlahqr on the reference's companion matrix."""
    N, d1 = C.shape
    n = d1 - 1
    M = np.zeros((N, n, n), complex)
    M[:, np.arange(1, n), np.arange(n - 1)] = 1.0
    M[:, :, n - 1] = -C[:, :n] / C[:, n:n + 1]
    rH, iH = ves.soa_from_complex(M, 1)
    rZ, iZ = ves.soa_from_complex(np.broadcast_to(np.eye(n), (N, n, n)).astype(complex), 1)
    rE, iE = np.zeros(N * n), np.zeros(N * n)
    oracle.restatement().vo_zlahqr(n, N, 1, ptr(rE), ptr(iE), ptr(rH), ptr(iH), ptr(rZ), ptr(iZ), None)
    return ves.complex_vec_from_soa(rE, iE, n, 1)


@pytest.mark.parametrize("deg,N,tc", [(1, 32, 4), (2, 64, 32), (5, 100, 10), (10, 512, 512), (24, 64, 32)])
def test_polyroots(deg, N, tc):
    import torch
    rng = np.random.default_rng(400 + deg)
    C = cgauss(rng, (N, deg + 1))
    rC, iC = ves.soa_vec_from_complex(C, tc)
    dRr = torch.empty(N * deg, dtype=torch.float64, device="cuda")
    dRi = torch.empty_like(dRr)
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    ves.polyroots(deg, N // tc, tc, torch.from_numpy(rC).cuda(), torch.from_numpy(iC).cuda(), dRr, dRi, status=st)
    torch.cuda.synchronize()
    R = ves.complex_vec_from_soa(dRr.cpu().numpy(), dRi.cpu().numpy(), deg, tc)
    assert (st.cpu().numpy() == 0).all()
    # against the oracle's QR on the same companion matrices
    Ro = companion_oracle_roots(C)
    scale = np.abs(C[:, :deg] / C[:, deg:]).sum(axis=1) + 1.0
    _, err, _ = match_eigs(R, Ro)
    assert (err / scale).max() <= 1e-12
    # backward error: |p(r)| relative to sum |c_i| |r|^i
    powers = R[:, :, None] ** np.arange(deg + 1)[None, None, :]
    val = np.abs((powers * C[:, None, :]).sum(axis=2))
    mag = (np.abs(powers) * np.abs(C[:, None, :])).sum(axis=2)
    assert (val / mag).max() <= 1e-12


def test_polyroots_bad_leading_coefficient():
    import torch
    C = np.ones((4, 4), complex)
    C[1, 3] = 0.0
    rC, iC = ves.soa_vec_from_complex(C, 4)
    dRr = torch.empty(4 * 3, dtype=torch.float64, device="cuda")
    dRi = torch.empty_like(dRr)
    st = torch.full((4,), -1, dtype=torch.int32, device="cuda")
    ves.polyroots(3, 1, 4, torch.from_numpy(rC).cuda(), torch.from_numpy(iC).cuda(), dRr, dRi, status=st)
    torch.cuda.synchronize()
    s = st.cpu().numpy()
    assert s[1] & ves.VES_STATUS_NONFINITE and (s[[0, 2, 3]] == 0).all()
    R = ves.complex_vec_from_soa(dRr.cpu().numpy(), dRi.cpu().numpy(), 3, 4)
    assert np.isnan(R[1]).all() and np.isfinite(R[[0, 2, 3]]).all()


@pytest.mark.parametrize("n,N,tc", [(4, 37, 1), (16, 1024, 512), (7, 91, 7), (33, 64, 32)])
def test_device_transposes(n, N, tc):
    import torch
    rng = np.random.default_rng(500 + n)
    A = cgauss(rng, (N, n, n))
    bc = N // tc
    zr = torch.from_numpy(A).cuda()                          # C order (row-major)
    zf = torch.from_numpy(np.ascontiguousarray(A.transpose(0, 2, 1))).cuda()  # Fortran order per matrix
    re = torch.empty(N * n * n, dtype=torch.float64, device="cuda")
    im = torch.empty_like(re)
    want_r, want_i = ves.soa_from_complex(A, tc)
    for z, rm in ((zr, True), (zf, False)):
        ves.soa_from_complex_dev(n, bc, tc, z, re, im, row_major=rm)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(re.cpu().numpy(), want_r)
        np.testing.assert_array_equal(im.cpu().numpy(), want_i)
        back = torch.empty_like(z)
        ves.complex_from_soa_dev(n, bc, tc, re, im, back, row_major=rm)
        torch.cuda.synchronize()
        assert torch.equal(back, z)
    v = cgauss(rng, (N, n))
    vr, vi = ves.soa_vec_from_complex(v, tc)
    dv = torch.from_numpy(v).cuda()
    r2 = torch.empty(N * n, dtype=torch.float64, device="cuda")
    i2 = torch.empty_like(r2)
    ves.soa_vec_from_complex_dev(n, bc, tc, dv, r2, i2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(r2.cpu().numpy(), vr)
    np.testing.assert_array_equal(i2.cpu().numpy(), vi)
    out = torch.empty_like(dv)
    ves.complex_from_soa_vec_dev(n, bc, tc, r2, i2, out)
    torch.cuda.synchronize()
    assert torch.equal(out, dv)


def test_split_batch_equals_one_call():
    """One batch solved as 3 parts of whole SoA blocks (ves_partition_blocks, the
    split each GPU of a multi-GPU job takes) gives the one-call result bit for
    bit: every matrix is solved by the same lane code whatever the launch."""
    import torch
    n, tc, bc = 12, 64, 50
    N = bc * tc
    rng = np.random.default_rng(77)
    A = rng.standard_normal((N, n, n)) + 1j * rng.standard_normal((N, n, n))
    rA, iA = ves.soa_from_complex(A, tc)
    dA = [torch.from_numpy(x).cuda() for x in (rA, iA)]
    whole = [torch.empty(N * n, dtype=torch.float64, device="cuda") for _ in range(2)] + \
            [torch.empty_like(dA[0]) for _ in range(2)]
    ves.eigensolve(n, bc, tc, dA[0], dA[1], *whole)
    parts = [torch.empty_like(t) for t in whole]
    for p in range(3):
        first, nb = ves.partition_blocks(bc, 3, p)
        m0, m1 = first * tc * n * n, (first + nb) * tc * n * n
        v0, v1 = first * tc * n, (first + nb) * tc * n
        ves.eigensolve(n, nb, tc, dA[0][m0:m1], dA[1][m0:m1], parts[0][v0:v1], parts[1][v0:v1],
                       parts[2][m0:m1], parts[3][m0:m1])
    torch.cuda.synchronize()
    for a, b in zip(whole, parts):
        assert torch.equal(a, b)
