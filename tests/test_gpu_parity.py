"""Parity of the sm_103a eigensolver (libves.so) with the oracle and with the
reference's own outputs.

Tolerances (the bar every form meets, floating point):
  eigenvalues, after optimal matching:      |lambda - lambda_ref| <= 1e-12 * ||A||_F
  normalised residual per eigenpair:        ||A v - lambda v|| / (||A||_F ||v||) <= 1e-13
Eigenvectors are compared up to a unit phase (the Schur basis is unique only
up to column phases), scaled by the eigenvalue separation.
"""
import os

import numpy as np
import pytest

import oracle
import ves
from gpu_util import run_fused, dev
from parity import match_eigs, residuals, vec_phase_err, separation

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-12
RES_TOL = 1e-13
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz")


def cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def oracle_solve(A, tc):
    N, n, _ = A.shape
    rA, iA = ves.soa_from_complex(A, tc)
    rE, iE, rV, iV, rT, iT, sw = oracle.eigensolve(rA, iA, n, tc)
    return (ves.complex_vec_from_soa(rE, iE, n, tc), ves.complex_from_soa(rV, iV, n, tc),
            ves.complex_from_soa(rT, iT, n, tc), sw)


def check_against_oracle(A, tc, out, order_frac=0.98):
    Eo, Vo, To, swo = oracle_solve(A, tc)
    nA = np.linalg.norm(A, axis=(1, 2))
    perm, err, same = match_eigs(out["E"], Eo)
    assert (err / nA).max() <= EIG_TOL, (err / nA).max()
    res = residuals(A, out["E"], out["V"])
    assert res.max() <= RES_TOL, res.max()
    # same algorithm, same shifts: the Schur order agrees for (almost) every
    # matrix, and the sweep counts up to rounding-borderline deflation tests
    assert same.mean() >= order_frac, same.mean()
    assert (np.abs(out["sweeps"] - swo) <= 1).mean() >= order_frac
    assert np.abs(out["sweeps"].mean() - swo.mean()) <= 0.05 * max(swo.mean(), 1.0)
    # eigenvectors agree up to phase where eigenvalues are separated; with the
    # reference scaling their norms agree as well
    Vm = np.take_along_axis(out["V"], perm[:, None, :], axis=2)
    sep = separation(Eo) / nA[:, None]
    well = sep > 1e-3
    pe = vec_phase_err(Vm, Vo)
    assert (pe[well] <= 1e-9 / sep[well]).all(), (pe[well] * sep[well]).max()
    nr = np.linalg.norm(Vm, axis=1) / np.linalg.norm(Vo, axis=1)
    assert np.abs(nr[well] - 1).max() <= 1e-8


@pytest.mark.parametrize("n,N,tc", [
    (1, 40, 4), (2, 64, 4), (3, 96, 32), (4, 100, 1), (5, 77, 7), (8, 2048, 4), (12, 512, 512),
    (16, 4096, 512), (16, 1000, 8), (24, 512, 32), (32, 512, 32), (33, 96, 32), (48, 64, 16), (64, 64, 32),
])
def test_fused_matches_oracle(n, N, tc):
    rng = np.random.default_rng(1000 + n)
    A = cgauss(rng, (N, n, n))
    out = run_fused(A, tc)
    assert (out["status"] == 0).all()
    check_against_oracle(A, tc, out)


def test_fused_schur_form_output():
    rng = np.random.default_rng(5)
    n, N, tc = 16, 256, 32
    A = cgauss(rng, (N, n, n))
    out = run_fused(A, tc, want_T=True)
    T = out["T"]
    assert np.abs(np.tril(T, -1)).max() == 0.0
    np.testing.assert_array_equal(np.diagonal(T, axis1=1, axis2=2), out["E"])
    _, _, To, _ = oracle_solve(A, tc)
    # |T| is invariant to the Schur basis phases
    np.testing.assert_allclose(np.abs(T), np.abs(To), atol=1e-11 * np.abs(To).max())


@pytest.mark.parametrize("vnorm", [1, 2])
def test_vector_scaling_options(vnorm):
    rng = np.random.default_rng(9)
    A = cgauss(rng, (128, 8, 8))
    ref = run_fused(A, 32)
    out = run_fused(A, 32, vnorm=vnorm)
    np.testing.assert_array_equal(out["E"], ref["E"])
    if vnorm == 1:
        np.testing.assert_allclose((np.abs(out["V"].real) + np.abs(out["V"].imag)).max(axis=1), 1.0, atol=1e-14)
    else:
        np.testing.assert_allclose(np.linalg.norm(out["V"], axis=1), 1.0, atol=1e-14)
    assert residuals(A, out["E"], out["V"]).max() <= RES_TOL


# --------------------------- edge cases -----------------------------------
def test_structured_and_degenerate_inputs():
    n = 6
    rng = np.random.default_rng(2)
    upper = np.triu(cgauss(rng, (1, n, n)))[0]
    real_upper = np.triu(rng.standard_normal((n, n)))
    cases = [np.zeros((n, n), complex), np.eye(n, dtype=complex), np.diag(np.arange(1, n + 1)).astype(complex),
             upper, real_upper.astype(complex), np.triu(real_upper, -1).astype(complex),
             np.diag(np.ones(n - 1), 1).astype(complex)]  # a nilpotent Jordan block
    A = np.stack(cases + [cgauss(rng, (n, n))] * (32 - len(cases)))
    out = run_fused(A, 32)
    assert np.isfinite(out["E"]).all() and np.isfinite(out["V"]).all()
    w = np.linalg.eigvals(A)
    _, err, _ = match_eigs(out["E"], w)
    nA = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1.0)
    jordan = len(cases) - 1
    ok = np.ones(32, bool)
    ok[jordan] = False  # eigenvalue 0 of a Jordan block is ill-posed (sensitivity eps^(1/n))
    assert (err[ok] / nA[ok]).max() <= EIG_TOL
    # the reference's reflector sign divides by zero on already-reduced real
    # columns (its zgehrd gives NaN for a real triangular input); here every
    # output is finite and the triangular cases keep their diagonal
    np.testing.assert_allclose(np.sort_complex(out["E"][4]), np.sort_complex(np.diag(real_upper).astype(complex)),
                               atol=1e-13 * np.abs(real_upper).max())


@pytest.mark.parametrize("precision", [0, 1])
def test_hermitian_and_unitary_inputs(precision):
    """Normal matrices: Hermitian (real spectrum) and unitary (spectrum on the
    unit circle); eigenvalues within the bar, every residual within the bar,
    eigenvectors of separated eigenvalues orthogonal."""
    rng = np.random.default_rng(5)
    n, N = 12, 64
    G = cgauss(rng, (N, n, n))
    herm = (G + np.conj(np.swapaxes(G, 1, 2))) / 2
    Q, _ = np.linalg.qr(cgauss(rng, (N, n, n)))
    A = np.concatenate([herm[:32], Q[:32]])
    out = run_fused(A, 32, precision=precision)
    w = np.linalg.eigvals(A)
    _, err, _ = match_eigs(out["E"], w)
    nA = np.linalg.norm(A, axis=(1, 2))
    assert (err / nA).max() <= EIG_TOL
    assert np.abs(out["E"][:32].imag).max() <= 1e-13 * nA[:32].max()
    np.testing.assert_allclose(np.abs(out["E"][32:]), 1.0, atol=1e-13)
    assert residuals(A, out["E"], out["V"]).max() <= RES_TOL
    V = out["V"] / np.linalg.norm(out["V"], axis=1, keepdims=True)
    gram = np.abs(np.conj(np.swapaxes(V, 1, 2)) @ V - np.eye(n))
    well = separation(w) / nA[:, None] > 1e-3
    for m in range(N):
        if well[m].all():
            assert gram[m].max() <= 1e-9


def test_nonfinite_input_flagged():
    rng = np.random.default_rng(4)
    A = cgauss(rng, (64, 5, 5))
    A[3, 2, 1] = np.nan
    A[40, 0, 0] = np.inf
    out = run_fused(A, 32)
    assert out["status"][3] & ves.VES_STATUS_NONFINITE and out["status"][40] & ves.VES_STATUS_NONFINITE
    good = np.ones(64, bool)
    good[[3, 40]] = False
    assert (out["status"][good] == 0).all()
    assert residuals(A[good], out["E"][good], out["V"][good]).max() <= RES_TOL


def test_iteration_cap_is_reported_not_hung():
    rng = np.random.default_rng(8)
    A = cgauss(rng, (64, 12, 12))
    out = run_fused(A, 32, max_its=0)  # one sweep per eigenvalue
    assert (out["status"] & ves.VES_STATUS_ITCAP).any()
    assert (out["sweeps"] <= 12).all()


def test_empty_and_ragged_batches():
    import torch
    z = torch.zeros(16, dtype=torch.float64, device="cuda")
    ves.eigensolve(4, 0, 4, z, z, z, z, z, z)  # empty batch: no-op
    rng = np.random.default_rng(6)
    A = cgauss(rng, (37, 7, 7))  # 37 matrices: one full warp group and a ragged one
    out = run_fused(A, 37)
    check_against_oracle(A, 37, out)
    out1 = run_fused(A, 1)  # thread_cnt = 1 (matrices stored one after another)
    np.testing.assert_array_equal(out1["E"], out["E"])


def test_large_dim():
    rng = np.random.default_rng(12)
    A = cgauss(rng, (32, 128, 128))
    out = run_fused(A, 32)
    assert residuals(A, out["E"], out["V"]).max() <= RES_TOL
    _, err, _ = match_eigs(out["E"], np.linalg.eigvals(A))
    assert (err / np.linalg.norm(A, axis=(1, 2))).max() <= EIG_TOL


def test_argument_errors():
    import torch
    z = torch.zeros(64, dtype=torch.float64, device="cuda")
    with pytest.raises(ves.VesError):
        ves.eigensolve(0, 1, 4, z, z, z, z, z, z)
    with pytest.raises(ves.VesError):
        ves.eigensolve(4, 1, 4, z, z, z, z, z, z, options=ves.default_options(vnorm=7))


# ------------------- drop-in entry points vs reference outputs -------------------
@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def gcases(g):
    return sorted({k.split("/")[0] for k in g.files})


def test_dropin_eigensolver_vs_reference(gold):
    for c in gcases(gold):
        n, bc, tc = (int(x) for x in gold[c + "/dims"])
        N = bc * tc
        rA, iA = gold[c + "/rA"].copy(), gold[c + "/iA"].copy()
        A = ves.complex_from_soa(rA, iA, n, tc)
        rE, iE = np.zeros(N * n), np.zeros(N * n)
        rV, iV = np.zeros_like(rA), np.zeros_like(iA)
        ves.eigensolver(n, bc, tc, rA, iA, rE, iE, rV, iV)
        E = ves.complex_vec_from_soa(rE, iE, n, tc)
        V = ves.complex_from_soa(rV, iV, n, tc)
        Eref = ves.complex_vec_from_soa(gold[c + "/eig_rE"], gold[c + "/eig_iE"], n, tc)
        _, err, same = match_eigs(E, Eref)
        nA = np.linalg.norm(A, axis=(1, 2))
        assert (err / nA).max() <= EIG_TOL
        assert same.all()
        assert residuals(A, E, V).max() <= RES_TOL
        Vref = ves.complex_from_soa(gold[c + "/eig_rV"], gold[c + "/eig_iV"], n, tc)
        well = separation(Eref) / nA[:, None] > 1e-3
        assert (vec_phase_err(V, Vref)[well] <= 1e-8).all()
        # A is overwritten with the Schur form (upper triangular, eigenvalues on the diagonal)
        T = ves.complex_from_soa(rA, iA, n, tc)
        assert np.abs(np.tril(T, -1)).max() == 0.0
        np.testing.assert_array_equal(np.diagonal(T, axis1=1, axis2=2), E)


def _unitary_err(Q):
    n = Q.shape[-1]
    return np.abs(np.conj(np.swapaxes(Q, 1, 2)) @ Q - np.eye(n)).max()


def test_dropin_zgehrd_hessenberg_zunghr(gold):
    for c in gcases(gold):
        n, bc, tc = (int(x) for x in gold[c + "/dims"])
        N = bc * tc
        A = ves.complex_from_soa(gold[c + "/rA"], gold[c + "/iA"], n, tc)
        s = np.linalg.norm(A, axis=(1, 2)).max()
        # hessenberg(): A = Q H Q^H; |H| equals the reference's (the reflector
        # sign only changes H by a diagonal unitary similarity)
        rA, iA = gold[c + "/rA"].copy(), gold[c + "/iA"].copy()
        rQ, iQ = np.zeros_like(rA), np.zeros_like(iA)
        ves.hessenberg(n, bc, tc, rA, iA, rQ, iQ)
        H = np.triu(ves.complex_from_soa(rA, iA, n, tc), -1)
        Q = ves.complex_from_soa(rQ, iQ, n, tc)
        assert _unitary_err(Q) <= 1e-13 * n
        assert np.abs(Q @ H @ np.conj(np.swapaxes(Q, 1, 2)) - A).max() <= 1e-13 * s
        Href = np.triu(ves.complex_from_soa(gold[c + "/hess_rH"], gold[c + "/hess_iH"], n, tc), -1)
        np.testing.assert_allclose(np.abs(H), np.abs(Href), atol=1e-12 * s)
        # call_zgehrd then call_zunghr gives the same H and Q
        rA2, iA2 = gold[c + "/rA"].copy(), gold[c + "/iA"].copy()
        rt, it = np.zeros(N * n), np.zeros(N * n)
        ves.call_zgehrd(n, bc, tc, rA2, iA2, rt, it)
        np.testing.assert_array_equal(rA2, rA)
        np.testing.assert_array_equal(iA2, iA)
        ves.call_zunghr(n, bc, tc, rA2, iA2, rt, it)
        np.testing.assert_array_equal(rA2, rQ)
        np.testing.assert_array_equal(iA2, iQ)


def test_dropin_zlahqr_ztrevc_vs_reference(gold):
    for c in gcases(gold):
        n, bc, tc = (int(x) for x in gold[c + "/dims"])
        N = bc * tc
        H0 = ves.complex_from_soa(gold[c + "/zlahqr_rH"], gold[c + "/zlahqr_iH"], n, tc)
        rH, iH = gold[c + "/zlahqr_rH"].copy(), gold[c + "/zlahqr_iH"].copy()
        rE, iE = np.zeros(N * n), np.zeros(N * n)
        rS, iS = np.full_like(rH, 7.0), np.full_like(iH, 7.0)  # ignored: reset to I
        ves.call_zlahqr_new(n, bc, tc, rE, iE, rH, iH, rS, iS)
        E = ves.complex_vec_from_soa(rE, iE, n, tc)
        Eref = ves.complex_vec_from_soa(gold[c + "/zlahqr_rE"], gold[c + "/zlahqr_iE"], n, tc)
        s = np.linalg.norm(H0, axis=(1, 2))
        _, err, same = match_eigs(E, Eref)
        assert (err / s).max() <= EIG_TOL and same.all()
        T = ves.complex_from_soa(rH, iH, n, tc)
        S = ves.complex_from_soa(rS, iS, n, tc)
        Tref = ves.complex_from_soa(gold[c + "/zlahqr_rT"], gold[c + "/zlahqr_iT"], n, tc)
        # A Schur form is unique only up to a diagonal unitary similarity, and
        # this algorithm fixes those phases from subdiagonals that have
        # converged to rounding level ("make H(I,I-1) real"), so two correct
        # implementations that round differently differ by such phases.
        # Compare the invariants: |T|, S unitary, S T S^H = M.
        assert np.abs(np.tril(T, -1)).max() == 0.0
        np.testing.assert_allclose(np.abs(T), np.abs(Tref), atol=1e-11 * s.max())
        assert _unitary_err(S) <= 1e-13 * n
        assert np.abs(S @ T @ np.conj(np.swapaxes(S, 1, 2)) - H0).max() <= 1e-13 * s.max()
        # ztrevc on the reference's own (T, S): same algorithm, same inputs
        rT, iT = gold[c + "/zlahqr_rT"].copy(), gold[c + "/zlahqr_iT"].copy()
        rR, iR = gold[c + "/zlahqr_rS"].copy(), gold[c + "/zlahqr_iS"].copy()
        ves.call_ztrevc(n, bc, tc, rT, iT, rR, iR)
        np.testing.assert_array_equal(rT, gold[c + "/zlahqr_rT"])  # T is read only here
        R = ves.complex_from_soa(rR, iR, n, tc)
        Rref = ves.complex_from_soa(gold[c + "/ztrevc_rR"], gold[c + "/ztrevc_iR"], n, tc)
        sc = np.abs(Rref).max()
        np.testing.assert_allclose(R, Rref, atol=1e-11 * sc)


def test_dropin_zgemv_backsubs_vs_reference(gold):
    for c in gcases(gold):
        n, bc, tc = (int(x) for x in gold[c + "/dims"])
        g = lambda k: gold[c + "/" + k].copy()  # noqa: E731
        yr, yi = g("zgemv_ry0"), g("zgemv_iy0")
        ves.call_zgemv(False, n, bc, tc, g("zgemv_rM"), g("zgemv_iM"), g("zgemv_rx"), g("zgemv_ix"), yr, yi, 0.5, -0.25)
        np.testing.assert_allclose(yr, gold[c + "/zgemv_n_ry"], atol=1e-13 * n)
        np.testing.assert_allclose(yi, gold[c + "/zgemv_n_iy"], atol=1e-13 * n)
        yr, yi = g("zgemv_ry0"), g("zgemv_iy0")
        ves.call_zgemv(True, n, bc, tc, g("zgemv_rM"), g("zgemv_iM"), g("zgemv_rx"), g("zgemv_ix"), yr, yi, 0.0, 0.0)
        np.testing.assert_allclose(yr, gold[c + "/zgemv_h_ry"], atol=1e-13 * n)
        np.testing.assert_allclose(yi, gold[c + "/zgemv_h_iy"], atol=1e-13 * n)
        br, bi = g("bs_rb"), g("bs_ib")
        ves.call_backsubstitution(n, bc, tc, g("bs_rT"), g("bs_iT"), br, bi)
        np.testing.assert_allclose(br, gold[c + "/bs_rx"], atol=1e-12)
        np.testing.assert_allclose(bi, gold[c + "/bs_ix"], atol=1e-12)


def test_zgemv_hermitian_with_complex_y():
    """The reference's Hermitian branch reads Re(y) for Im(y) (Toolbox.hpp:1125);
    here it computes M^H x + beta y correctly."""
    rng = np.random.default_rng(21)
    n, bc, tc = 5, 2, 4
    N = bc * tc
    M = cgauss(rng, (N, n, n)); x = cgauss(rng, (N, n)); y = cgauss(rng, (N, n))
    mr, mi = ves.soa_from_complex(M, tc)
    xr, xi = ves.soa_vec_from_complex(x, tc)
    yr, yi = ves.soa_vec_from_complex(y, tc)
    ves.call_zgemv(True, n, bc, tc, mr, mi, xr, xi, yr, yi, 1.0, 0.5)
    got = ves.complex_vec_from_soa(yr, yi, n, tc)
    want = np.einsum("kij,ki->kj", np.conj(M), x) + (1.0 + 0.5j) * y
    np.testing.assert_allclose(got, want, atol=1e-13)


# ---------------- the reference's own Python test helpers -----------------
def test_reference_python_helpers():
    import python_interface as pi
    np.random.seed(0)
    for dim, bc, tc in ((8, 2, 4), (12, 1, 32), (3, 4, 1)):
        assert np.abs(pi.test_backsubs(dim, bc, tc)).max() < 1e-10
        for herm in (False, True):
            assert pi.test_zgemv(dim, bc, tc, herm).max() < 1e-13
        h, q, a = pi.test_hessenberg(dim, bc, tc)
        assert np.abs(q @ np.triu(h, -1) @ q.conj().T - a).max() < 1e-13 * dim
        eigs, z, t, a = pi.test_zlahqr(dim, bc, tc)
        assert np.abs(z @ t @ z.conj().T - a).max() < 1e-13 * dim
        _, err, _ = match_eigs(eigs[None], np.linalg.eigvals(a)[None])
        assert err.max() < 1e-12 * np.linalg.norm(a)
        eigs, vecs, a = pi.test_eigenvectors(dim, bc, tc)
        assert residuals(a[None].astype(complex), eigs[None], vecs[None]).max() < RES_TOL
        erg, a = pi.test_zgehrd(dim, bc, tc)
        assert erg.shape == (dim, dim)


def test_device_stage_entry_points():
    """The ves_* stage entry points on device buffers agree with the drop-ins."""
    import torch
    rng = np.random.default_rng(31)
    n, bc, tc = 9, 4, 32
    N = bc * tc
    A = cgauss(rng, (N, n, n))
    rA, iA = ves.soa_from_complex(A, tc)
    dr, di = dev(rA), dev(iA)
    tr = torch.zeros(N * n, dtype=torch.float64, device="cuda"); ti = torch.zeros_like(tr)
    ves.zgehrd_dev(n, bc, tc, dr, di, tr, ti)
    hr, hi = rA.copy(), iA.copy()
    t2r, t2i = np.zeros(N * n), np.zeros(N * n)
    ves.call_zgehrd(n, bc, tc, hr, hi, t2r, t2i)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dr.cpu().numpy(), hr)
    ves.zunghr_dev(n, bc, tc, dr, di, tr, ti)
    ves.call_zunghr(n, bc, tc, hr, hi, t2r, t2i)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dr.cpu().numpy(), hr)


@pytest.mark.parametrize("chunks", [None, "7"])
def test_dropin_pipeline_chunks_equal_one_launch(chunks, monkeypatch):
    """The drop-in eigensolver() splits a large batch into chunks of SoA blocks
    solved on two streams; its results equal one device launch bit for bit
    (unequal chunks: by default 3 chunks of 141, 141 and 139 blocks; with
    VES_DROPIN_CHUNKS=7, six of 61 and one of 55)."""
    import torch
    import workloads
    if chunks:
        monkeypatch.setenv("VES_DROPIN_CHUNKS", chunks)
    n, tc, bc = 4, 512, 421
    N = bc * tc
    rA, iA = workloads.gaussian_soa(N, n, seed=11, thread_cnt=tc)
    dA = [torch.from_numpy(x).cuda() for x in (rA, iA)]
    dE = [torch.empty(N * n, dtype=torch.float64, device="cuda") for _ in range(2)]
    dV = [torch.empty_like(dA[0]) for _ in range(2)]
    dT = [torch.empty_like(dA[0]) for _ in range(2)]
    ves.eigensolve(n, bc, tc, dA[0], dA[1], dE[0], dE[1], dV[0], dV[1], rT=dT[0], iT=dT[1])
    torch.cuda.synchronize()
    hA = [rA.copy(), iA.copy()]
    hE = [np.zeros(N * n) for _ in range(2)]
    hV = [np.zeros_like(rA) for _ in range(2)]
    ves.eigensolver(n, bc, tc, hA[0], hA[1], hE[0], hE[1], hV[0], hV[1])
    for h, d in zip(hE + hV + hA, dE + dV + dT):
        np.testing.assert_array_equal(h, d.cpu().numpy())
