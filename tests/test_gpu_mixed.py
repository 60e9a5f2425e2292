"""Mixed-precision form (complex FP32 reduction + QR + back substitution,
FP64 Newton refinement of every eigenpair) against the FP64 oracle.

Same bar as the FP64 path: eigenvalues within 1e-12 ||A||_F of the oracle's
after matching, residual ||A v - lambda v|| / (||A||_F ||v||) <= 1e-13 for
every pair.  Matrices the refinement cannot certify are re-solved in FP64
(status bit VES_STATUS_REFINE_FALLBACK).
"""
import numpy as np
import pytest

import oracle
import ves
import workloads
from gpu_util import run_fused, soa_planes_to_batch, soa_vec_to_batch, device_residuals
from parity import match_eigs, residuals

pytestmark = pytest.mark.gpu
MIX = ves.VES_PREC_FP32_REFINE


def cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def oracle_E(A, tc):
    N, n, _ = A.shape
    rA, iA = ves.soa_from_complex(A, tc)
    rE, iE, *_ = oracle.eigensolve(rA, iA, n, tc)
    return ves.complex_vec_from_soa(rE, iE, n, tc)


@pytest.mark.parametrize("n,N,tc", [(2, 64, 4), (4, 256, 32), (8, 1024, 32), (16, 2048, 512), (24, 512, 32),
                                    (32, 512, 32), (7, 77, 7)])
def test_mixed_matches_oracle(n, N, tc):
    rng = np.random.default_rng(2000 + n)
    A = cgauss(rng, (N, n, n))
    out = run_fused(A, tc, precision=MIX)
    nA = np.linalg.norm(A, axis=(1, 2))
    _, err, _ = match_eigs(out["E"], oracle_E(A, tc))
    assert (err / nA).max() <= 1e-12, (err / nA).max()
    assert residuals(A, out["E"], out["V"]).max() <= 1e-13
    fb = (out["status"] & ves.VES_STATUS_REFINE_FALLBACK) != 0
    assert fb.mean() <= 0.02, fb.mean()
    assert (out["status"] & ~ves.VES_STATUS_REFINE_FALLBACK == 0).all()


@pytest.mark.parametrize("n,N,tc,vnorm", [(10, 96, 32, 0), (1, 64, 32, 0), (2, 96, 8, 0), (5, 160, 32, 1),
                                         (16, 96, 32, 2), (24, 64, 16, 0), (32, 96, 32, 1), (40, 64, 32, 0),
                                         (64, 64, 32, 1), (16, 5000, 40, 0), (32, 5120, 512, 2), (48, 1000, 40, 2)])
def test_mixed_forced_fallback_equals_fp64(n, N, tc, vnorm):
    """With no Newton step allowed nothing can be certified: every matrix goes
    through the FP64 solver and the result is the plain FP64 result bit for
    bit, sweep counts included.  The first list entries (one per warp slot of
    the GPU) go to the warp-per-matrix FP64 kernel (a lane owns two rows and
    columns for n > 32) and the rest (N = 5000, 5120, 1000) to the lane
    kernel."""
    rng = np.random.default_rng(3 + n)
    A = cgauss(rng, (N, n, n))
    A[3] = np.triu(A[3])  # already triangular: the reflectors' trivial branch
    fp64 = run_fused_opts(A, tc, vnorm=vnorm)
    out = run_fused_opts(A, tc, precision=MIX, refine_steps=0, vnorm=vnorm)
    assert ((out["status"] & ves.VES_STATUS_REFINE_FALLBACK) != 0).all()
    np.testing.assert_array_equal(out["status"] & ~ves.VES_STATUS_REFINE_FALLBACK, fp64["status"])
    np.testing.assert_array_equal(out["sweeps"], fp64["sweeps"])
    np.testing.assert_array_equal(out["E"], fp64["E"])
    np.testing.assert_array_equal(out["V"], fp64["V"])


def run_fused_opts(A, tc, **kw):
    import torch
    N, n, _ = A.shape
    bc = N // tc
    rA, iA = ves.soa_from_complex(A, tc)
    d = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    dAr, dAi = d(rA), d(iA)
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda"); dEi = torch.empty_like(dEr)
    dVr, dVi = torch.empty_like(dAr), torch.empty_like(dAi)
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    sw = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    ves.eigensolve(n, bc, tc, dAr, dAi, dEr, dEi, dVr, dVi, status=st, sweeps=sw, options=ves.default_options(**kw))
    torch.cuda.synchronize()
    return dict(E=ves.complex_vec_from_soa(dEr.cpu().numpy(), dEi.cpu().numpy(), n, tc),
                V=ves.complex_from_soa(dVr.cpu().numpy(), dVi.cpu().numpy(), n, tc), status=st.cpu().numpy(),
                sweeps=sw.cpu().numpy())


def test_mixed_nonfinite_and_degenerate():
    rng = np.random.default_rng(5)
    n = 6
    A = cgauss(rng, (64, n, n))
    A[1] = 0
    A[2] = np.eye(n)
    A[3] = np.triu(rng.standard_normal((n, n)))
    A[4, 1, 1] = np.nan
    A[5] *= 1e30  # beyond FP32 range once squared
    out = run_fused(A, 32, precision=MIX)
    assert out["status"][4] & ves.VES_STATUS_NONFINITE
    assert out["status"][5] & ves.VES_STATUS_REFINE_FALLBACK
    good = np.ones(64, bool)
    good[4] = False
    assert np.isfinite(out["E"][good]).all()
    res = residuals(A[good], out["E"][good], out["V"][good])
    zero = np.linalg.norm(A[good], axis=(1, 2)) == 0
    assert res[~zero].max() <= 1e-13


def test_mixed_clustered_spectrum():
    """Eigenvalues 1e-6 apart are below FP32 resolution: the refinement must
    either separate them to FP64 accuracy or hand the matrix to FP64."""
    rng = np.random.default_rng(7)
    n, N = 8, 128
    A = np.empty((N, n, n), complex)
    for k in range(N):
        c = cgauss(rng, 2)
        lam = np.concatenate([c[0] + 1e-6 * cgauss(rng, n // 2), c[1] + 1e-6 * cgauss(rng, n // 2)])
        X = np.eye(n) + 0.3 * cgauss(rng, (n, n))
        A[k] = X @ np.diag(lam) @ np.linalg.inv(X)
    out = run_fused(A, 32, precision=MIX)
    assert residuals(A, out["E"], out["V"]).max() <= 1e-13
    _, err, _ = match_eigs(out["E"], oracle_E(A, 32))
    assert (err / np.linalg.norm(A, axis=(1, 2))).max() <= 1e-12


@pytest.mark.parametrize("vnorm", [0, 2])
def test_mixed_vector_scaling(vnorm):
    rng = np.random.default_rng(11)
    A = cgauss(rng, (128, 12, 12))
    ref = run_fused(A, 32, vnorm=vnorm)
    out = run_fused(A, 32, vnorm=vnorm, precision=MIX)
    perm, err, same = match_eigs(out["E"], ref["E"])
    Vm = np.take_along_axis(out["V"], perm[:, None, :], axis=2)
    ratio = np.linalg.norm(Vm, axis=1) / np.linalg.norm(ref["V"], axis=1)
    if vnorm == 2:
        assert np.abs(ratio - 1).max() <= 1e-14
    else:
        # the reference scaling (unit component along the k-th Schur vector)
        # depends on the Schur order, and the FP32 QR deflates at FP32
        # precision, so its order often differs from the FP64 run's; where the
        # two orders agree the scaling holds to FP32 accuracy
        assert same.any()
        assert np.abs(ratio[same] - 1).max() <= 1e-4


@pytest.mark.slow
def test_mixed_fullsize_n32():
    """262,144 x 32x32 (seed 3): every pair certified on the device; eigenvalues
    against the oracle on the first 16,384; FP64 path as the comparison."""
    import torch
    w = workloads.WORKLOADS["gauss32"]
    N, n, tc = w["N"], w["n"], 512
    rA, iA = workloads.gaussian_soa(N, n, w["seed"], tc)
    dAr, dAi = torch.from_numpy(rA).cuda(), torch.from_numpy(iA).cuda()
    outs = {}
    for prec in (0, MIX):
        dEr = torch.empty(N * n, dtype=torch.float64, device="cuda"); dEi = torch.empty_like(dEr)
        dVr, dVi = torch.empty_like(dAr), torch.empty_like(dAi)
        st = torch.zeros(N, dtype=torch.int32, device="cuda")
        ves.eigensolve(n, N // tc, tc, dAr, dAi, dEr, dEi, dVr, dVi, status=st,
                       options=ves.default_options(precision=prec))
        torch.cuda.synchronize()
        A = soa_planes_to_batch(dAr, dAi, n, tc)
        res = device_residuals(A, soa_vec_to_batch(dEr, dEi, n, tc), soa_planes_to_batch(dVr, dVi, n, tc))
        assert float(res.max()) <= 1e-13
        outs[prec] = (dEr[: 16384 * n].cpu().numpy(), dEi[: 16384 * n].cpu().numpy(), st)
    fb = int(((outs[MIX][2] & ves.VES_STATUS_REFINE_FALLBACK) != 0).sum())
    assert fb <= N // 100
    k = 16384 * n * n
    rE, iE, *_ = oracle.eigensolve(rA[:k], iA[:k], n, tc)
    Eo = ves.complex_vec_from_soa(rE, iE, n, tc)
    nA = np.linalg.norm(ves.complex_from_soa(rA[:k], iA[:k], n, tc), axis=(1, 2))
    for prec in (0, MIX):
        E = ves.complex_vec_from_soa(outs[prec][0], outs[prec][1], n, tc)
        _, err, _ = match_eigs(E, Eo)
        assert (err / nA).max() <= 1e-12


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9, 12, 16, 24, 31, 32])
@pytest.mark.parametrize("mode", ["lane", "warp", "warp32", "group4", "group8"])
def test_mixed_schur_kernels(n, mode, monkeypatch):
    """Every FP32 Schur kernel (lane per matrix; a matrix per group of 4 or 8
    lanes, per half warp or per warp, in shared memory) meets the bar, with
    thread_cnt not a multiple of the warp and a batch (203) that is not a
    multiple of a block's matrices, so the last warp's groups are partly
    empty."""
    if mode == "warp32" and n > 16:
        pytest.skip("the same kernel as mode warp for n > 16")
    if mode.startswith("group") and n > 16:
        pytest.skip("the group kernels take n <= 16")
    if n == 1 and mode != "lane" and not mode.startswith("group"):
        pytest.skip("covered by the lane and group kernels")
    monkeypatch.setenv("VES_MIXED_SCHUR", mode)
    rng = np.random.default_rng(4000 + n)
    N, tc = 203, 7
    A = cgauss(rng, (N, n, n))
    A[5] = np.triu(A[5])                        # already triangular
    A[6] = np.diag(np.arange(1, n + 1)) + 0j    # diagonal, distinct
    A[7, :, :] = 0                              # zero matrix
    out = run_fused(A, tc, precision=MIX)
    nA = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1.0)
    # the oracle restates the reference's zgehrd, which divides by zero on
    # already-reduced columns (NaN for triangular input): LAPACK for those
    special = [5, 6, 7]
    Eref = oracle_E(A, tc)
    Eref[special] = np.linalg.eigvals(A[special])
    _, err, _ = match_eigs(out["E"], Eref)
    assert (err / nA).max() <= 1e-12, (err / nA).max()
    assert residuals(A, out["E"], out["V"]).max() <= 1e-13
    assert (out["status"] & ~ves.VES_STATUS_REFINE_FALLBACK == 0).all()


@pytest.mark.parametrize("n,N", [(8, 50688), (24, 33280)])
def test_mixed_overlap_equals_serial(n, N, monkeypatch):
    """The FP32+refine form cuts large batches into chunks and overlaps one
    chunk's Schur stage with the previous chunk's refinement on two streams;
    the results equal the serial launch order bit for bit (n = 8: the lane
    Schur kernel, n = 24: the warp one; unequal last chunk)."""
    import torch
    tc = 512
    rA, iA = workloads.gaussian_soa(N, n, 17, tc)
    dA = [torch.from_numpy(x).cuda() for x in (rA, iA)]
    outs = []
    for ov in ("1", "0"):
        monkeypatch.setenv("VES_MIXED_OVERLAP", ov)
        dE = [torch.empty(N * n, dtype=torch.float64, device="cuda") for _ in range(2)]
        dV = [torch.empty_like(dA[0]) for _ in range(2)]
        st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
        ves.eigensolve(n, N // tc, tc, dA[0], dA[1], dE[0], dE[1], dV[0], dV[1], status=st,
                       options=ves.default_options(precision=MIX))
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in dE + dV + [st]])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
    assert ((outs[0][4] & ~ves.VES_STATUS_REFINE_FALLBACK) == 0).all()


def _unitary(rng, n):
    q, r = np.linalg.qr(cgauss(rng, (n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_mixed_close_clusters_no_duplicate_eigenvalues():
    """Normal matrices whose eigenvalues come in clusters 1e-9 ||A||_F wide:
    far below FP32 resolution, so Newton from the FP32 Schur form can bring
    two pairs to one eigenvalue.  Every true eigenvalue must still be found to
    1e-12 ||A||_F (a duplicate would leave one ~1e-9 away), either by the
    refinement or by the FP64 solve the distinctness check hands it to."""
    rng = np.random.default_rng(23)
    n, N, tc = 16, 256, 32
    A = np.empty((N, n, n), complex)
    lam = np.empty((N, n), complex)
    for k in range(N):
        centres = cgauss(rng, 4)
        off = cgauss(rng, n) / np.sqrt(2)
        lam[k] = np.repeat(centres, n // 4) + 1e-9 * np.linalg.norm(centres) * off
        U = _unitary(rng, n)
        A[k] = U @ np.diag(lam[k]) @ U.conj().T
    out = run_fused(A, tc, precision=MIX)
    nA = np.linalg.norm(A, axis=(1, 2))
    _, err, _ = match_eigs(out["E"], lam)
    assert (err / nA).max() <= 1e-12, (err / nA).max()
    assert residuals(A, out["E"], out["V"]).max() <= 1e-13
    assert (out["status"] & ~ves.VES_STATUS_REFINE_FALLBACK == 0).all()


def test_mixed_work_counters():
    """work_counts: two float-float residuals per refined pair (the ones that
    drive the first two corrections), at least one FP64 residual (the one that
    accepts) and two corrections per pair; no polish steps in this form."""
    import torch
    rng = np.random.default_rng(31)
    n, N, tc = 12, 512, 32
    A = cgauss(rng, (N, n, n))
    wc = torch.zeros(ves.VES_WORK_COUNTS, dtype=torch.int64, device="cuda")
    out = run_fused(A, tc, precision=MIX, work_counts=wc)
    fb = int(((out["status"] & ves.VES_STATUS_REFINE_FALLBACK) != 0).sum())
    res64, corr, ff, polish = (int(x) for x in wc.cpu())
    pairs = (N - fb) * n
    assert ff == 2 * pairs
    assert pairs <= res64 <= 7 * pairs and 3 * pairs <= corr <= 9 * pairs
    assert polish == 0


def test_mixed_concurrent_callers(monkeypatch):
    """Two host threads, each with its own stream and workspace, run the
    FP32+refine form at once on the overlapped two-stream path (forced on;
    the threads share its library streams): each gets the result of a call
    made alone, bit for bit."""
    import threading

    import torch
    monkeypatch.setenv("VES_MIXED_OVERLAP", "1")
    n, N, tc = 8, 65536, 512
    batches = [workloads.gaussian_soa(N, n, s, tc) for s in (41, 42)]
    opt = ves.default_options(precision=MIX)

    def solve(b, stream, out, idx):
        with torch.cuda.stream(stream):
            dA = [torch.from_numpy(x).cuda() for x in b]
            dE = [torch.empty(N * n, dtype=torch.float64, device="cuda") for _ in range(2)]
            dV = [torch.empty_like(dA[0]) for _ in range(2)]
            ws = ves.Workspace(n, N // tc, tc, opt)
            for _ in range(3):
                ves.eigensolve(n, N // tc, tc, dA[0], dA[1], dE[0], dE[1], dV[0], dV[1], options=opt, workspace=ws,
                               stream=stream)
            stream.synchronize()
            out[idx] = [t.cpu().numpy() for t in dE + dV]

    alone = [None, None]
    for i, b in enumerate(batches):
        solve(b, torch.cuda.Stream(), alone, i)
    together = [None, None]
    ths = [threading.Thread(target=solve, args=(b, torch.cuda.Stream(), together, i)) for i, b in enumerate(batches)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for i in range(2):
        for a, b in zip(alone[i], together[i]):
            np.testing.assert_array_equal(a, b)


def test_mixed_graph_capture(monkeypatch):
    """A FP32+refine call captured in a CUDA graph (it stays on the capturing
    stream instead of forking the shared library streams, which it would do
    uncaptured: overlap forced on) replays to the result of a direct call, bit
    for bit."""
    import torch
    monkeypatch.setenv("VES_MIXED_OVERLAP", "1")
    n, N, tc = 8, 65536, 512
    rA, iA = workloads.gaussian_soa(N, n, 43, tc)
    dA = [torch.from_numpy(x).cuda() for x in (rA, iA)]
    opt = ves.default_options(precision=MIX)
    ws = ves.Workspace(n, N // tc, tc, opt)
    outs = []
    for captured in (False, True):
        dE = [torch.zeros(N * n, dtype=torch.float64, device="cuda") for _ in range(2)]
        dV = [torch.zeros_like(dA[0]) for _ in range(2)]
        st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
        call = lambda: ves.eigensolve(n, N // tc, tc, dA[0], dA[1], dE[0], dE[1], dV[0], dV[1], status=st,  # noqa
                                      options=opt, workspace=ws, stream=torch.cuda.current_stream())
        if captured:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                call()
            g.replay()
        else:
            call()
        torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in dE + dV + [st]])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
