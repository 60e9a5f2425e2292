"""Learned shifts: whatever the predictions, the solve meets the same bar as
the plain FP64 solver (the reference's shifts take over after the first
sweep); good predictions cut the sweep count; the network trains, predicts,
and round-trips through its checkpoint."""
import os
import tempfile

import numpy as np
import pytest

import learned_shift
import ves
from gpu_util import soa_planes_to_batch, soa_vec_to_batch, device_residuals
from parity import match_eigs

pytestmark = pytest.mark.gpu
TC = 512


def solve_shifts(n, N, rA, iA, rS, iS, **opt):
    import torch
    rE = torch.empty(N * n, dtype=torch.float64, device="cuda")
    iE = torch.empty_like(rE)
    rV, iV = torch.empty_like(rA), torch.empty_like(iA)
    st = torch.zeros(N, dtype=torch.int32, device="cuda")
    sw = torch.zeros(N, dtype=torch.int32, device="cuda")
    fb = torch.zeros(N, dtype=torch.int32, device="cuda")
    ves.eigensolve_shifts(n, N // TC, TC, rA, iA, rE, iE, rV, iV, rS, iS, status=st, sweeps=sw, fallbacks=fb,
                          options=ves.default_options(**opt))
    torch.cuda.synchronize()
    res = device_residuals(soa_planes_to_batch(rA, iA, n, TC), soa_vec_to_batch(rE, iE, n, TC),
                           soa_planes_to_batch(rV, iV, n, TC))
    return rE, iE, st, sw, fb, float(res.max())


@pytest.mark.parametrize("n", [8, 16, 24])
def test_exact_and_garbage_predictions(n):
    import torch
    N = 4096
    p, rA, iA = learned_shift.family(N, n, param_seed=11)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC)
    E0 = ves.complex_vec_from_soa(rE0.cpu().numpy(), iE0.cpu().numpy(), n, TC)
    nA = np.linalg.norm(ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC), axis=(1, 2))
    # exact eigenvalues as predictions: same spectrum, fewer sweeps
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, rE0, iE0)
    assert res <= 1e-13
    _, err, _ = match_eigs(ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC), E0)
    assert (err / nA).max() <= 1e-12
    assert sw.double().mean().item() < 0.8 * sw0.double().mean().item()
    # useless predictions (all far away): still correct, fallbacks reported
    far = torch.full_like(rE0, 100.0)
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, far, torch.zeros_like(far))
    assert res <= 1e-13
    _, err, _ = match_eigs(ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC), E0)
    assert (err / nA).max() <= 1e-12
    assert fb.sum().item() > 0 and ((st & ves.VES_STATUS_SHIFT_FALLBACK) != 0).any()


@pytest.mark.parametrize("subdiag", [0, 1])
def test_train_predict_checkpoint(subdiag):
    """Training lowers the loss and beats the trivial diag(A) guess; a saved
    checkpoint (with or without the subdiagonal-norm features) predicts the
    same bits after loading."""
    import torch
    n, N = 8, 16384
    net, losses = learned_shift.train(n, count=N, epochs=8, batch=512, lr=2e-3, hidden=128, param_seed=21,
                                      subdiag=subdiag)
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.5 * losses[0]
    p, rA, iA = learned_shift.family(4096, n, param_seed=22)
    rE, iE, _ = learned_shift.solve_plain(n, 4096, rA, iA, TC)
    rS, iS = learned_shift.predict(net, n, 4096, p, rA, iA)
    torch.cuda.synchronize()
    err_net = learned_shift.prediction_error(n, 4096, rS, iS, rE, iE)
    # the diagonal of A(p) is the trivial guess the network must beat
    A = ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC)
    E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
    d = np.diagonal(A, axis1=1, axis2=2)
    err_diag = np.abs(d[:, :, None] - E[:, None, :]).min(axis=2)
    assert np.median(err_net) < 0.5 * np.median(err_diag)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "net.bin")
        net.save(path)
        net2 = ves.ShiftNet(path=path)
        rS2, iS2 = learned_shift.predict(net2, n, 4096, p, rA, iA)
        torch.cuda.synchronize()
        assert torch.equal(rS, rS2) and torch.equal(iS, iS2)


def test_gate_closed_equals_plain_solver():
    """With the gate closed (predictions never used) the shift-seeded solve is
    the plain solver, bit for bit, and reports no fallbacks."""
    import torch
    n, N = 16, 4096
    p, rA, iA = learned_shift.family(N, n, param_seed=12)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC, vectors=True)
    far = torch.full_like(rE0, 100.0)
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, far, torch.zeros_like(far), shift_gate=1e6)
    assert torch.equal(rE, rE0) and torch.equal(iE, iE0) and torch.equal(sw, sw0)
    assert fb.sum().item() == 0 and (st == 0).all()


@pytest.mark.parametrize("n", [16, 40])
def test_polish_far_predictions_dropped(n):
    """Predictions far from the spectrum do not converge in a few Newton
    steps and are dropped: the solve is then the plain solver, bit for bit
    (n = 16 runs the warp pre-pass, n = 40 the in-kernel polish)."""
    import torch
    N = 2048
    p, rA, iA = learned_shift.family(N, n, param_seed=13)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC, vectors=True)
    far = torch.full_like(rE0, 100.0)
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, far, torch.zeros_like(far), shift_polish=4)
    assert torch.equal(rE, rE0) and torch.equal(iE, iE0) and torch.equal(sw, sw0)
    assert fb.sum().item() == 0


@pytest.mark.parametrize("n", [16, 32, 40, 64])
def test_polish_recovers_noisy_predictions(n):
    """Eigenvalues with 1% noise as predictions: the Newton polish brings them
    back to FP32 accuracy, the QR needs clearly fewer sweeps, the result meets
    the plain solver's bar."""
    import torch
    N = 4096
    p, rA, iA = learned_shift.family(N, n, param_seed=14)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC)
    g = torch.Generator(device="cuda").manual_seed(1)
    rS = rE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    iS = iE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, rS, iS, shift_polish=4)
    assert res <= 1e-13
    E0 = ves.complex_vec_from_soa(rE0.cpu().numpy(), iE0.cpu().numpy(), n, TC)
    E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
    nA = np.linalg.norm(ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC), axis=(1, 2))
    _, err, _ = match_eigs(E, E0)
    assert (err / nA).max() <= 1e-12
    assert sw.double().mean().item() < 0.8 * sw0.double().mean().item()
    assert ((st & ~ves.VES_STATUS_SHIFT_FALLBACK) == 0).all()


@pytest.mark.parametrize("n", [16, 40])
def test_polish_separates_duplicate_predictions(n):
    """Predictions in coinciding pairs (the prediction of every odd-numbered
    eigenvalue replaced by its neighbour's, 1e-3 apart): the Aberth polish
    pushes one of each pair to the eigenvalue that has no prediction, so the
    QR needs fewer sweeps than when every prediction is polished on its own
    (Newton, the n <= 32 pre-pass's VES_POLISH_METHOD=newton); the result
    meets the plain solver's bar either way."""
    import torch
    N = 4096
    p, rA, iA = learned_shift.family(N, n, param_seed=15)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC)
    g = torch.Generator(device="cuda").manual_seed(2)
    rS = rE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    iS = iE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    for P in (rS, iS):
        v = P.view(N // TC, n, TC)
        v[:, 1::2, :] = v[:, 0:n - 1:2, :] + 1e-3
    E0 = ves.complex_vec_from_soa(rE0.cpu().numpy(), iE0.cpu().numpy(), n, TC)
    nA = np.linalg.norm(ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC), axis=(1, 2))
    sweeps = {}
    for method in (["aberth", "newton"] if n <= 32 else ["aberth"]):
        os.environ["VES_POLISH_METHOD"] = method
        try:
            rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, rS, iS, shift_polish=16)
        finally:
            del os.environ["VES_POLISH_METHOD"]
        assert res <= 1e-13
        E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
        _, err, _ = match_eigs(E, E0)
        assert (err / nA).max() <= 1e-12
        assert ((st & ~ves.VES_STATUS_SHIFT_FALLBACK) == 0).all()
        sweeps[method] = sw.double().mean().item()
    plain = sw0.double().mean().item()
    print("sweeps per matrix: plain %.2f, %s" % (plain, sweeps))
    assert sweeps["aberth"] < 0.8 * plain
    if "newton" in sweeps:
        assert sweeps["aberth"] < 0.95 * sweeps["newton"]


@pytest.mark.parametrize("n", [16, 40, 64])
def test_fp64_newton_step_cuts_sweeps(n):
    """After the FP32 polish (predictions at ~1e-6 of the eigenvalue scale), one
    FP64 Newton step on the solve's own Hessenberg matrix brings them to ~1e-12:
    fewer QR sweeps than without it (VES_POLISH_FP64_STEP=0), the same bar."""
    import torch
    N = 4096
    p, rA, iA = learned_shift.family(N, n, param_seed=16)
    rE0, iE0, sw0 = learned_shift.solve_plain(n, N, rA, iA, TC)
    g = torch.Generator(device="cuda").manual_seed(3)
    rS = rE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    iS = iE0 + 1e-2 * torch.randn(rE0.shape, generator=g, device="cuda", dtype=torch.float64)
    E0 = ves.complex_vec_from_soa(rE0.cpu().numpy(), iE0.cpu().numpy(), n, TC)
    nA = np.linalg.norm(ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC), axis=(1, 2))
    sweeps = {}
    for step in ("1", "0"):
        os.environ["VES_POLISH_FP64_STEP"] = step
        try:
            rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, rS, iS, shift_polish=8)
        finally:
            del os.environ["VES_POLISH_FP64_STEP"]
        assert res <= 1e-13
        E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
        _, err, _ = match_eigs(E, E0)
        assert (err / nA).max() <= 1e-12
        assert ((st & ~ves.VES_STATUS_SHIFT_FALLBACK) == 0).all()
        sweeps[step] = sw.double().mean().item()
    print("sweeps per matrix: plain %.2f, with / without the FP64 step %.2f / %.2f"
          % (sw0.double().mean().item(), sweeps["1"], sweeps["0"]))
    assert sweeps["1"] < 0.95 * sweeps["0"]


@pytest.mark.parametrize("n", [8, 16, 40])
def test_polish_special_matrices(n):
    """The Aberth polish and the FP64 Newton step on structured inputs: an
    upper-triangular matrix (the Hessenberg form splits at once: no FP64 step),
    a diagonal one, a repeated eigenvalue (2 I plus a rank-one term), the zero
    matrix, and predictions that are NaN or infinite.  Every solve meets the
    plain solver's bar against LAPACK."""
    import torch
    rng = np.random.default_rng(900 + n)
    N = TC
    A = rng.standard_normal((N, n, n)) + 1j * rng.standard_normal((N, n, n))
    A[1] = np.triu(A[1])
    A[2] = np.diag(np.arange(1, n + 1) * (1 + 0.5j))
    u = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    A[3] = 2 * np.eye(n) + np.outer(u, u.conj()) / n
    A[4] = 0
    E = np.linalg.eigvals(A)
    P = E + 1e-2 * (rng.standard_normal(E.shape) + 1j * rng.standard_normal(E.shape))
    P[5, :] = np.nan
    P[6, 0] = np.inf
    rA, iA = (torch.from_numpy(x).cuda() for x in ves.soa_from_complex(A, TC))
    rS, iS = (torch.from_numpy(x).cuda() for x in ves.soa_vec_from_complex(P, TC))
    rE, iE, st, sw, fb, res = solve_shifts(n, N, rA, iA, rS, iS, shift_polish=8)
    Eg = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
    V = ves.complex_from_soa(*(t.cpu().numpy() for t in solve_vectors(n, N, rA, iA, rS, iS)), n, TC)
    nA = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1.0)
    _, err, _ = match_eigs(Eg, E)
    assert (err / nA).max() <= 1e-12
    r = np.linalg.norm(A @ V - V * Eg[:, None, :], axis=1) / (nA[:, None] * np.maximum(np.linalg.norm(V, axis=1), 1e-300))
    assert r.max() <= 1e-13
    assert ((st & ~ves.VES_STATUS_SHIFT_FALLBACK) == 0).all()


def solve_vectors(n, N, rA, iA, rS, iS):
    """The eigenvectors of the shift-seeded solve with shift_polish=8 (planes)."""
    import torch
    rE = torch.empty(N * n, dtype=torch.float64, device="cuda")
    iE = torch.empty_like(rE)
    rV, iV = torch.empty_like(rA), torch.empty_like(iA)
    ves.eigensolve_shifts(n, N // TC, TC, rA, iA, rE, iE, rV, iV, rS, iS,
                          options=ves.default_options(shift_polish=8))
    torch.cuda.synchronize()
    return rV, iV
