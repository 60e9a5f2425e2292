"""Learned shift proposal: the parametric family, training on the plain
solver's eigenvalues, and the predict-then-solve path.

Family (per order n): A(p) = A0 + p1 A1 + p2 A2 + p3 A3 with A0..A3 fixed
complex Gaussian matrices (torch generator seeded `family_seed`) scaled by
1/sqrt(n), and p uniform in [-1, 1]^3 per instance (generator seeded
`param_seed`).  The network sees p and diag(A(p)) and predicts the n
eigenvalues; the solver uses them as the first QR shift of every eigenvalue
(ves_eigensolve_shifts) and falls back to the reference's Wilkinson shift
after it.  Everything runs through libves.so: the plain FP64 solver makes the
labels, the tcgen05 network is trained and evaluated by the library's own
kernels.
"""
import numpy as np

import ves


def family(N, n, family_seed=4, param_seed=5, thread_cnt=512, device="cuda"):
    """Returns (params (N, 3) float64, rA, iA SoA planes) on `device`; N must be
    a multiple of thread_cnt."""
    import torch
    if N % thread_cnt:
        raise ValueError("N=%d is not a multiple of thread_cnt=%d" % (N, thread_cnt))
    g = torch.Generator(device=device).manual_seed(family_seed)
    basis = torch.complex(torch.randn(4, n, n, generator=g, dtype=torch.float64, device=device),
                          torch.randn(4, n, n, generator=g, dtype=torch.float64, device=device)) / np.sqrt(n)
    gp = torch.Generator(device=device).manual_seed(param_seed)
    p = torch.rand(N, 3, generator=gp, dtype=torch.float64, device=device) * 2 - 1
    A = basis[0][None] + torch.einsum("mk,kij->mij", p.to(torch.complex128), basis[1:])
    bc = N // thread_cnt
    s = A.reshape(bc, thread_cnt, n, n).permute(0, 3, 2, 1)  # b, j, i, t
    return p.contiguous(), s.real.contiguous().reshape(-1), s.imag.contiguous().reshape(-1)


def solve_plain(n, N, rA, iA, thread_cnt=512, vectors=False):
    import torch
    rE = torch.empty(N * n, dtype=torch.float64, device=rA.device)
    iE = torch.empty_like(rE)
    sw = torch.zeros(N, dtype=torch.int32, device=rA.device)
    if vectors:
        rV, iV = torch.empty_like(rA), torch.empty_like(iA)
        ves.eigensolve(n, N // thread_cnt, thread_cnt, rA, iA, rE, iE, rV, iV, sweeps=sw)
    else:
        ves.eigensolve(n, N // thread_cnt, thread_cnt, rA, iA, rE, iE, None, None, sweeps=sw,
                       options=ves.default_options(want_vectors=0))
    return rE, iE, sw


def train(n, count=200_000, epochs=60, batch=1024, lr=1e-3, hidden=256, family_seed=4, param_seed=5, seed=0,
          thread_cnt=512, **config):
    """Train a ShiftNet for order n on `count` plain-solver solutions (rounded
    down to a multiple of thread_cnt); `config` passes ves_shiftnet_config
    fields (layers, fourier, loss, delta)."""
    import torch
    count = max(thread_cnt, count // thread_cnt * thread_cnt)
    p, rA, iA = family(count, n, family_seed, param_seed, thread_cnt)
    rE, iE, _ = solve_plain(n, count, rA, iA, thread_cnt)
    torch.cuda.synchronize()
    net = ves.ShiftNet(dim=n, n_params=3, hidden=hidden, seed=seed, **config)
    losses = net.train(count, thread_cnt, p, rA, iA, rE, iE, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, losses


def predict(net, n, N, params, rA, iA, thread_cnt=512):
    import torch
    rS = torch.empty(N * n, dtype=torch.float64, device=rA.device)
    iS = torch.empty_like(rS)
    net.predict(N, thread_cnt, params, rA, iA, rS, iS)
    return rS, iS


def prediction_error(n, N, rS, iS, rE, iE, thread_cnt=512):
    """Per predicted eigenvalue, the distance to the nearest true eigenvalue."""
    S = ves.complex_vec_from_soa(rS.cpu().numpy(), iS.cpu().numpy(), n, thread_cnt)
    E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, thread_cnt)
    return np.abs(S[:, :, None] - E[:, None, :]).min(axis=2)


def relative_error(n, rA, iA, rS, iS, rE, iE, thread_cnt=512):
    """Per true eigenvalue, the distance to the nearest prediction in units of
    ||A||_F / sqrt(n) (the units of ves_options.shift_gate); a device tensor
    (N, n)."""
    import torch

    def vec(re, im):
        return torch.complex(re.view(-1, n, thread_cnt), im.view(-1, n, thread_cnt)).permute(0, 2, 1).reshape(-1, n)
    S, E = vec(rS, iS), vec(rE, iE)
    fro = torch.linalg.vector_norm(torch.complex(rA.view(-1, n * n, thread_cnt), iA.view(-1, n * n, thread_cnt)),
                                   dim=1).reshape(-1)
    d = (E[:, :, None] - S[:, None, :]).abs().amin(dim=2)
    return d / (fro[:, None] / np.sqrt(n))


def calibrate(net, n, count=32768, family_seed=4, param_seed=7, thread_cnt=512, factor=1.0):
    """The gate for ves_options.shift_gate: `factor` x the median prediction
    error (relative_error) on a held-out draw of the family."""
    import torch
    p, rA, iA = family(count, n, family_seed, param_seed, thread_cnt)
    rE, iE, _ = solve_plain(n, count, rA, iA, thread_cnt)
    rS, iS = predict(net, n, count, p, rA, iA, thread_cnt)
    torch.cuda.synchronize()
    err = relative_error(n, rA, iA, rS, iS, rE, iE, thread_cnt)
    return factor * float(err.median())
