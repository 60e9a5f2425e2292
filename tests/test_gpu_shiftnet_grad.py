"""The shift network's backward pass against an FP32 torch autograd reference.

ves_shiftnet_gradient computes one training step's loss and gradients the
way ves_shiftnet_train does: the hidden layers' weight and input gradients as
tcgen05 BF16 GEMMs (dW = dZ^T Hin split over the batch, dH = dZ W) with FP32
accumulation, the output layer in FP32.  The reference runs the same forward
(BF16 features, BF16 weights and activations of the hidden layers, FP32
output layer, tanh-GELU, symmetric Chamfer loss) in torch with autograd in
FP32, the BF16 roundings passed straight through.  Bar: the loss to 1e-4
relative; every layer's weight and bias gradient within 2e-2 of the
reference in relative Frobenius norm (dZ is rounded to BF16 for the tensor
cores), the FP32 output layer within 1e-3.
"""
import math
import os
import tempfile

import numpy as np
import pytest

import learned_shift
import ves

pytestmark = pytest.mark.gpu
TC = 512


def read_checkpoint(path):
    """Weights and standardisation of a version-3 checkpoint (ves_shiftnet_save)."""
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw[:40], dtype=np.int32)
    assert hdr[0] == 0x56455353 and hdr[1] == 3
    n, P, H, L, F, S = (int(hdr[k]) for k in (2, 3, 4, 5, 6, 9))
    kin = P + 2 * P * F + 2 * n + S * (n - 1)
    kin_pad = (kin + 31) // 32 * 32
    nout_pad = (2 * n + 15) // 16 * 16
    fl = np.frombuffer(raw[40 + 4 + 8:], dtype=np.float32)
    o, W, b = 0, [], []
    for l in range(L + 1):
        fin = kin_pad if l == 0 else H
        fout = nout_pad if l == L else H
        W.append(fl[o:o + fout * fin].reshape(fout, fin).copy())
        o += fout * fin
        b.append(fl[o:o + fout].copy())
        o += fout
    return dict(n=n, P=P, H=H, L=L, F=F, S=S, kin=kin, kin_pad=kin_pad, nout_pad=nout_pad, W=W, b=b,
                fmean=fl[o:o + kin_pad], fstd=fl[o + kin_pad:o + 2 * kin_pad])


def reference(ck, p, A, E):
    """Loss and gradients (checkpoint order) of one batch, torch FP32 autograd."""
    import torch
    n, L, S = ck["n"], ck["L"], ck["S"]
    d = np.diagonal(A, axis1=1, axis2=2)
    feats = [p, d.real, d.imag]
    if S:
        feats.append(np.stack([np.linalg.norm(np.diagonal(A, offset=-k, axis1=1, axis2=2), axis=1)
                               for k in range(1, n)], axis=1))
    f = np.concatenate(feats, axis=1).astype(np.float32)
    f = (f - ck["fmean"][:ck["kin"]]) / ck["fstd"][:ck["kin"]]
    X = np.zeros((A.shape[0], ck["kin_pad"]), np.float32)
    X[:, :ck["kin"]] = f
    bf = lambda x: x + (x.to(torch.bfloat16).float() - x).detach()  # noqa: E731  (straight-through BF16)
    gelu = lambda z: torch.nn.functional.gelu(z, approximate="tanh")  # noqa: E731
    W = [torch.tensor(w, requires_grad=True) for w in ck["W"]]
    b = [torch.tensor(v, requires_grad=True) for v in ck["b"]]
    h = torch.tensor(X).to(torch.bfloat16).float()
    for l in range(L):
        z = h @ bf(W[l]).T + b[l]
        h = bf(gelu(z)) if l < L - 1 else gelu(z)
    Y = h @ W[L].T + b[L]
    T = torch.tensor(np.concatenate([E.real, E.imag], axis=1).astype(np.float32))
    yr, yi, tr, ti = Y[:, :n], Y[:, n:2 * n], T[:, :n], T[:, n:]
    D = (yr[:, :, None] - tr[:, None, :]) ** 2 + (yi[:, :, None] - ti[:, None, :]) ** 2
    B = A.shape[0]
    loss = (D.min(dim=2).values.sum() + D.min(dim=1).values.sum()) / (2.0 * n * B)
    loss.backward()
    grads = []
    for l in range(L + 1):
        grads += [W[l].grad.numpy().ravel(), b[l].grad.numpy().ravel()]
    return float(loss), grads


@pytest.mark.parametrize("subdiag", [0, 1])
def test_gradient_matches_fp32_autograd(subdiag):
    import torch
    n, N = 8, 1024
    net = ves.ShiftNet(dim=n, n_params=3, hidden=64, seed=3, layers=3, subdiag=subdiag)
    p, rA, iA = learned_shift.family(N, n, param_seed=31, thread_cnt=TC)
    rE, iE, _ = learned_shift.solve_plain(n, N, rA, iA, TC)
    grad, loss = net.gradient(N, TC, p, rA, iA, rE, iE)
    torch.cuda.synchronize()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "net.bin")
        net.save(path)
        ck = read_checkpoint(path)
    A = ves.complex_from_soa(rA.cpu().numpy(), iA.cpu().numpy(), n, TC)
    E = ves.complex_vec_from_soa(rE.cpu().numpy(), iE.cpu().numpy(), n, TC)
    ref_loss, ref_grads = reference(ck, p.cpu().numpy(), A, E)
    assert abs(float(loss.item()) - ref_loss) <= 1e-4 * abs(ref_loss)
    g = grad.cpu().numpy()
    o = 0
    for k, rg in enumerate(ref_grads):
        got = g[o:o + rg.size]
        o += rg.size
        tol = 1e-3 if k >= 2 * ck["L"] else 2e-2  # the last pair is the FP32 output layer
        rel = np.linalg.norm(got - rg) / max(np.linalg.norm(rg), 1e-30)
        assert rel <= tol, (k, rel)
    assert o == g.size


def test_training_step_count_and_loss_drop():
    """The tensor-core backward trains: the loss falls by half within a few
    epochs on a small family (as with the FP32 backward it replaces)."""
    n, N = 8, 8192
    net, losses = learned_shift.train(n, count=N, epochs=6, batch=512, lr=2e-3, hidden=128, param_seed=41)
    assert np.isfinite(losses).all() and losses[-1] < 0.5 * losses[0]
    assert not math.isnan(losses[0])
