"""Helpers for the GPU tests: run libves.so's native entry points on NumPy
inputs through torch device buffers, and FP64 checks on the device."""
import numpy as np

import ves


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def run_fused(A, tc, vnorm=0, max_its=30, want_T=False, precision=0, **opts):
    """ves_eigensolve on the complex batch A (N, n, n) in SoA layout with
    interleave tc.  Returns dict of numpy outputs (E, V, T, status, sweeps)."""
    import torch
    N, n, _ = A.shape
    bc = N // tc
    rA, iA = ves.soa_from_complex(A, tc)
    dAr, dAi = dev(rA), dev(iA)
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    dVr = torch.empty_like(dAr)
    dVi = torch.empty_like(dAi)
    dTr = torch.empty_like(dAr) if want_T else None
    dTi = torch.empty_like(dAi) if want_T else None
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    sw = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    opt = ves.default_options(vnorm=vnorm, max_its=max_its, precision=precision, **opts)
    ves.eigensolve(n, bc, tc, dAr, dAi, dEr, dEi, dVr, dVi, dTr, dTi, st, sw, options=opt)
    torch.cuda.synchronize()
    out = dict(
        E=ves.complex_vec_from_soa(dEr.cpu().numpy(), dEi.cpu().numpy(), n, tc),
        V=ves.complex_from_soa(dVr.cpu().numpy(), dVi.cpu().numpy(), n, tc),
        status=st.cpu().numpy(), sweeps=sw.cpu().numpy(),
    )
    if want_T:
        out["T"] = ves.complex_from_soa(dTr.cpu().numpy(), dTi.cpu().numpy(), n, tc)
    # the input is read only
    assert np.array_equal(dAr.cpu().numpy(), rA, equal_nan=True) and np.array_equal(dAi.cpu().numpy(), iA, equal_nan=True)
    return out


def soa_planes_to_batch(re, im, n, tc):
    """torch SoA planes -> (N, n, n) complex128 on the device."""
    import torch
    r = re.view(-1, n, n, tc).permute(0, 3, 2, 1)
    i = im.view(-1, n, n, tc).permute(0, 3, 2, 1)
    return torch.complex(r, i).reshape(-1, n, n)


def soa_vec_to_batch(re, im, n, tc):
    import torch
    r = re.view(-1, n, tc).permute(0, 2, 1)
    i = im.view(-1, n, tc).permute(0, 2, 1)
    return torch.complex(r, i).reshape(-1, n)


def device_residuals(A, E, V, chunk=1 << 18):
    """max over pairs of ||A v - lambda v|| / (||A||_F ||v||), FP64 on device,
    per matrix (N,)."""
    import torch
    out = []
    for s in range(0, A.shape[0], chunk):
        a, e, v = A[s:s + chunk], E[s:s + chunk], V[s:s + chunk]
        r = torch.matmul(a, v) - v * e[:, None, :]
        num = torch.linalg.vector_norm(r, dim=1)
        den = torch.linalg.matrix_norm(a)[:, None] * torch.linalg.vector_norm(v, dim=1)
        out.append((num / den).amax(dim=1))
    return torch.cat(out)
