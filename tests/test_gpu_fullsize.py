"""Full-size workloads: every matrix checked on the device in FP64, the
oracle on a prefix.

  1,048,576 x 16x16, seed 1  (oracle on the first 65,536)
    262,144 x 32x32, seed 3  (oracle on the first 16,384)
"""
import numpy as np
import pytest

import oracle
import ves
import workloads
from gpu_util import soa_planes_to_batch, soa_vec_to_batch, device_residuals
from parity import match_eigs

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
TC = 512


@pytest.mark.parametrize("name", ["gauss16", "gauss32"])
def test_fullsize_plain_fp64(name):
    import torch
    w = workloads.WORKLOADS[name]
    N, n, seed, sub = w["N"], w["n"], w["seed"], w["oracle_subset"]
    bc = N // TC
    rA, iA = workloads.gaussian_soa(N, n, seed, TC)
    dAr = torch.from_numpy(rA).cuda()
    dAi = torch.from_numpy(iA).cuda()
    dEr = torch.empty(N * n, dtype=torch.float64, device="cuda")
    dEi = torch.empty_like(dEr)
    dVr = torch.empty_like(dAr)
    dVi = torch.empty_like(dAi)
    st = torch.full((N,), -1, dtype=torch.int32, device="cuda")
    sw = torch.zeros(N, dtype=torch.int32, device="cuda")
    ves.eigensolve(n, bc, TC, dAr, dAi, dEr, dEi, dVr, dVi, status=st, sweeps=sw)
    torch.cuda.synchronize()
    assert int((st != 0).sum()) == 0
    A = soa_planes_to_batch(dAr, dAi, n, TC)
    V = soa_planes_to_batch(dVr, dVi, n, TC)
    E = soa_vec_to_batch(dEr, dEi, n, TC)
    res = device_residuals(A, E, V)
    assert float(res.max()) <= 1e-13, float(res.max())
    spe = float(sw.double().mean()) / n
    assert 2.5 < spe < 4.0
    # oracle on the prefix (identical bytes: the first sub matrices are the
    # first sub/TC blocks of the SoA planes)
    k = sub * n * n
    rE, iE, _, _, _, _, swo = oracle.eigensolve(rA[:k], iA[:k], n, TC)
    Eo = ves.complex_vec_from_soa(rE, iE, n, TC)
    Eg = ves.complex_vec_from_soa(dEr[:sub * n].cpu().numpy(), dEi[:sub * n].cpu().numpy(), n, TC)
    Ah = ves.complex_from_soa(rA[:k], iA[:k], n, TC)
    _, err, same = match_eigs(Eg, Eo)
    assert (err / np.linalg.norm(Ah, axis=(1, 2))).max() <= 1e-12
    assert same.mean() > 0.99
    assert (sw[:sub].cpu().numpy() == swo).mean() > 0.99
