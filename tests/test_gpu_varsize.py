"""Mixed-size batches (ves_eigensolve_varsize): binned by order on the device,
one persistent launch, capturable as a CUDA graph.  Every matrix is solved by
the same lockstep lane code at its own order, so its results equal the
fixed-size solver's bit for bit."""
import numpy as np
import pytest

import ves
from gpu_util import run_fused
from parity import residuals

pytestmark = pytest.mark.gpu


def cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def pack(mats):
    """list of (n, n) complex -> dims, re plane, im plane (packed, column-major per matrix)."""
    dims = np.array([m.shape[0] for m in mats], dtype=np.int32)
    flat = np.concatenate([m.T.reshape(-1) for m in mats]) if mats else np.zeros(0, complex)
    return dims, np.ascontiguousarray(flat.real), np.ascontiguousarray(flat.imag)


def unpack(dims, re, im, vec=False):
    out, o = [], 0
    for d in dims:
        k = d if vec else d * d
        z = re[o:o + k] + 1j * im[o:o + k]
        out.append(z if vec else z.reshape(d, d).T)
        o += k
    return out


def run_varsize(mats, max_dim=64, graph=False, **opt):
    import torch
    dims, re, im = pack(mats)
    count = len(mats)
    ne = int(dims.sum())
    t = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    dd, dr, di = t(dims), t(re), t(im)
    er = torch.full((max(ne, 1),), np.nan, dtype=torch.float64, device="cuda")
    ei = torch.full_like(er, np.nan)
    vr = torch.full_like(dr, np.nan)
    vi = torch.full_like(di, np.nan)
    st = torch.full((count,), -1, dtype=torch.int32, device="cuda")
    sw = torch.full((count,), -1, dtype=torch.int32, device="cuda")
    o = ves.default_options(**opt)
    if graph:
        g = ves.VarsizeGraph(count, max_dim, dd, dr, di, er, ei, vr, vi, status=st, sweeps=sw, options=o)
        g.launch()
        torch.cuda.synchronize()
        return g, (dd, dr, di, er, ei, vr, vi, st, sw)
    ves.eigensolve_varsize(count, max_dim, dd, dr, di, er, ei, vr, vi, status=st, sweeps=sw, options=o)
    torch.cuda.synchronize()
    E = unpack(dims, er.cpu().numpy(), ei.cpu().numpy(), vec=True)
    V = unpack(dims, vr.cpu().numpy(), vi.cpu().numpy())
    return E, V, st.cpu().numpy(), sw.cpu().numpy()


def test_varsize_equals_fixed_size_solver():
    rng = np.random.default_rng(600)
    sizes = rng.integers(1, 65, size=1500)
    mats = [cgauss(rng, (n, n)) for n in sizes]
    E, V, st, sw = run_varsize(mats)
    assert (st == 0).all()
    for n in np.unique(sizes):
        idx = np.nonzero(sizes == n)[0]
        A = np.stack([mats[i] for i in idx])
        ref = run_fused(A, 1)
        for j, i in enumerate(idx):
            np.testing.assert_array_equal(E[i], ref["E"][j])
            np.testing.assert_array_equal(V[i], ref["V"][j])
            assert sw[i] == ref["sweeps"][j]


def test_varsize_order_and_graph_replay():
    import torch
    rng = np.random.default_rng(601)
    sizes = rng.integers(4, 33, size=700)
    mats = [cgauss(rng, (n, n)) for n in sizes]
    E0, V0, _, _ = run_varsize(mats)
    E1, V1, _, _ = run_varsize(mats, varsize_order=1, blocks_per_sm=3)
    for a, b in zip(E0, E1):
        np.testing.assert_array_equal(a, b)
    g, bufs = run_varsize(mats, max_dim=32, graph=True)
    dd, dr, di, er, ei, vr, vi, st, sw = bufs
    dims = sizes.astype(np.int32)
    Eg = unpack(dims, er.cpu().numpy(), ei.cpu().numpy(), vec=True)
    for a, b in zip(E0, Eg):
        np.testing.assert_array_equal(a, b)
    # new matrices in the same buffers, replay the graph
    mats2 = [cgauss(rng, (n, n)) for n in sizes]
    _, re2, im2 = pack(mats2)
    dr.copy_(torch.from_numpy(re2))
    di.copy_(torch.from_numpy(im2))
    g.launch()
    torch.cuda.synchronize()
    E2 = unpack(dims, er.cpu().numpy(), ei.cpu().numpy(), vec=True)
    V2 = unpack(dims, vr.cpu().numpy(), vi.cpu().numpy())
    for A, e, v in zip(mats2, E2, V2):
        assert residuals(A[None], e[None], v[None]).max() <= 1e-13


def test_varsize_bad_orders_flagged():
    rng = np.random.default_rng(602)
    mats = [cgauss(rng, (n, n)) for n in (3, 9, 5, 20, 2)]
    # order 20 exceeds max_dim = 16: skipped and flagged, the others solved
    E, V, st, _ = run_varsize(mats, max_dim=16)
    assert st[3] == ves.VES_STATUS_BAD_DIM
    assert (st[[0, 1, 2, 4]] == 0).all()
    assert np.isnan(E[3]).all()
    for i in (0, 1, 2, 4):
        assert residuals(mats[i][None], E[i][None], V[i][None]).max() <= 1e-13


def test_varsize_families():
    """The three families of the mixed-size benchmark: Gaussian, non-normal
    (eigenvector condition ~1e4), clustered (4 clusters of radius 1e-6)."""
    import workloads
    mats = workloads.mixed_families(600, seed=9)
    E, V, st, _ = run_varsize(mats)
    assert (st == 0).all()
    for A, e, v in zip(mats, E, V):
        assert residuals(A[None], e[None], v[None]).max() <= 1e-13
