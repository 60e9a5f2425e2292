"""Seeded synthetic batches for the eigensolver benchmarks and parity tests.

The reference ships no data (README.md:48-51; its benchmark reads
testcases/{real,imag}.bin, zlahqr.cpp:52-53), so every batch here is
synthetic and reproducible from its seed:

  gaussian(N, n, seed):  A = X + iY, X and Y i.i.d. N(0,1),
      rng = numpy.random.default_rng(seed); X = rng.standard_normal((N,n,n));
      Y = rng.standard_normal((N,n,n))  (in that order); A[m][i, j] = X[m,i,j] + iY[m,i,j].

Workloads used by the benchmark (sizes as the reference's configurations):
  N=10,000     n=8   seed 0   (reference CPU case)
  N=1,048,576  n=16  seed 1   (plain FP64 GPU case; oracle on the first 65,536)
  N=262,144    n=32  seed 3   (mixed-precision case)
"""
import numpy as np

WORKLOADS = {
    "gauss8": dict(N=10_000, n=8, seed=0),
    "gauss16": dict(N=1_048_576, n=16, seed=1, oracle_subset=65_536),
    "gauss32": dict(N=262_144, n=32, seed=3, oracle_subset=16_384),
}


def gaussian(N, n, seed, count=None):
    """Complex Gaussian batch; `count` (<= N) returns only the first matrices
    of the batch (identical to the prefix of the full batch)."""
    rng = np.random.default_rng(seed)
    if count is None or count >= N:
        X = rng.standard_normal((N, n, n))
        Y = rng.standard_normal((N, n, n))
        return X + 1j * Y
    # The prefix of X is the first count*n*n draws; Y starts after all N*n*n
    # draws of X, so those must be consumed (in chunks, to bound memory).
    X = rng.standard_normal((count, n, n))
    left = (N - count) * n * n
    chunk = 1 << 24
    while left > 0:
        k = min(chunk, left)
        rng.standard_normal(k)
        left -= k
    Y = rng.standard_normal((count, n, n))
    return X + 1j * Y


def gaussian_soa(N, n, seed, thread_cnt):
    """The same batch directly as SoA planes (re, im), each N*n*n float64.

    Element (i, j) of matrix m = b*thread_cnt + t goes to
    b*thread_cnt*n*n + (i + j*n)*thread_cnt + t."""
    if N % thread_cnt:
        raise ValueError("N must be a multiple of thread_cnt")
    rng = np.random.default_rng(seed)
    planes = []
    for _ in range(2):
        X = rng.standard_normal((N, n, n))
        bc = N // thread_cnt
        planes.append(np.ascontiguousarray(X.reshape(bc, thread_cnt, n, n).transpose(0, 3, 2, 1)).reshape(-1))
        del X
    return planes[0], planes[1]


def _haar(gen, k, n, device):
    """k Haar-distributed n x n unitaries as a product of n - 1 Householder
    reflections with complex Gaussian vectors of decreasing length and a
    diagonal of uniform phases (Stewart 1980, "The efficient generation of
    random orthogonal matrices"); batched matrix products only."""
    import torch
    U = torch.eye(n, dtype=torch.complex128, device=device).repeat(k, 1, 1)
    for j in range(n - 1):
        m = n - j
        x = torch.complex(torch.randn(k, m, generator=gen, dtype=torch.float64, device=device),
                          torch.randn(k, m, generator=gen, dtype=torch.float64, device=device))
        a = x[:, 0]
        ph = torch.where(a.abs() > 0, a / a.abs().clamp_min(1e-300), torch.ones_like(a))
        v = x.clone()
        v[:, 0] = a + ph * torch.linalg.vector_norm(x, dim=1)
        v = v / torch.linalg.vector_norm(v, dim=1, keepdim=True)
        Uc = U[:, :, j:]
        U[:, :, j:] = Uc - 2 * (Uc @ v[:, :, None]) * v.conj()[:, None, :]
    d = torch.polar(torch.ones(k, n, dtype=torch.float64, device=device),
                    2 * np.pi * torch.rand(k, n, generator=gen, dtype=torch.float64, device=device))
    return U * d[:, None, :]


def _similar(U, s, W, lam):
    """A = (U diag(s) W) diag(lam) (U diag(s) W)^-1, the inverse taken exactly as
    W^H diag(1/s) U^H because U and W are unitary."""
    V = (U * s[None, None, :]) @ W
    Vinv = (W.conj().transpose(1, 2) * (1.0 / s)[None, None, :]) @ U.conj().transpose(1, 2)
    return (V * lam[:, None, :]) @ Vinv


def _inverse_near_unitary(X, U, iters=10):
    """X^-1 for X = U + E with U unitary and ||E||_2 < 1: Newton-Schulz
    iteration Y <- Y (2I - X Y) from Y = U^H (quadratic convergence from
    ||I - X U^H|| = ||E||)."""
    import torch
    Y = U.conj().transpose(1, 2)
    two = 2 * torch.eye(X.shape[-1], dtype=X.dtype, device=X.device)
    for _ in range(iters):
        Y = Y @ (two - X @ Y)
    return Y


def mixed_families(N, seed=2, nmin=4, nmax=64, device="cpu", as_list=True):
    """The mixed-size workload: N complex128 matrices, order uniform in
    [nmin, nmax], matrix m of family m % 3:
      0  i.i.d. complex Gaussian;
      1  non-normal A = V diag(l) V^-1, V = U diag(logspace(0, -4, n)) W with U, W
         Haar unitaries (cond(V) = 1e4, V^-1 = W^H diag(1/s) U^H exactly),
         l uniform in the unit disk (r = sqrt(u));
      2  clustered A = X diag(l) X^-1, X = U + 0.3 G / sqrt(n) (U Haar, G complex
         Gaussian with E|g|^2 = 1; ||X - U||_2 is about 0.6, so X is well conditioned and
         X^-1 comes from a Newton-Schulz iteration started at U^H),
         l = one of 4 complex-Gaussian centres plus an offset uniform in a disk
         of radius 1e-6.
    Generated with torch (seeded), batched by order, matrix products only.
    Returns a list of (n, n) numpy arrays (as_list) or (sizes, dict n -> (indices,
    tensor))."""
    import torch
    gen = torch.Generator(device=device).manual_seed(seed)
    sizes = torch.randint(nmin, nmax + 1, (N,), generator=gen, device=device).cpu().numpy()
    fam = np.arange(N) % 3
    by_n = {}
    for n in np.unique(sizes):
        idx = np.nonzero(sizes == n)[0]
        k = len(idx)
        out = torch.empty(k, n, n, dtype=torch.complex128, device=device)
        f = torch.from_numpy(fam[idx]).to(device)
        g = f == 0
        if g.any():
            c = int(g.sum())
            out[g] = torch.complex(torch.randn(c, n, n, generator=gen, dtype=torch.float64, device=device),
                                   torch.randn(c, n, n, generator=gen, dtype=torch.float64, device=device))
        g = f == 1
        if g.any():
            c = int(g.sum())
            s = torch.logspace(0, -4, n, dtype=torch.float64, device=device).to(torch.complex128)
            r = torch.sqrt(torch.rand(c, n, generator=gen, dtype=torch.float64, device=device))
            th = 2 * np.pi * torch.rand(c, n, generator=gen, dtype=torch.float64, device=device)
            out[g] = _similar(_haar(gen, c, n, device), s, _haar(gen, c, n, device), torch.polar(r, th))
        g = f == 2
        if g.any():
            c = int(g.sum())
            centres = torch.complex(torch.randn(c, 4, generator=gen, dtype=torch.float64, device=device),
                                    torch.randn(c, 4, generator=gen, dtype=torch.float64, device=device))
            r = 1e-6 * torch.sqrt(torch.rand(c, n, generator=gen, dtype=torch.float64, device=device))
            th = 2 * np.pi * torch.rand(c, n, generator=gen, dtype=torch.float64, device=device)
            lam = centres[:, torch.arange(n, device=device) % 4] + torch.polar(r, th)
            U = _haar(gen, c, n, device)
            G = torch.complex(torch.randn(c, n, n, generator=gen, dtype=torch.float64, device=device),
                              torch.randn(c, n, n, generator=gen, dtype=torch.float64, device=device))
            X = U + (0.3 / np.sqrt(2 * n)) * G
            out[g] = (X * lam[:, None, :]) @ _inverse_near_unitary(X, U)
        by_n[int(n)] = (idx, out)
    if not as_list:
        return sizes, by_n
    mats = [None] * N
    for n, (idx, out) in by_n.items():
        arr = out.cpu().numpy()
        for j, i in enumerate(idx):
            mats[i] = arr[j]
    return mats


def pack_varsize(sizes, by_n, device="cpu"):
    """Packed mixed-size layout (ves_eigensolve_varsize): per matrix column-major
    and contiguous, in index order.  Returns (dims int32, re, im) tensors."""
    import torch
    sizes = np.asarray(sizes)
    off = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
    total = int(off[-1])
    re = torch.empty(total, dtype=torch.float64, device=device)
    im = torch.empty(total, dtype=torch.float64, device=device)
    for n, (idx, out) in by_n.items():
        cm = out.transpose(1, 2).reshape(len(idx), n * n)  # column-major rows
        pos = torch.from_numpy(off[idx]).to(device)[:, None] + torch.arange(n * n, device=device)[None, :]
        re[pos.reshape(-1)] = cm.real.reshape(-1)
        im[pos.reshape(-1)] = cm.imag.reshape(-1)
    return torch.from_numpy(sizes.astype(np.int32)).to(device), re, im
