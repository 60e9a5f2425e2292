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
