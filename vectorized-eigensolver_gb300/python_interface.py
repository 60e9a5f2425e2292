"""Drop-in replacement for the reference's Cython module `python_interface`
(python_interface.pyx:1-220), backed by libves.so on the GPU.

Same module name, function names, argument order and in-place semantics:
every `my_*` function takes 1-D float64 NumPy arrays in the reference's
structure-of-arrays layout plus (dim, block_cnt, thread_cnt) and writes its
results into the arrays it is given.  Where the Cython module rejects an
array of the wrong dtype or rank (its `np.ndarray[dtype_t, ndim=1]` typed
arguments), this module raises ValueError.  The `test_*` helpers build the
same random inputs as the reference's and return the same tuples.

Import with this directory on sys.path:  `import python_interface`.
"""
import numpy as np

import ves

__all__ = [
    "my_repMatrix", "arrangeMatrices", "my_zlahqr", "my_backsubs", "my_repVector", "my_ztrevec", "my_zgemv",
    "my_zgehrd", "my_zunghr", "my_hessenberg", "my_eigensolver", "extractMatrix", "extractVector",
    "test_backsubs", "test_zgehrd", "test_hessenberg", "test_zgemv", "test_zlahqr", "test_eigenvectors",
]


def my_repMatrix(dim, block_cnt, thread_cnt, matrix, out):
    """pyx:31-34 -> repMatrixSoA (utils.cpp:125-142)."""
    ves.repMatrixSoA(dim, block_cnt, thread_cnt, matrix, out)


def arrangeMatrices(dim, block_cnt, thread_cnt, inputMat, outputMat):
    """pyx:36-39 -> rearrangeMatrices (utils.cpp:85-103)."""
    ves.rearrangeMatrices(dim, block_cnt, thread_cnt, inputMat, outputMat)


def my_zlahqr(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS):
    """pyx:41-46 -> call_zlahqr_new (utils.cpp:159-216): M -> T, S -> Schur vectors, E eigenvalues."""
    ves.call_zlahqr_new(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS)


def my_backsubs(dim, block_cnt, thread_cnt, rT, iT, rb, ib):
    """pyx:48-52 -> call_backsubstitution (utils.cpp:269-277)."""
    ves.call_backsubstitution(dim, block_cnt, thread_cnt, rT, iT, rb, ib)


def my_repVector(dim, block_cnt, thread_cnt, vector, out):
    """pyx:54-57 -> repVectorSoA (utils.cpp:144-157)."""
    ves.repVectorSoA(dim, block_cnt, thread_cnt, vector, out)


def my_ztrevec(dim, block_cnt, thread_cnt, rT, iT, rR, iR):
    """pyx:59-63 -> call_ztrevc (utils.cpp:279-328)."""
    ves.call_ztrevc(dim, block_cnt, thread_cnt, rT, iT, rR, iR)


def my_zgemv(hermitian, dim, block_cnt, thread_cnt, rA, iA, rx, ix, rbeta, ibeta, ry, iy):
    """pyx:65-73 -> call_zgemv (utils.cpp:218-267)."""
    ves.call_zgemv(hermitian, dim, block_cnt, thread_cnt, rA, iA, rx, ix, ry, iy, rbeta, ibeta)


def my_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau):
    """pyx:75-79 -> call_zgehrd (utils.cpp:330-374)."""
    ves.call_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau)


def my_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau):
    """pyx:81-85 -> call_zunghr (utils.cpp:376-415)."""
    ves.call_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau)


def my_hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ):
    """pyx:86-90 -> hessenberg (utils.cpp:417-479)."""
    ves.hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ)


def my_eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV):
    """The C++-only full path eigensolver() (utils.cpp:578-698), exposed to Python.

    Not in the Cython module (which cannot chain zunghr's Q into zlahqr because
    call_zlahqr_new resets S to the identity); added here."""
    ves.eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV)


def extractMatrix(dim, thread_cnt, matrix):
    """pyx:92-93: matrix of slot 0 of block 0."""
    return matrix[::thread_cnt][:dim * dim].reshape(dim, dim).T


def extractVector(dim, thread_cnt, vector):
    """pyx:95-96."""
    return vector[::thread_cnt][:dim]


# --------------------------- reference test helpers ---------------------------
def test_backsubs(dim, block_cnt, thread_cnt):
    """pyx:98-113: returns a.x - b for a random upper-triangular a."""
    a = np.random.random((dim, dim))
    a = np.triu(a)
    ra = np.zeros(dim * dim * thread_cnt * block_cnt, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim * dim)), ra)
    x = np.random.random(dim)
    rx = np.zeros(dim * thread_cnt * block_cnt, dtype='double')
    ix = np.zeros_like(rx)
    my_repVector(dim, block_cnt, thread_cnt, x, rx)
    my_backsubs(dim, block_cnt, thread_cnt, ra, ia, rx, ix)
    sol = extractVector(dim, thread_cnt, rx)
    return a.dot(sol) - x


def test_zgehrd(dim, block_cnt, thread_cnt):
    """pyx:115-125: returns (reduced matrix of slot 0, a)."""
    a = np.random.random((dim, dim))
    ra = np.zeros(dim * dim * thread_cnt * block_cnt, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim * dim)), ra)
    rtau = np.zeros(dim * thread_cnt * block_cnt, dtype='double')
    itau = np.zeros_like(rtau)
    my_zgehrd(dim, block_cnt, thread_cnt, ra, ia, rtau, itau)
    erg = extractMatrix(dim, thread_cnt, ra) + 1.0j * extractMatrix(dim, thread_cnt, ia)
    return erg, a


def test_hessenberg(dim, block_cnt, thread_cnt):
    """pyx:127-141: returns (h, q, a)."""
    a = np.random.random((dim, dim))
    ra = np.zeros(dim * dim * thread_cnt * block_cnt, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim * dim)), ra)
    rq = np.zeros_like(ra)
    iq = np.zeros_like(rq)
    my_hessenberg(dim, block_cnt, thread_cnt, ra, ia, rq, iq)
    h = extractMatrix(dim, thread_cnt, ra) + 1.0j * extractMatrix(dim, thread_cnt, ia)
    q = extractMatrix(dim, thread_cnt, rq) + 1.0j * extractMatrix(dim, thread_cnt, iq)
    return h, q, a


def test_zgemv(dim, block_cnt, thread_cnt, hermitian=False):
    """pyx:143-166: returns |computed - expected| (real part, as the reference)."""
    a = np.random.random((dim, dim))
    ra = np.zeros(dim * dim * thread_cnt * block_cnt, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim * dim)), ra)
    y = np.random.random(dim)
    ry = np.zeros(dim * thread_cnt * block_cnt, dtype='double')
    iy = np.zeros_like(ry)
    my_repVector(dim, block_cnt, thread_cnt, y, ry)
    x = np.random.random(dim)
    rx = np.zeros_like(iy)
    ix = np.zeros_like(rx)
    my_repVector(dim, block_cnt, thread_cnt, x, rx)
    my_zgemv(hermitian, dim, block_cnt, thread_cnt, ra, ia, rx, ix, 1.0, 0.0, ry, iy)
    axpy = extractVector(dim, thread_cnt, ry)
    if hermitian:
        sol = np.conj(a.T).dot(x) + y
    else:
        sol = a.dot(x) + y
    return np.abs(axpy - sol)


def test_zlahqr(dim, block_cnt, thread_cnt):
    """pyx:168-193: returns (eigs, schur vectors, T, a) for a random Hessenberg a."""
    dim2 = dim * dim
    size = dim2 * block_cnt * thread_cnt
    sizev = dim * block_cnt * thread_cnt
    a = np.random.random((dim, dim))
    a = np.triu(a, -1)
    ra = np.zeros(size, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim2)), ra)
    s = np.eye(dim)
    rschur = np.zeros(size, dtype='double')
    ischur = np.zeros(size, dtype='double')
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(s.T.reshape(dim2)), rschur)
    re = np.zeros(sizev, dtype='double')
    ie = np.zeros(sizev, dtype='double')
    my_zlahqr(dim, block_cnt, thread_cnt, re, ie, ra, ia, rschur, ischur)
    eigs = extractVector(dim, thread_cnt, re) + 1.0j * extractVector(dim, thread_cnt, ie)
    schurv = extractMatrix(dim, thread_cnt, rschur) + 1.0j * extractMatrix(dim, thread_cnt, ischur)
    t = extractMatrix(dim, thread_cnt, ra) + 1.0j * extractMatrix(dim, thread_cnt, ia)
    return (eigs, schurv, t, a)


def test_eigenvectors(dim, block_cnt, thread_cnt):
    """pyx:195-220: returns (eigs, eigenvectors, a) for a random Hessenberg a."""
    dim2 = dim * dim
    size = dim2 * block_cnt * thread_cnt
    sizev = dim * block_cnt * thread_cnt
    a = np.random.random((dim, dim))
    a = np.triu(a, -1)
    ra = np.zeros(size, dtype='double')
    ia = np.zeros_like(ra)
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(a.T.reshape(dim2)), ra)
    s = np.eye(dim)
    rsch = np.zeros(size, dtype='double')
    isch = np.zeros(size, dtype='double')
    my_repMatrix(dim, block_cnt, thread_cnt, np.ascontiguousarray(s.T.reshape(dim2)), rsch)
    re = np.zeros(sizev, dtype='double')
    ie = np.zeros(sizev, dtype='double')
    my_zlahqr(dim, block_cnt, thread_cnt, re, ie, ra, ia, rsch, isch)
    my_ztrevec(dim, block_cnt, thread_cnt, ra, ia, rsch, isch)
    eigs = extractVector(dim, thread_cnt, re) + 1.0j * extractVector(dim, thread_cnt, ie)
    vecs = extractMatrix(dim, thread_cnt, rsch) + 1.0j * extractMatrix(dim, thread_cnt, isch)
    return (eigs, vecs, a)
