"""Generate tests/golden/ref_golden.npz from the compiled reference.

Runs the UNMODIFIED reference sources (built by `make -C oracle ref` into
oracle/_ref/libref.so, which needs the reference checkout) on small seeded
batches and stores inputs and outputs of every entry point on the path.  The
fixtures pin the C restatement (oracle/ves_oracle.c) and the GPU product on
machines where the reference itself is not available.

    python tests/golden/make_golden.py

Entries (one group of keys per case, prefix "<case>/"):
  eig:        full path with H(i,j), i >= j+2 cleared before the QR sweep
              (ref_eigensolver_cleared): inputs rA,iA -> rE,iE,rV,iV
  shipped:    the shipped eigensolver() without that step (defect B1)
  zgehrd:     test_zgehrd with zeroed work (call_zgehrd's work arrays are
              uninitialised and leak NaNs) -> rA,iA (H + reflectors), rtau,itau
  hess:       test_zgehrd + copy + test_zunghr with zeroed work -> rH,iH, rQ,iQ
  zlahqr:     call_zlahqr_new on a clean Hessenberg input -> rE,iE, rT,iT, rS,iS
  ztrevc:     call_ztrevc on (T, S) of the zlahqr case -> rR,iR
  zgemv:      call_zgemv, hermitian=False, complex beta; hermitian=True, beta=0
  backsubs:   call_backsubstitution on an upper-triangular T
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "vectorized-eigensolver_gb300"))

import oracle  # noqa: E402
from oracle import ptr  # noqa: E402
import ves  # noqa: E402  (layout helpers only; no GPU)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")

# (name, dim, block_cnt, thread_cnt, seed)
CASES = [
    ("n1", 1, 2, 4, 101),
    ("n2", 2, 4, 4, 102),
    ("n3", 3, 3, 8, 103),
    ("n4_aos", 4, 16, 1, 104),
    ("n5", 5, 2, 8, 105),
    ("n8", 8, 8, 4, 106),
    ("n12", 12, 1, 16, 107),
    ("n16", 16, 1, 8, 108),
    ("n24", 24, 1, 2, 109),
    ("n32", 32, 1, 2, 110),
]


def cgauss(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def main():
    oracle.build(ref=True)
    R = oracle.reference()
    if R is None:
        sys.exit("reference build not available (needs the reference checkout)")
    R.ref_set_threads(1)
    out = {}
    for name, n, bc, tc, seed in CASES:
        rng = np.random.default_rng(seed)
        N = bc * tc
        A = cgauss(rng, (N, n, n))
        rA, iA = ves.soa_from_complex(A, tc)
        p = name + "/"
        out[p + "dims"] = np.array([n, bc, tc])
        out[p + "rA"], out[p + "iA"] = rA.copy(), iA.copy()

        # full path, cleared and shipped
        for tag, fn in (("eig", R.ref_eigensolver_cleared), ("shipped", R.ref_eigensolver_shipped)):
            a_r, a_i = rA.copy(), iA.copy()
            e_r, e_i = np.zeros(N * n), np.zeros(N * n)
            v_r, v_i = np.zeros_like(a_r), np.zeros_like(a_i)
            fn(n, bc, tc, ptr(a_r), ptr(a_i), ptr(e_r), ptr(e_i), ptr(v_r), ptr(v_i))
            out[p + tag + "_rE"], out[p + tag + "_iE"] = e_r, e_i
            out[p + tag + "_rV"], out[p + tag + "_iV"] = v_r, v_i

        # zgehrd
        a_r, a_i = rA.copy(), iA.copy()
        t_r, t_i = np.zeros(N * n), np.zeros(N * n)
        R.ref_zgehrd_zw(n, bc, tc, ptr(a_r), ptr(a_i), ptr(t_r), ptr(t_i))
        out[p + "zgehrd_rA"], out[p + "zgehrd_iA"] = a_r, a_i
        out[p + "zgehrd_rtau"], out[p + "zgehrd_itau"] = t_r, t_i

        # hessenberg
        a_r, a_i = rA.copy(), iA.copy()
        q_r, q_i = np.zeros_like(a_r), np.zeros_like(a_i)
        R.ref_hessenberg_zw(n, bc, tc, ptr(a_r), ptr(a_i), ptr(q_r), ptr(q_i))
        out[p + "hess_rH"], out[p + "hess_iH"] = a_r, a_i
        out[p + "hess_rQ"], out[p + "hess_iQ"] = q_r, q_i

        # zlahqr on a clean (upper Hessenberg) input, then ztrevc
        Hs = np.triu(cgauss(rng, (N, n, n)), -1)
        h_r, h_i = ves.soa_from_complex(Hs, tc)
        out[p + "zlahqr_rH"], out[p + "zlahqr_iH"] = h_r.copy(), h_i.copy()
        e_r, e_i = np.zeros(N * n), np.zeros(N * n)
        s_r, s_i = np.zeros_like(h_r), np.zeros_like(h_i)
        R.ref_call_zlahqr_new(n, bc, tc, ptr(e_r), ptr(e_i), ptr(h_r), ptr(h_i), ptr(s_r), ptr(s_i))
        out[p + "zlahqr_rE"], out[p + "zlahqr_iE"] = e_r, e_i
        out[p + "zlahqr_rT"], out[p + "zlahqr_iT"] = h_r.copy(), h_i.copy()
        out[p + "zlahqr_rS"], out[p + "zlahqr_iS"] = s_r.copy(), s_i.copy()
        R.ref_call_ztrevc(n, bc, tc, ptr(h_r), ptr(h_i), ptr(s_r), ptr(s_i))
        out[p + "ztrevc_rR"], out[p + "ztrevc_iR"] = s_r, s_i

        # zgemv
        M = cgauss(rng, (N, n, n))
        x = cgauss(rng, (N, n))
        y = cgauss(rng, (N, n))
        m_r, m_i = ves.soa_from_complex(M, tc)
        x_r, x_i = ves.soa_vec_from_complex(x, tc)
        y_r, y_i = ves.soa_vec_from_complex(y, tc)
        out[p + "zgemv_rM"], out[p + "zgemv_iM"] = m_r, m_i
        out[p + "zgemv_rx"], out[p + "zgemv_ix"] = x_r, x_i
        out[p + "zgemv_ry0"], out[p + "zgemv_iy0"] = y_r.copy(), y_i.copy()
        yr, yi = y_r.copy(), y_i.copy()
        R.ref_call_zgemv(0, n, bc, tc, ptr(m_r), ptr(m_i), ptr(x_r), ptr(x_i), ptr(yr), ptr(yi), 0.5, -0.25)
        out[p + "zgemv_n_ry"], out[p + "zgemv_n_iy"] = yr, yi
        yr, yi = y_r.copy(), y_i.copy()
        R.ref_call_zgemv(1, n, bc, tc, ptr(m_r), ptr(m_i), ptr(x_r), ptr(x_i), ptr(yr), ptr(yi), 0.0, 0.0)
        out[p + "zgemv_h_ry"], out[p + "zgemv_h_iy"] = yr, yi

        # back substitution on a well-conditioned upper-triangular T
        T = np.triu(cgauss(rng, (N, n, n))) + 3.0 * np.eye(n)[None]
        b = cgauss(rng, (N, n))
        tr, ti = ves.soa_from_complex(T, tc)
        br, bi = ves.soa_vec_from_complex(b, tc)
        out[p + "bs_rT"], out[p + "bs_iT"] = tr, ti
        out[p + "bs_rb"], out[p + "bs_ib"] = br.copy(), bi.copy()
        R.ref_call_backsubstitution(n, bc, tc, ptr(tr), ptr(ti), ptr(br), ptr(bi))
        out[p + "bs_rx"], out[p + "bs_ix"] = br, bi

    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
