"""The bounds-checked build (libves_bc.so, -DVES_BOUNDS_CHECK) on small and
ragged cases of every kernel family: no matrix or vector index of the
numerical routines leaves its operand (the checked accessors count such an
index and redirect the access instead of touching memory outside), and the
results still meet the residual bar.  Runs in a child process bound to the
checked library (VES_LIBRARY), so the normal library of this process is
untouched."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vectorized-eigensolver_gb300")

CHILD = r'''
import ctypes, os, sys
import numpy as np
import torch
sys.path.insert(0, os.environ["VES_PKG"])
import ves

def cg(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()

def solve(A, tc, **opt):
    N, n, _ = A.shape
    rA, iA = ves.soa_from_complex(A, tc)
    dA = [dev(rA), dev(iA)]
    dE = [torch.empty(N * n, dtype=torch.float64, device="cuda") for _ in range(2)]
    want_v = opt.get("want_vectors", 1)
    dV = [torch.empty_like(dA[0]) for _ in range(2)] if want_v else [None, None]
    dT = [torch.empty_like(dA[0]) for _ in range(2)] if opt.pop("schur", False) else [None, None]
    st = torch.zeros(N, dtype=torch.int32, device="cuda")
    ves.eigensolve(n, N // tc, tc, dA[0], dA[1], dE[0], dE[1], dV[0], dV[1], dT[0], dT[1], st,
                   options=ves.default_options(**opt))
    torch.cuda.synchronize()
    E = ves.complex_vec_from_soa(dE[0].cpu().numpy(), dE[1].cpu().numpy(), n, tc)
    if want_v:
        V = ves.complex_from_soa(dV[0].cpu().numpy(), dV[1].cpu().numpy(), n, tc)
        R = A @ V - V * E[:, None, :]
        res = np.linalg.norm(R, axis=1) / (np.linalg.norm(A, axis=(1, 2))[:, None] * np.linalg.norm(V, axis=1))
        assert np.nanmax(res) <= 1e-13, (n, opt, np.nanmax(res))

rng = np.random.default_rng(5)
for n in (1, 2, 3, 8, 17):
    solve(cg(rng, (21, n, n)), 7, schur=True)                       # FP64 fused kernel, Schur output
    solve(cg(rng, (21, n, n)), 7, want_vectors=0)                   # eigenvalues only
for mode in ("lane", "group4", "group8", "warp16", "warp32"):
    os.environ["VES_MIXED_SCHUR"] = mode
    for n in (1, 2, 3, 9, 16, 24):
        solve(cg(rng, (45, n, n)), 9, precision=1)                  # FP32 Schur + refinement
os.environ.pop("VES_MIXED_SCHUR")
for n in (5, 40):
    solve(cg(rng, (40, n, n)), 8, precision=1, refine_steps=0)      # FP64 fallback: warp and lane kernels
# polynomial roots
deg, N = 6, 24
C = cg(rng, (N, deg + 1))
rC = np.ascontiguousarray(C.real.reshape(N // 8, 8, deg + 1).transpose(0, 2, 1)).reshape(-1)
iC = np.ascontiguousarray(C.imag.reshape(N // 8, 8, deg + 1).transpose(0, 2, 1)).reshape(-1)
rR = torch.empty(N * deg, dtype=torch.float64, device="cuda"); iR = torch.empty_like(rR)
ves.polyroots(deg, N // 8, 8, dev(rC), dev(iC), rR, iR)
# mixed-size batch, orders 1..12
sizes = rng.integers(1, 13, size=37)
mats = [cg(rng, (k, k)) for k in sizes]
re = np.concatenate([m.T.reshape(-1).real for m in mats]); im = np.concatenate([m.T.reshape(-1).imag for m in mats])
dims = dev(sizes.astype(np.int32))
er = torch.empty(int(sizes.sum()), dtype=torch.float64, device="cuda"); ei = torch.empty_like(er)
vr, vi = torch.empty(re.size, dtype=torch.float64, device="cuda"), torch.empty(re.size, dtype=torch.float64, device="cuda")
ves.eigensolve_varsize(len(sizes), 12, dims, dev(re), dev(im), er, ei, vr, vi)
# learned shifts: exact predictions, polish in the warp pre-pass (n = 8) and in the solve kernel (n = 40)
for n in (8, 40):
    A = cg(rng, (32, n, n))
    rA, iA = ves.soa_from_complex(A, 16)
    E = np.linalg.eigvals(A)
    Es = np.ascontiguousarray(E.reshape(2, 16, n).transpose(0, 2, 1)).reshape(-1)  # SoA vectors
    dS = [dev(Es.real.copy()), dev(Es.imag.copy())]
    out = [torch.empty(32 * n, dtype=torch.float64, device="cuda") for _ in range(2)] + \
          [torch.empty(32 * n * n, dtype=torch.float64, device="cuda") for _ in range(2)]
    ves.eigensolve_shifts(n, 2, 16, dev(rA), dev(iA), *out, dS[0], dS[1],
                          options=ves.default_options(shift_polish=3, shift_gate=0.0))
# the reference's stage entry points (host pointers) and the allocation-free path
n, bc, tc = 7, 3, 5
A = cg(rng, (bc * tc, n, n)); rA, iA = ves.soa_from_complex(A, tc)
t = [np.zeros(bc * tc * n) for _ in range(2)]
ves.call_zgehrd(n, bc, tc, rA.copy(), iA.copy(), t[0], t[1])
Q = [rA.copy(), iA.copy()]; ves.hessenberg(n, bc, tc, rA.copy(), iA.copy(), Q[0], Q[1])
E = [np.zeros(bc * tc * n) for _ in range(2)]; V = [np.zeros(rA.size) for _ in range(2)]
ves.eigensolver(n, bc, tc, rA.copy(), iA.copy(), E[0], E[1], V[0], V[1])
dA = [dev(rA), dev(iA)]
o = [torch.empty(bc * tc * n, dtype=torch.float64, device="cuda") for _ in range(2)] + [torch.empty_like(dA[0]) for _ in range(2)]
L = ves.lib()
assert L.ves_eigensolve_noalloc(n, bc, tc, *(ctypes.c_void_p(x.data_ptr()) for x in dA + o), None, None) == 0
torch.cuda.synchronize()
cnt = ctypes.c_ulonglong(99)
assert L.ves_bounds_violations(ctypes.byref(cnt), 1) == 0
print("VIOLATIONS", cnt.value)
'''


def test_bounds_checked_build_has_no_violations():
    sys.path.insert(0, PKG)
    import build as ves_build
    lib = ves_build.build(variant="bc")
    env = dict(os.environ, VES_LIBRARY=lib, VES_PKG=PKG, VES_AUTOBUILD="0")
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("VIOLATIONS")]
    assert line and line[0].split()[1] == "0", r.stdout[-2000:]

