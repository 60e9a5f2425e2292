"""The reference's host API with C++ linkage.

kipfstuhl/vectorized-eigensolver declares its host entry points as C++
functions (utils.h:37-65), so a program compiled against utils.h refers to
mangled names.  libves.so exports those next to the C names of
include/ves.h.  These tests compile a small C++ caller that declares the
reference's prototypes itself (no include of ves.h), link it against
libves.so and run it: on a CPU-only machine the call must fail loudly (no
CPU fallback); on a GPU it must give the C entry point's results bit for bit.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import ves

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vectorized-eigensolver_gb300")
CUDA_LIB = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")

# the mangled names a utils.h caller refers to (Itanium C++ ABI)
MANGLED = [
    "_Z11eigensolveriiiPdS_S_S_S_S_",                                             # utils.h:62-63
    "_Z11eigensolveriiiNSt7__cxx1112basic_stringIcSt11char_traitsIcESaIcEEES4_",  # utils.h:60
    "_Z10hessenbergiiiPdS_S_S_",                                                  # utils.h:58
    "_Z11call_zgehrdiiiPdS_S_S_",                                                 # utils.h:54
    "_Z11call_zunghriiiPdS_S_S_",                                                 # utils.h:56
    "_Z15call_zlahqr_newiiiPdS_S_S_S_S_",                                         # utils.h:45-46
    "_Z11call_ztrevciiiPdS_S_S_",                                                 # utils.h:51-52
    "_Z10call_zgemvbiiiPdS_S_S_S_S_dd",                                           # utils.h:48-50
    "_Z12repMatrixSoAiiiPdS_",                                                    # utils.h:42
    "_Z12repVectorSoAiiiPdS_",                                                    # utils.h:43
    "_Z17rearrangeMatricesiiiPdS_",                                               # utils.cpp:85
    "_Z18arrangeMatricesAoSiiiPdS_",                                              # utils.cpp:105
    "_Z21call_backsubstitutioniiiPdS_S_S_",                                       # utils.cpp:269
]

# A caller written against the reference's header: its prototypes, C++ linkage.
CALLER = r"""
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

void eigensolver(int dim, int block_cnt, int thread_cnt,
                 double *rA, double *iA, double *rE, double *iE, double *rV, double *iV);
void eigensolver(int dim, int block_cnt, int thread_cnt, std::string real, std::string imag);
void repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out);
extern "C" const char *ves_last_error(void);

static bool rd(const char *p, std::vector<double> &v)
{
    FILE *f = std::fopen(p, "rb");
    if (!f) return false;
    size_t g = std::fread(v.data(), 8, v.size(), f);
    std::fclose(f);
    return g == v.size();
}
static void wr(const char *p, const std::vector<double> &v)
{
    FILE *f = std::fopen(p, "wb");
    std::fwrite(v.data(), 8, v.size(), f);
    std::fclose(f);
}

int main(int argc, char **argv)
{
    // usage: caller dim block_cnt thread_cnt dir
    int dim = std::atoi(argv[1]), bc = std::atoi(argv[2]), tc = std::atoi(argv[3]);
    std::string d = argv[4];
    size_t nm = (size_t)dim * dim * bc * tc, nv = (size_t)dim * bc * tc;
    std::vector<double> rA(nm), iA(nm), rE(nv), iE(nv), rV(nm), iV(nm);
    if (!rd((d + "/rA.bin").c_str(), rA) || !rd((d + "/iA.bin").c_str(), iA)) return 3;
    // a host helper with C++ linkage: no GPU needed
    std::vector<double> m(dim * dim), rep(nm);
    for (int e = 0; e < dim * dim; ++e) m[e] = e;
    repMatrixSoA(dim, bc, tc, m.data(), rep.data());
    if (rep[(size_t)tc * 1 + 0] != 1.0) return 4;
    eigensolver(dim, bc, tc, rA.data(), iA.data(), rE.data(), iE.data(), rV.data(), iV.data());
    std::printf("error1=[%s]\n", ves_last_error());
    wr((d + "/rE.bin").c_str(), rE); wr((d + "/iE.bin").c_str(), iE);
    wr((d + "/rV.bin").c_str(), rV); wr((d + "/iV.bin").c_str(), iV);
    wr((d + "/rT.bin").c_str(), rA); wr((d + "/iT.bin").c_str(), iA);
    eigensolver(dim, bc, tc, d + "/rA.bin", d + "/iA.bin");   // the file-path overload
    std::printf("error2=[%s]\n", ves_last_error());
    eigensolver(dim, bc, tc, d + "/missing.bin", d + "/iA.bin");
    std::printf("error3=[%s]\n", ves_last_error());
    return 0;
}
"""


def test_cxx_names_exported():
    L = ctypes.CDLL(ves.LIBPATH if hasattr(ves, "LIBPATH") else os.path.join(PKG, "libves.so"))
    missing = [nm for nm in MANGLED if not hasattr(L, nm)]
    assert not missing, missing


def _build_caller(tmp_path):
    ves.lib()  # builds libves.so when the sources are newer
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    cmd = ["g++", "-std=c++17", "-O1", str(src), "-o", str(exe), "-L" + PKG, "-lves", "-Wl,-rpath," + PKG,
           "-Wl,-rpath," + CUDA_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _inputs(tmp_path, n, bc, tc, seed=7):
    rng = np.random.default_rng(seed)
    N = bc * tc
    A = rng.standard_normal((N, n, n)) + 1j * rng.standard_normal((N, n, n))
    rA, iA = ves.soa_from_complex(A, tc)
    rA.tofile(tmp_path / "rA.bin")
    iA.tofile(tmp_path / "iA.bin")
    return rA, iA


def _run(exe, tmp_path, n, bc, tc):
    r = subprocess.run([str(exe), str(n), str(bc), str(tc), str(tmp_path)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    return r


def test_cxx_caller_links_and_fails_loudly_without_gpu(tmp_path):
    """Links a utils.h-style C++ caller; with no GPU the drop-in reports an error (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("this machine has a GPU: covered by test_cxx_caller_matches_c_entry_point")
    exe = _build_caller(tmp_path)
    _inputs(tmp_path, 4, 2, 8)
    r = _run(exe, tmp_path, 4, 2, 8)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("error1=")][0]
    assert line != "error1=[]", r.stdout
    assert "eigensolver" in r.stderr


@pytest.mark.gpu
def test_cxx_caller_matches_c_entry_point(tmp_path):
    """The C++-linkage eigensolver() gives the C entry point's E, V and T bit for bit;
    the file-path overload solves without error and reports a missing file."""
    n, bc, tc = 12, 3, 32
    exe = _build_caller(tmp_path)
    rA, iA = _inputs(tmp_path, n, bc, tc)
    r = _run(exe, tmp_path, n, bc, tc)
    lines = dict(ln.split("=", 1) for ln in r.stdout.splitlines() if "=" in ln)
    assert lines["error1"] == "[]" and lines["error2"] == "[]", r.stdout
    assert lines["error3"] != "[]", r.stdout
    N = bc * tc
    E = [np.zeros(N * n) for _ in range(2)]
    V = [np.zeros(N * n * n) for _ in range(2)]
    T = [rA.copy(), iA.copy()]
    ves.eigensolver(n, bc, tc, T[0], T[1], E[0], E[1], V[0], V[1])
    for name, want in (("rE", E[0]), ("iE", E[1]), ("rV", V[0]), ("iV", V[1]), ("rT", T[0]), ("iT", T[1])):
        got = np.fromfile(tmp_path / (name + ".bin"))
        assert np.array_equal(got, want), name
