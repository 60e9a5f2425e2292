// ves_dropin_cxx.cpp -- the reference host API with C++ linkage.
//
// kipfstuhl/vectorized-eigensolver declares its host entry points as plain
// C++ functions (utils.h:37-65, defined in utils.cpp), and its Cython module
// binds utils.cpp the same way (python_interface.pyx:10-29).  A program
// compiled against utils.h therefore refers to the mangled C++ names, not to
// the C names that include/ves.h exports.  This file defines exactly those
// C++ signatures, so such a program links against libves.so with no source
// change; each forwards to the same body as the C entry point of the same
// name (ves_api.cu).  It must not include ves.h: a C++ function and an
// extern "C" function with one name and one parameter list cannot be
// declared in the same translation unit.
#include <cstdio>
#include <string>
#include <vector>

#include "ves_internal.h"

// utils.h:42
void repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out)
{
    ves::dropin_repMatrixSoA(dim, block_cnt, thread_cnt, matrix, out);
}

// utils.h:43
void repVectorSoA(int dim, int block_cnt, int thread_cnt, double *vec, double *out)
{
    ves::dropin_repVectorSoA(dim, block_cnt, thread_cnt, vec, out);
}

// utils.cpp:85 (bound by python_interface.pyx:14)
void rearrangeMatrices(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    ves::dropin_rearrangeMatrices(dim, block_cnt, thread_cnt, in, out);
}

// utils.cpp:105
void arrangeMatricesAoS(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    ves::dropin_arrangeMatricesAoS(dim, block_cnt, thread_cnt, in, out);
}

// utils.h:45-46
void call_zlahqr_new(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM,
                     double *rS, double *iS)
{
    ves::dropin_call_zlahqr_new(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS);
}

// utils.h:48-50
void call_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, double *rM, double *iM, double *rx,
                double *ix, double *ry, double *iy, double rbeta, double ibeta)
{
    ves::dropin_call_zgemv(hermitian, dim, block_cnt, thread_cnt, rM, iM, rx, ix, ry, iy, rbeta, ibeta);
}

// utils.h:51-52
void call_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR)
{
    ves::dropin_call_ztrevc(dim, block_cnt, thread_cnt, rT, iT, rR, iR);
}

// utils.cpp:269 (bound by python_interface.pyx:24-25)
void call_backsubstitution(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rb, double *ib)
{
    ves::dropin_call_backsubstitution(dim, block_cnt, thread_cnt, rT, iT, rb, ib);
}

// utils.h:54
void call_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    ves::dropin_call_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau);
}

// utils.h:56
void call_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    ves::dropin_call_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau);
}

// utils.h:58
void hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ)
{
    ves::dropin_hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ);
}

// utils.h:62-63
void eigensolver(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rE, double *iE,
                 double *rV, double *iV)
{
    ves::dropin_eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV);
}

namespace {

// dim*dim*n_matrices doubles of raw binary (the SoA plane as the reference's
// readMatricesFromFile, utils.cpp:77-83, reads it); false if the file is
// missing or short.
bool read_plane(const std::string &path, std::vector<double> &out)
{
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    const size_t got = std::fread(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return got == out.size();
}

}  // namespace

// utils.h:60 (utils.cpp:481-576): the same solve on the SoA planes read from
// two binary files (real and imaginary parts, block_cnt * thread_cnt matrices
// of order dim in the layout of eigensolver()).  As in the reference the
// results are not returned: the call is the reference's timing driver.  The
// reference copies A into its Q buffer with a count of doubles passed as a
// byte count (utils.cpp:508-509), so its Q starts from an eighth of A; here
// the whole solve of eigensolver() runs.  A missing or short file is reported
// on stderr and through ves_last_error() instead of solving uninitialised
// memory.
void eigensolver(int dim, int block_cnt, int thread_cnt, std::string real, std::string imag)
{
    if (dim < 1 || block_cnt < 0 || thread_cnt < 1) {
        ves::set_error_message("eigensolver: invalid sizes");
        std::fprintf(stderr, "eigensolver: invalid sizes\n");
        return;
    }
    const size_t nm = (size_t)dim * dim * (size_t)block_cnt * thread_cnt, nv = (size_t)dim * block_cnt * thread_cnt;
    std::vector<double> rA(nm), iA(nm), rE(nv), iE(nv), rV(nm), iV(nm);
    if (!read_plane(real, rA) || !read_plane(imag, iA)) {
        ves::set_error_message("eigensolver: cannot read the matrix files");
        std::fprintf(stderr, "eigensolver: cannot read %zu doubles from %s and %s\n", nm, real.c_str(), imag.c_str());
        return;
    }
    ves::dropin_eigensolver(dim, block_cnt, thread_cnt, rA.data(), iA.data(), rE.data(), iE.data(), rV.data(),
                            iV.data());
}
