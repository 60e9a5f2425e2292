// ref_harness.cpp -- C entry points over the UNMODIFIED reference sources.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) with the
// reference directory on the include path; the reference's utils.cpp (which in
// turn includes Toolbox.hpp and ComplexDouble.hpp) is compiled as-is with the
// reference's own CPU flags (-O3 -fopenmp -DOPENMP, Makefile:18).  The result
// lands in oracle/_ref/ and is used only to pin the C restatement in
// ves_oracle.c and, where it exists, as the timed CPU reference.
#include "utils.cpp"

#include <omp.h>

extern "C" {

void ref_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

// The shipped host wrappers.  call_zgehrd, call_zunghr and hessenberg hand
// the batch kernels work arrays from `new double[]` without initialising
// them, and zgemv_simple scales them by beta = 0 before accumulating
// (Toolbox.hpp:1068-1078): whatever NaN bit patterns the heap holds leak
// into the results.
void ref_call_zgehrd(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{ call_zgehrd(dim, bc, tc, rA, iA, rtau, itau); }

void ref_call_zunghr(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{ call_zunghr(dim, bc, tc, rA, iA, rtau, itau); }

void ref_hessenberg(int dim, int bc, int tc, double *rA, double *iA, double *rQ, double *iQ)
{ hessenberg(dim, bc, tc, rA, iA, rQ, iQ); }

// The same batch kernels (test_zgehrd, test_zunghr) with zero-initialised
// work arrays: deterministic outputs for the fixtures.
void ref_zgehrd_zw(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{
  size_t nv = (size_t)dim * bc * tc;
  double *rw = new double[nv](), *iw = new double[nv]();
  test_zgehrd(rA, iA, rtau, itau, rw, iw, dim, bc, tc);
  delete[] rw; delete[] iw;
}

void ref_zunghr_zw(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{
  size_t nv = (size_t)dim * bc * tc;
  double *rw = new double[nv](), *iw = new double[nv]();
  test_zunghr(rA, iA, rtau, itau, rw, iw, dim, bc, tc);
  delete[] rw; delete[] iw;
}

void ref_hessenberg_zw(int dim, int bc, int tc, double *rA, double *iA, double *rQ, double *iQ)
{
  size_t nv = (size_t)dim * bc * tc, nm = nv * dim;
  double *rt = new double[nv](), *it = new double[nv]();
  ref_zgehrd_zw(dim, bc, tc, rA, iA, rt, it);
  memcpy(rQ, rA, nm * sizeof(double));
  memcpy(iQ, iA, nm * sizeof(double));
  ref_zunghr_zw(dim, bc, tc, rQ, iQ, rt, it);
  delete[] rt; delete[] it;
}

void ref_call_zlahqr_new(int dim, int bc, int tc, double *rE, double *iE, double *rM, double *iM,
                         double *rS, double *iS)
{ call_zlahqr_new(dim, bc, tc, rE, iE, rM, iM, rS, iS); }

void ref_call_ztrevc(int dim, int bc, int tc, double *rT, double *iT, double *rR, double *iR)
{ call_ztrevc(dim, bc, tc, rT, iT, rR, iR); }

void ref_call_zgemv(int hermitian, int dim, int bc, int tc, double *rM, double *iM, double *rx, double *ix,
                    double *ry, double *iy, double rbeta, double ibeta)
{ call_zgemv(hermitian != 0, dim, bc, tc, rM, iM, rx, ix, ry, iy, rbeta, ibeta); }

void ref_call_backsubstitution(int dim, int bc, int tc, double *rT, double *iT, double *rb, double *ib)
{ call_backsubstitution(dim, bc, tc, rT, iT, rb, ib); }

// The shipped driver (utils.cpp:578), unchanged: reflector storage is passed
// into the QR sweep.  Prints its own elapsed time to stdout.
void ref_eigensolver_shipped(int dim, int bc, int tc, double *rA, double *iA, double *rE, double *iE,
                             double *rV, double *iV)
{ eigensolver(dim, bc, tc, rA, iA, rE, iE, rV, iV); }

// The same four batch kernels with H(i,j), i >= j+2, cleared between zunghr
// and zlahqr -- the step LAPACK zlahqr performs on entry.
void ref_eigensolver_cleared(int dim, int bc, int tc, double *rA, double *iA, double *rE, double *iE,
                             double *rV, double *iV)
{
  size_t nv = (size_t)dim * bc * tc, nm = nv * dim;
  double *rtau = new double[nv](), *itau = new double[nv]();
  double *rwork = new double[2 * nv](), *iwork = new double[2 * nv]();
  test_zgehrd(rA, iA, rtau, itau, rwork, iwork, dim, bc, tc);
  memcpy(rV, rA, nm * sizeof(double));
  memcpy(iV, iA, nm * sizeof(double));
  test_zunghr(rV, iV, rtau, itau, rwork, iwork, dim, bc, tc);
#pragma omp parallel for schedule(static, 8)
  for (int b = 0; b < bc; ++b)
    for (int t = 0; t < tc; ++t)
      for (int j = 0; j < dim; ++j)
        for (int i = j + 2; i < dim; ++i) {
          size_t k = (size_t)b * tc * dim * dim + (size_t)(i + j * dim) * tc + t;
          rA[k] = 0.0;
          iA[k] = 0.0;
        }
  zlahqr_new(rE, iE, rA, iA, rV, iV, dim, dim * dim, bc, tc);
  test_ztrevc(rA, iA, rV, iV, rwork, iwork, dim, dim * dim, bc, tc);
  delete[] rtau; delete[] itau; delete[] rwork; delete[] iwork;
}

void ref_repMatrixSoA(int dim, int bc, int tc, double *m, double *out) { repMatrixSoA(dim, bc, tc, m, out); }
void ref_repVectorSoA(int dim, int bc, int tc, double *v, double *out) { repVectorSoA(dim, bc, tc, v, out); }
void ref_rearrangeMatrices(int dim, int bc, int tc, double *in, double *out) { rearrangeMatrices(dim, bc, tc, in, out); }
void ref_arrangeMatricesAoS(int dim, int bc, int tc, double *in, double *out) { arrangeMatricesAoS(dim, bc, tc, in, out); }

}  // extern "C"
