/*
 * ves_oracle.h -- CPU restatement of the reference eigensolver path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * product and the timed CPU baseline ("port") of the benchmark.  Nothing in
 * the product (libves.so, its Python mirror) links, loads or calls it.
 *
 * Layout contract (reference utils.cpp:85-157, Toolbox.hpp:2015-2020): a batch
 * of N = block_cnt*thread_cnt complex matrices of order `dim`, stored as two
 * separate double planes (real, imaginary).  Matrix m = b*thread_cnt + t has
 * its 0-based column-major element (i,j) at
 *      b*thread_cnt*dim*dim + (i + j*dim)*thread_cnt + t
 * and a length-dim vector belonging to it at b*thread_cnt*dim + i*thread_cnt + t.
 */
#ifndef VES_ORACLE_H_
#define VES_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* Number of OpenMP threads the batch loops use (0 = library default). */
void vo_set_threads(int nthreads);
int vo_get_threads(void);

/* Householder reduction to upper Hessenberg form (reference Toolbox.hpp:1315-1490,
 * batch loop :2150-2177).  On exit A holds H on and above the subdiagonal and the
 * reflector vectors below it; tau[dim] per matrix (the last entry is left as is). */
void vo_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA,
               double *rtau, double *itau);

/* Form Q from the reflectors left by vo_zgehrd (reference Toolbox.hpp:1492-1659,
 * batch loop :2179-2206).  Q holds a copy of the reduced A on entry. */
void vo_zunghr(int dim, int block_cnt, int thread_cnt, double *rQ, double *iQ,
               const double *rtau, const double *itau);

/* Zero H(i,j) for i >= j+2: the step LAPACK zlahqr performs on entry and the
 * reference omits (Toolbox.hpp:721-723). */
void vo_clear_below_subdiag(int dim, int block_cnt, int thread_cnt, double *rH, double *iH);

/* Single-shift complex QR with Schur vectors (reference Toolbox.hpp:690-1031 with
 * :138-369 and :14-29, batch loop :1984-2033).  H -> T in place, Z -> Z*S in place,
 * eigenvalues (diag T) in E.  `sweeps` (nullable, one int per matrix, plain
 * matrix index order) receives the number of QR sweeps performed. */
void vo_zlahqr(int dim, int block_cnt, int thread_cnt, double *rE, double *iE,
               double *rH, double *iH, double *rZ, double *iZ, int *sweeps);

/* Right eigenvectors of T back-transformed by Z, in place in Z (reference
 * Toolbox.hpp:1133-1313 with :31-136, batch loop :2060-2088).  T is restored on
 * exit except for rounding of the diagonal shifts.  Eigenvectors are scaled as
 * the reference leaves them: the T-eigenvector has a unit entry at position k. */
void vo_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT,
               double *rZ, double *iZ);

/* y := A*x + beta*y (hermitian = 0) or A^H*x + beta*y (hermitian = 1) on full
 * dim x dim matrices (reference Toolbox.hpp:1033-1131, batch loop :2118-2148),
 * with the Hermitian-branch defect at :1125 corrected (imag(y) is read). */
void vo_zgemv(int hermitian, int dim, int block_cnt, int thread_cnt,
              const double *rA, const double *iA, const double *rx, const double *ix,
              double rbeta, double ibeta, double *ry, double *iy);

/* Solve T x = b for upper-triangular T, b in x on entry (reference
 * Toolbox.hpp:31-136, batch loop :2090-2116). */
void vo_backsubstitution(int dim, int block_cnt, int thread_cnt,
                         const double *rT, const double *iT, double *rx, double *ix);

/* Full path: zgehrd -> copy -> zunghr -> clear -> zlahqr -> ztrevc, as the
 * reference's eigensolver() (utils.cpp:578-698) with the clearing step added.
 * A is overwritten with T; E gets eigenvalues in Schur order; V eigenvectors. */
void vo_eigensolver(int dim, int block_cnt, int thread_cnt,
                    double *rA, double *iA, double *rE, double *iE,
                    double *rV, double *iV, int *sweeps);

#ifdef __cplusplus
}
#endif

#endif /* VES_ORACLE_H_ */
