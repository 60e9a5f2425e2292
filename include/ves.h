/*
 * ves.h -- C ABI of libves.so, the GB300 (sm_103a) batched complex eigensolver.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the names, argument order and semantics of the
 *    reference kipfstuhl/vectorized-eigensolver host API (utils.h:37-65,
 *    utils.cpp): HOST pointers, synchronous, void return.  The matrices of a
 *    batch live in the reference's structure-of-arrays layout: n_matrices =
 *    block_cnt * thread_cnt matrices of order dim, real and imaginary parts in
 *    separate double arrays; matrix m = b*thread_cnt + t has its 0-based
 *    column-major element (i,j) at b*thread_cnt*dim*dim + (i + j*dim)*thread_cnt + t,
 *    and a length-dim vector at b*thread_cnt*dim + i*thread_cnt + t.
 *    thread_cnt is a layout parameter only; the GPU launch shape is chosen
 *    independently.  On failure (no GPU, bad sizes, CUDA error) these print a
 *    message to stderr and record it for ves_last_error(); outputs are then
 *    undefined.  There is no CPU fallback.
 *
 * 2. Native entry points (ves_*): DEVICE pointers in the same layout, work
 *    enqueued on a caller-supplied CUDA stream (pass the cudaStream_t as
 *    void*; NULL = legacy default stream), per-matrix status, an options
 *    struct, and an int return code (0 = success, negative = error, message in
 *    ves_last_error()).
 */
#ifndef VES_H_
#define VES_H_

#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ======================================================================= */
/* 1. Drop-in layer (reference utils.h).                                    */
/* ======================================================================= */

/* Full eigen-decomposition: eigenvalues (E) and right eigenvectors (V) of every
 * matrix in A.  A is overwritten with the upper-triangular Schur form T.
 * Replaces eigensolver(int, int, int, double*, ...) of utils.cpp:578-698
 * (declared utils.h:62-63).  Eigenvalues come in Schur order (diagonal of T),
 * eigenvector k = Z*[x;1;0] exactly as the reference scales it; the reference
 * feeds zgehrd's reflector storage into the QR sweep (utils.cpp:613) and so
 * returns wrong eigenvalues -- this entry point clears it first, as LAPACK's
 * zlahqr does. */
void eigensolver(int dim, int block_cnt, int thread_cnt,
                 double *rA, double *iA, double *rE, double *iE, double *rV, double *iV);

/* Hessenberg form A = Q H Q^H: H (with the reflectors below the subdiagonal,
 * as zgehrd leaves them) in A, Q in (rQ, iQ).  Replaces hessenberg() of
 * utils.cpp:417-479 (utils.h:58).  Reflector signs follow LAPACK, so H and Q
 * may differ from the reference's by a diagonal unitary similarity. */
void hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ);

/* Householder reduction: H and reflectors in A, tau in (rtau, itau) (dim
 * entries per matrix, the last unused).  Replaces call_zgehrd of
 * utils.cpp:330-374 (utils.h:54). */
void call_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau);

/* Q from the output of call_zgehrd, in place in A.  Replaces call_zunghr of
 * utils.cpp:376-415 (utils.h:56). */
void call_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau);

/* Schur decomposition of upper Hessenberg M: M -> T, S -> Schur vectors (S is
 * reset to the identity on entry, as the reference does at utils.cpp:167-169),
 * E = diag(T).  Entries below the subdiagonal of M are treated as zero.
 * Replaces call_zlahqr_new of utils.cpp:159-216 (utils.h:45-46). */
void call_zlahqr_new(int dim, int block_cnt, int thread_cnt, double *rE, double *iE,
                     double *rM, double *iM, double *rS, double *iS);

/* Right eigenvectors of upper-triangular T back-transformed by R, in place in
 * R.  T is left unchanged.  Replaces call_ztrevc of utils.cpp:279-328 (utils.h:51-52). */
void call_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR);

/* y := M x + beta y (hermitian = false) or M^H x + beta y.  Replaces call_zgemv
 * of utils.cpp:218-267 (utils.h:48-50); the imaginary part of y is read in the
 * Hermitian branch (the reference reads the real part, Toolbox.hpp:1125). */
void call_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, double *rM, double *iM,
                double *rx, double *ix, double *ry, double *iy, double rbeta, double ibeta);

/* Solve T x = b, T upper triangular, b in (rb, ib) on entry, x on exit.
 * Replaces call_backsubstitution of utils.cpp:269-277 (declared in the Cython
 * interface, python_interface.pyx:24-25; CPU-only in the reference). */
void call_backsubstitution(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rb, double *ib);

/* Host-side layout helpers, same semantics as utils.cpp:85-157. */
void repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out);  /* utils.h:42 */
void repVectorSoA(int dim, int block_cnt, int thread_cnt, double *vec, double *out);     /* utils.h:43 */
void rearrangeMatrices(int dim, int block_cnt, int thread_cnt, double *in, double *out); /* utils.cpp:85, pyx:16 */
void arrangeMatricesAoS(int dim, int block_cnt, int thread_cnt, double *in, double *out);/* utils.cpp:105 */

/* ======================================================================= */
/* 2. Native layer: device pointers, stream-ordered.                        */
/* ======================================================================= */

enum {
    VES_OK = 0,
    VES_ERR_ARG = -1,    /* invalid sizes or pointers */
    VES_ERR_CUDA = -2,   /* a CUDA call failed */
    VES_ERR_NOMEM = -3,  /* device allocation failed */
    VES_ERR_UNSUPPORTED = -4
};

/* per-matrix status bits (int32 per matrix, plain index m = b*thread_cnt + t) */
enum {
    VES_STATUS_ITCAP = 1,           /* an eigenvalue used up its sweep budget (the reference moves on silently) */
    VES_STATUS_NONFINITE = 2,       /* input held Inf/NaN; outputs are NaN */
    VES_STATUS_SHIFT_FALLBACK = 4,  /* learned shift replaced by Wilkinson's at least once */
    VES_STATUS_REFINE_FALLBACK = 8  /* mixed precision: re-solved in FP64 */
};

enum { VES_PREC_FP64 = 0, VES_PREC_FP32_REFINE = 1 };
enum { VES_VNORM_REFERENCE = 0, VES_VNORM_MAX = 1, VES_VNORM_TWO = 2 };

typedef struct ves_options {
    int precision;     /* VES_PREC_*; default FP64 */
    int max_its;       /* sweeps per eigenvalue = max_its + 1; default 30 (reference Toolbox.hpp:808) */
    int vnorm;         /* eigenvector scaling, VES_VNORM_*; default REFERENCE */
    int refine_steps;  /* FP32_REFINE: Newton corrections per eigenpair before falling back to FP64; default 3 */
    double refine_tol; /* FP32_REFINE: accept when ||A v - lambda v|| <= refine_tol ||A||_F ||v||; default 5e-14 */
    int reserved[6];
} ves_options;

void ves_default_options(ves_options *opt);

/* Bytes of device workspace ves_eigensolve needs for this batch. */
size_t ves_eigensolve_workspace_size(int dim, int block_cnt, int thread_cnt, const ves_options *opt);

/* Full eigen-decomposition on device data.
 * precision = VES_PREC_FP64: the reference path in FP64 (one launch).
 * precision = VES_PREC_FP32_REFINE: the reference path in complex FP32, then
 *   every eigenpair refined by Newton steps whose residual is computed in
 *   FP64, until ||A v - lambda v|| <= refine_tol ||A||_F ||v||; a matrix that
 *   does not get there (or whose FP32 QR hit the sweep cap, or whose data do
 *   not fit FP32) is solved again in FP64 (status bit VES_STATUS_REFINE_FALLBACK).
 *   Eigenvalues come in the FP32 Schur order; the REFERENCE eigenvector scaling
 *   (unit component along the k-th Schur vector) then holds to FP32 accuracy.
 *   rT/iT must be NULL in this mode.
 * rA/iA are read only.  rT/iT
 * (nullable, may alias rA/iA) receive the Schur form.  status and sweeps
 * (nullable) receive one int per matrix: VES_STATUS_* bits and the number of
 * QR sweeps.  workspace may be NULL (the library then uses a cached
 * allocation of its own, grown on demand and held until ves_release()),
 * otherwise it must hold ves_eigensolve_workspace_size() bytes, 256-byte
 * aligned.  Asynchronous on `stream`. */
int ves_eigensolve(int dim, int block_cnt, int thread_cnt,
                   const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                   double *rT, double *iT, int *status, int *sweeps,
                   const ves_options *opt, void *workspace, size_t workspace_bytes, void *stream);

/* Stage entry points on device data (same semantics as the drop-ins above). */
int ves_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau, void *stream);
int ves_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, const double *rtau, const double *itau,
               void *stream);
int ves_hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ,
                   double *rtau, double *itau, void *stream);
int ves_zlahqr(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM,
               double *rS, double *iS, int *status, int max_its, void *stream);
/* rwork/iwork: dim*block_cnt*thread_cnt doubles each */
int ves_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR,
               double *rwork, double *iwork, void *stream);
int ves_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, const double *rM, const double *iM,
              const double *rx, const double *ix, double *ry, double *iy, double rbeta, double ibeta, void *stream);
int ves_backsubstitution(int dim, int block_cnt, int thread_cnt, const double *rT, const double *iT,
                         double *rb, double *ib, void *stream);

/* Measured FP64 FMA throughput of the current GPU in flop/s (an FMA counts
 * as 2 flops): the roofline denominator of the FP64-bound solver.  Runs a
 * few milliseconds of dependent-FMA chains on all SMs; synchronous.  No
 * counterpart in the reference. */
int ves_fp64_fma_rate(double *flops_per_s, void *stream);

/* Allocation-free variant of ves_eigensolve (FP64, reference eigenvector
 * scaling, no Schur-form or sweep output).  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory: hosts whose allocator is
 * owned by someone else, code that may not allocate (or let the driver
 * synchronise) after start-up.  It calls no cudaMalloc, cudaFree or other
 * allocating routine; its scratch space is a static device array of
 * VES_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * process exit.  The caller passes the inputs and outputs (device pointers,
 * layout as ves_eigensolve).  dim must not exceed VES_NOALLOC_MAX_DIM;
 * larger dims return VES_ERR_ARG with a message in ves_last_error().
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current: make that first call
 * before any stream capture.  All calls on a device share the array, so calls
 * that overlap on the GPU race and must be serialised by the caller.
 * Asynchronous on `stream`. */
#define VES_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
#define VES_NOALLOC_MAX_DIM 64
int ves_eigensolve_noalloc(int dim, int block_cnt, int thread_cnt,
                           const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                           int *status, void *stream);

/* Last error message of the calling thread ("" if none). */
const char *ves_last_error(void);
/* Free the library's cached device buffers. */
void ves_release(void);
/* Library version, major*10000 + minor*100 + patch. */
int ves_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* VES_H_ */
