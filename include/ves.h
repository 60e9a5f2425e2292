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
    VES_STATUS_REFINE_FALLBACK = 8, /* mixed precision: re-solved in FP64 */
    VES_STATUS_BAD_DIM = 16         /* mixed-size batch: order outside [1, max_dim], not solved */
};

enum { VES_PREC_FP64 = 0, VES_PREC_FP32_REFINE = 1 };
enum { VES_VNORM_REFERENCE = 0, VES_VNORM_MAX = 1, VES_VNORM_TWO = 2 };

typedef struct ves_options {
    int precision;     /* VES_PREC_*; default FP64 */
    int max_its;       /* sweeps per eigenvalue = max_its + 1; default 30 (reference Toolbox.hpp:808) */
    int vnorm;         /* eigenvector scaling, VES_VNORM_*; default REFERENCE */
    int refine_steps;  /* FP32_REFINE: Newton corrections per eigenpair before falling back to FP64; default 8 */
    double refine_tol; /* FP32_REFINE: accept when ||A v - lambda v|| <= refine_tol ||A||_F ||v|| and the
                        * correction that residual gives to lambda is <= 4 refine_tol ||A||_F; default 5e-14 */
    int want_vectors;  /* 1 (default): eigenvalues and eigenvectors; 0: eigenvalues only (FP64; the QR
                        * runs on the active block only, no Q and no Schur vectors -- the same
                        * eigenvalues, about a third of the QR work; rV/iV may be NULL) */
    int blocks_per_sm; /* launch shape of the persistent kernels (4 warps per block); 0 = library default */
    int varsize_order; /* mixed-size batches: 0 (default) largest order first, 1 smallest first */
    int shift_sweeps;  /* ves_eigensolve_shifts: sweeps per eigenvalue that use a predicted shift; default 1 */
    float shift_gate;  /* ves_eigensolve_shifts: an eigenvalue uses the predictions only while its subdiagonal
                        * |H(I,I-1)| exceeds shift_gate * ||A||_F / sqrt(n) (below that the Wilkinson shift
                        * is the better estimate); set it to the predictor's typical error; default 0 */
    int shift_polish;  /* ves_eigensolve_shifts: steps (0..64) of simultaneous Aberth iteration on det(H - sI)
                        * (FP32, Hyman's recurrence on the Hessenberg matrix) that refine all predictions of a
                        * matrix together before the QR, then one FP64 Newton step per prediction on the
                        * solve's own Hessenberg matrix; a prediction that does not converge or lands on an
                        * eigenvalue already seeded is dropped; for dim <= 32 the FP32 steps run as a
                        * warp-per-matrix pre-pass (environment VES_POLISH_METHOD=newton: each prediction on
                        * its own; VES_POLISH_FP64_STEP=0 / 2: no / two FP64 steps); 0 (default) = none */
    unsigned long long *work_counts; /* nullable DEVICE array of VES_WORK_COUNTS counters that the call ADDS to
                        * (zero them first; stream-ordered like the outputs): the work of the data-dependent
                        * stages, for flop accounting.  Default NULL. */
} ves_options;

/* Indices into ves_options.work_counts. */
enum {
    VES_WORK_RES64 = 0,   /* FP32_REFINE: FP64 residuals r = A v - lambda v (one per pair and Newton step) */
    VES_WORK_CORR32 = 1,  /* FP32_REFINE: FP32 Newton corrections through the Schur form */
    VES_WORK_RESFF = 2,   /* FP32_REFINE: first residuals in float-float (one per refined pair) */
    VES_WORK_POLISH = 3,  /* ves_eigensolve_shifts: FP32 Newton steps on det(H - sI), over all predictions */
    VES_WORK_COUNTS = 4
};

void ves_default_options(ves_options *opt);

/* Bytes of device workspace ves_eigensolve needs for this batch. */
size_t ves_eigensolve_workspace_size(int dim, int block_cnt, int thread_cnt, const ves_options *opt);

/* Full eigen-decomposition on device data.
 * precision = VES_PREC_FP64: the reference path in FP64 (one launch).
 * precision = VES_PREC_FP32_REFINE: the reference path in complex FP32, then
 *   every eigenpair refined by Newton steps whose residual is computed in
 *   FP64, until ||A v - lambda v|| <= refine_tol ||A||_F ||v|| and the next
 *   Newton correction to lambda (its error estimate) is <= 4 refine_tol
 *   ||A||_F; a matrix that does not get there within refine_steps corrections
 *   (or whose FP32 QR hit the sweep cap, or whose data do not fit FP32) is
 *   solved again in FP64 (status bit VES_STATUS_REFINE_FALLBACK).
 *   Eigenvalues come in the FP32 Schur order; the REFERENCE eigenvector scaling
 *   (unit component along the k-th Schur vector) then holds to FP32 accuracy.
 *   rT/iT must be NULL in this mode.
 * rA/iA are read only.  rT/iT
 * (nullable, may alias rA/iA) receive the Schur form.  status and sweeps
 * (nullable) receive one int per matrix: VES_STATUS_* bits and the number of
 * QR sweeps.  workspace may be NULL (the library then uses a cached
 * allocation of its own, grown on demand and held until ves_release(); it is
 * shared by every call on the device, so calls that can run at the same time
 * on different streams must each pass their own workspace), otherwise it must
 * hold ves_eigensolve_workspace_size() bytes, 256-byte aligned.  Asynchronous
 * on `stream`; for large batches of dim >= 32 the FP32 + refinement form runs
 * on two library streams forked from `stream` by an event and joined back into
 * it (VES_MIXED_OVERLAP=0 / 1 in the environment forces this off / on).
 * The two library streams are shared by all callers on a device: concurrent
 * FP32 + refinement calls from several host threads are correct (each with
 * its own workspace) but their overlapped stages run one call after the
 * other.  While `stream` is being captured into a CUDA graph the call stays
 * on `stream` (the two stages in sequence), so no library stream joins the
 * capture.  An FP32 + refinement pair is accepted only if no other eigenvalue
 * of its matrix lies within 16 refine_tol ||A||_F of it (two Newton runs that
 * converged to one eigenvalue would otherwise hide another); such a matrix is
 * solved in FP64 instead. */
int ves_eigensolve(int dim, int block_cnt, int thread_cnt,
                   const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                   double *rT, double *iT, int *status, int *sweeps,
                   const ves_options *opt, void *workspace, size_t workspace_bytes, void *stream);

/* Mixed-size batches (no counterpart in the reference, which solves one order
 * per call).  `count` matrices, matrix m of order dims[m] (device array), in
 * the packed layout: its dims[m]^2 elements column-major and contiguous at
 * element offset sum_{j<m} dims[j]^2 of each plane (rA, iA; the same layout for
 * rV, iV), its eigenvalues at sum_{j<m} dims[j] of rE, iE.  Orders must lie in
 * [1, max_dim] with max_dim <= VES_VARSIZE_MAX_DIM; other matrices are skipped
 * and flagged VES_STATUS_BAD_DIM.  The batch is binned by order on the device
 * and solved by one persistent FP64 launch (largest orders first unless
 * varsize_order = 1); no host synchronisation, so the call can be captured in
 * a CUDA graph (see ves_graph_capture_varsize).  workspace must hold
 * ves_eigensolve_varsize_workspace_size() bytes (or be NULL: cached). */
#define VES_VARSIZE_MAX_DIM 64
size_t ves_eigensolve_varsize_workspace_size(long long count, int max_dim, const ves_options *opt);
int ves_eigensolve_varsize(long long count, int max_dim, const int *dims,
                           const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                           int *status, int *sweeps, const ves_options *opt,
                           void *workspace, size_t workspace_bytes, void *stream);

/* A CUDA graph of one ves_eigensolve_varsize call (pointers, count and
 * options are baked in; the contents of dims and A may change between
 * launches).  workspace must not be NULL.  Replay with ves_graph_launch. */
typedef struct ves_graph ves_graph;
int ves_graph_capture_varsize(ves_graph **out, long long count, int max_dim, const int *dims,
                              const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                              int *status, int *sweeps, const ves_options *opt,
                              void *workspace, size_t workspace_bytes);
int ves_graph_launch(ves_graph *graph, void *stream);
void ves_graph_destroy(ves_graph *graph);

/* ---- learned shifts (no counterpart in the reference) ------------------------
 * ves_eigensolve_shifts: the FP64 solver of ves_eigensolve, except that for the
 * first opt->shift_sweeps sweeps of each eigenvalue the QR shift is the unused
 * predicted eigenvalue nearest to the Wilkinson estimate (rS, iS: n predictions
 * per matrix, SoA vectors like rE, iE).  After those sweeps, at the exceptional
 * sweeps, and whenever predictions run out, the reference's shifts are used;
 * results carry the same backward-error guarantee.  fallbacks (nullable) gets
 * per matrix the number of eigenvalues that needed more than shift_sweeps + 2
 * sweeps (VES_STATUS_SHIFT_FALLBACK marks those matrices). */
size_t ves_eigensolve_shifts_workspace_size(int dim, int block_cnt, int thread_cnt, const ves_options *opt);
int ves_eigensolve_shifts(int dim, int block_cnt, int thread_cnt,
                          const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                          const double *rS, const double *iS, int *status, int *sweeps, int *fallbacks,
                          const ves_options *opt, void *workspace, size_t workspace_bytes, void *stream);

/* The shift network: features [family parameters (n_params per matrix, a
 * row-major FP64 device array), optional sin/cos features of them, Re diag A,
 * Im diag A, optional subdiagonal norms] -> n predicted eigenvalues; hidden
 * layers of `hidden` units, GELU, BF16 on the tcgen05 tensor cores; an FP32
 * output layer.  Trained on eigenvalues from the FP64 solver (rE, iE in the
 * SoA layout of rA, iA) with a permutation-invariant
 * loss (symmetric Chamfer distance between the predicted and the true
 * eigenvalue sets), Adam with cosine learning-rate decay from lr to lr/50 over
 * the call's epochs.  Checkpoints are flat binary. */
typedef struct ves_shiftnet ves_shiftnet;
enum { VES_SHIFTNET_LOSS_CHAMFER = 0, VES_SHIFTNET_LOSS_ROBUST = 1 };
typedef struct ves_shiftnet_config {
    int dim;       /* matrix order n, 1..64 */
    int n_params;  /* family parameters per matrix, 0..64 */
    int hidden;    /* units per hidden layer: multiple of 16, 16..256; default 256 */
    int layers;    /* hidden layers (tcgen05 BF16 GEMMs), 1..6; the output layer is FP32; default 3 */
    int fourier;   /* extra features per parameter p: sin and cos of (pi/2) k p, k = 1..fourier
                    * (n_params * fourier <= 64); default 0 */
    int loss;      /* VES_SHIFTNET_LOSS_CHAMFER (squared distances, default) or _ROBUST
                    * (sqrt(d^2 + delta^2) - delta per matched pair) */
    float delta;   /* robust loss scale in standardised units; default 0.01 */
    unsigned long long seed;  /* weight initialisation */
    int subdiag;   /* 1: also the 2-norms of the n - 1 subdiagonals of A as features; default 0 */
} ves_shiftnet_config;
void ves_shiftnet_default_config(ves_shiftnet_config *cfg);
int ves_shiftnet_create_config(ves_shiftnet **net, const ves_shiftnet_config *cfg);
/* the default configuration with the given order, parameter count, width and seed */
int ves_shiftnet_create(ves_shiftnet **net, int dim, int n_params, int hidden, unsigned long long seed);
void ves_shiftnet_destroy(ves_shiftnet *net);
int ves_shiftnet_train(ves_shiftnet *net, long long count, int thread_cnt, const double *params,
                       const double *rA, const double *iA, const double *rE, const double *iE,
                       int epochs, int batch, float lr, unsigned long long seed, float *loss_per_epoch, void *stream);
/* Number of parameters (floats): W and b of every layer, W row-major out x in. */
size_t ves_shiftnet_param_count(const ves_shiftnet *net);
/* The loss and its gradient over ONE batch of all `count` matrices (32 <= count
 * <= 65536, a multiple of thread_cnt) at the network's current weights and
 * standardisation, computed as a training step computes them (hidden layers:
 * tcgen05 BF16 GEMMs with FP32 accumulation; output layer: FP32).  grad
 * (device, ves_shiftnet_param_count floats) receives the gradients in
 * checkpoint order (W then b of layer 0, 1, ...); loss (device, one float) the
 * batch loss.  Synchronous.  For tests and tooling. */
int ves_shiftnet_gradient(const ves_shiftnet *net, long long count, int thread_cnt, const double *params,
                          const double *rA, const double *iA, const double *rE, const double *iE, float *grad,
                          float *loss, void *stream);
size_t ves_shiftnet_predict_workspace_size(const ves_shiftnet *net, long long count);
int ves_shiftnet_predict(const ves_shiftnet *net, long long count, int thread_cnt, const double *params,
                         const double *rA, const double *iA, double *rS, double *iS,
                         void *workspace, size_t workspace_bytes, void *stream);
int ves_shiftnet_save(const ves_shiftnet *net, const char *path);
int ves_shiftnet_load(ves_shiftnet **net, const char *path);

/* The learned-shift network's GEMM on the tcgen05 tensor cores: C = A * B
 * (+ bias) (GELU if act = 1), A row-major M x K BF16 (lda), Bt = B transposed,
 * row-major N x K BF16 (ldb); C (nullable) gets act(A*B + bias) as BF16 and Cf
 * (nullable) the pre-activation A*B + bias as FP32, both row-major M x N with
 * leading dimension ldc; K, lda, ldb multiples of 8 and
 * 16-byte aligned rows.  `err` (device int, nullable) is set to 1 if the
 * tensor-core pipeline did not complete.  No counterpart in the reference. */
int ves_gemm_bf16(int M, int N, int K, const void *A, int lda, const void *Bt, int ldb, const float *bias, int act,
                  void *C, float *Cf, int ldc, int *err, void *stream);

/* Roots of polynomials c_0 + c_1 x + ... + c_d x^d (d = degree), as eigenvalues
 * of their companion matrices (the reference's create_companion_matrices +
 * zlahqr kernel, Toolbox.hpp:607-643, :1894-1957), on the eigenvalues-only QR.
 * Coefficients: SoA vectors of length degree+1 per polynomial (rC, iC: element i
 * of polynomial m = b*thread_cnt + t at b*thread_cnt*(degree+1) + i*thread_cnt + t);
 * roots: SoA vectors of length degree.  A zero leading coefficient or non-finite
 * data gives NaN roots and VES_STATUS_NONFINITE.  workspace as ves_eigensolve. */
size_t ves_polyroots_workspace_size(int degree, int block_cnt, int thread_cnt);
int ves_polyroots(int degree, int block_cnt, int thread_cnt, const double *rC, const double *iC,
                  double *rR, double *iR, int *status, void *workspace, size_t workspace_bytes, void *stream);

/* Device transposes between the SoA planes and interleaved complex batches
 * (re, im pairs; matrix m at z + 2*m*dim*dim, row-major i.e. C/NumPy order if
 * row_major != 0, else column-major), and the same for length-dim vectors.
 * z must be 16-byte aligned.  Replace the host-side rearrangeMatrices /
 * arrangeMatricesAoS (utils.cpp:85-123) for interleaved complex data. */
int ves_soa_from_complex(int dim, int block_cnt, int thread_cnt, const void *z, int row_major,
                         double *re, double *im, void *stream);
int ves_complex_from_soa(int dim, int block_cnt, int thread_cnt, const double *re, const double *im,
                         int row_major, void *z, void *stream);
int ves_soa_vec_from_complex(int dim, int block_cnt, int thread_cnt, const void *z, double *re, double *im,
                             void *stream);
int ves_complex_from_soa_vec(int dim, int block_cnt, int thread_cnt, const double *re, const double *im,
                             void *z, void *stream);

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
/* The same for FP32 FMAs: the roofline denominator of the FP32 stages of the
 * FP32 + refinement form and of the learned-shift polish. */
int ves_fp32_fma_rate(double *flops_per_s, void *stream);

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
 * before any stream capture.  cudaDeviceReset() ends the context that holds
 * the array, and the address looked up before it is then stale: do not call
 * this entry point on a device after resetting it in the same process.
 * All calls on a device share the array, so calls
 * that overlap on the GPU race and must be serialised by the caller.
 * Asynchronous on `stream`. */
#define VES_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
#define VES_NOALLOC_MAX_DIM 64
int ves_eigensolve_noalloc(int dim, int block_cnt, int thread_cnt,
                           const double *rA, const double *iA, double *rE, double *iE, double *rV, double *iV,
                           int *status, void *stream);

/* One batch over several GPUs (no counterpart in the reference, which runs on
 * one device): the batch is split into `parts` contiguous ranges of whole SoA
 * blocks, sizes differing by at most one block; part `part` (0-based) owns
 * blocks [*first_block, *first_block + *n_blocks).  Whole blocks are
 * contiguous in every plane, so a part is the caller's arrays offset by
 * first_block * thread_cnt * dim * dim (matrices) or first_block * thread_cnt
 * * dim (vectors), solved by any entry point above with block_cnt = n_blocks
 * on that part's own GPU (one process or host thread per GPU; the parts share
 * nothing, so no collective is involved).  Host arithmetic only.  Returns
 * VES_ERR_ARG for block_cnt < 0, parts < 1 or part outside [0, parts). */
int ves_partition_blocks(int block_cnt, int parts, int part, int *first_block, int *n_blocks);

/* Index violations counted by the bounds-checked build of this library
 * (libves_bc.so, compiled with -DVES_BOUNDS_CHECK): every matrix and vector
 * element access of the numerical routines checks its indices, counts one
 * that is out of range and reads or writes the first element instead, so a
 * kernel never touches memory outside its operand.  *count = the number since
 * the last reset (reset != 0 clears the counters after reading; synchronous).
 * The normal build returns VES_ERR_UNSUPPORTED.  No counterpart in the
 * reference. */
int ves_bounds_violations(unsigned long long *count, int reset);

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
