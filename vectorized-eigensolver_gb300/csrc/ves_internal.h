// ves_internal.h -- launchers shared by the C-ABI layer (ves_api.cu) and the
// kernels (ves_kernels.cu).  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstddef>
#include <cstdlib>

namespace ves {

// An NVTX range for the lifetime of the object: the host-side stages of the
// entry points (copies, launches) show up named in Nsight Systems.  NVTX is
// header-only and costs a pointer test when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Batch geometry of the reference's SoA layout: N = block_cnt * thread_cnt
// matrices of order n, interleave stride tc = thread_cnt.
struct Geom {
    int n;
    long long N;
    int tc;
};

struct FusedArgs {
    Geom g;
    const double *rA, *iA;  // input (read only)
    double *rE, *iE;        // eigenvalues, SoA vector layout
    double *rV, *iV;        // eigenvectors, SoA matrix layout
    double *rT, *iT;        // optional Schur form T (may alias rA/iA)
    int *status;            // optional, one per matrix (plain index order)
    int *sweeps;            // optional, QR sweeps per matrix
    void *ws;               // workspace
    int max_its;
    int vnorm;
    // optional index list: solve only matrices list[0 .. *list_count) (the
    // mixed-precision form's fallback pass); status gets ST_REFINE_FALLBACK.
    // The lane kernel takes entries from list_split on, fp64_warp_kernel the
    // ones before it (launch_fp64_list sets it).
    const int *list;
    const int *list_count;
    long long list_split;
    // optional predicted eigenvalues (SoA vectors, n per matrix) used as the
    // first `shift_sweeps` QR shifts of every eigenvalue; `fallbacks` (nullable)
    // counts per matrix the eigenvalues that still needed Wilkinson's shift
    const double *rS, *iS;
    int shift_sweeps;
    float shift_gate;  // predictions used only while |H(I,I-1)| > shift_gate * ||A||_F / sqrt(n)
    int shift_polish;  // Aberth steps on det(H - sI) per prediction (FP32) before the QR; 0 = none
    int shift_newton64;  // then this many FP64 Newton steps per prediction on the solve's own H
    int *fallbacks;
    int blocks_per_sm;  // persistent grid: blocks (4 warps) per SM; 0 = default
};

struct MixedArgs {
    Geom g;
    const double *rA, *iA;
    double *rE, *iE;
    double *rV, *iV;
    int *status;
    int *sweeps;
    void *ws;
    int max_its;
    int vnorm;
    int max_steps;  // Newton corrections per eigenpair
    double tol;     // ||r|| <= tol ||A||_F ||v||
    int *fb_list;   // matrices handed to the FP64 solver
    int *fb_count;
    int blocks_per_sm;  // FP32 Schur kernel grid: blocks per SM; 0 = default
    // matrices [m_begin, m_end) of the batch (a multiple of 32 where a chunk
    // ends inside the batch); launch_mixed sets the whole batch when m_end == 0
    long long m_begin, m_end;
    unsigned long long *work;  // optional work counters (WORK_*)
    int ff_steps;              // refinement steps whose residual is float-float (1 or 2)
};

size_t mixed_workspace_bytes(int n, long long N, int blocks_per_sm, int *out_blocks, int *out_threads);
cudaError_t launch_mixed(const MixedArgs &a, cudaStream_t st);
// The same work with the batch cut into chunks: the FP32 Schur stage of a
// chunk runs on s_schur while the previous chunk's FP64 refinement runs on
// s_refine (the two kernels are bound by different units: latency of the FP32
// sweeps, the FP64 pipe), forked from and joined back into `st`.
cudaError_t launch_mixed_overlap(const MixedArgs &a, cudaStream_t st, cudaStream_t s_schur, cudaStream_t s_refine);

// Fused zgehrd -> zunghr -> zlahqr -> ztrevc, FP64.
// blocks_per_sm = 0 takes the library default (VES_FUSED_BLOCKS_PER_SM, else 4; 3 for 21 <= n <= 28).
// learned = the shift-seeded kernel, whose slots also hold an FP32 copy of H
// and the n predictions.
size_t fused_workspace_bytes(int n, long long N, int blocks_per_sm, int *out_blocks, int *out_threads,
                             bool learned = false);
cudaError_t launch_fused_fp64(const FusedArgs &a, cudaStream_t st);
// The FP64 solve of the matrices on a.list: the first entries (one per warp
// slot of the GPU) by fp64_warp_kernel (one matrix per warp, n <= 64), the
// rest by the lane kernel; the same results bit for bit either way.
cudaError_t launch_fp64_list(FusedArgs a, cudaStream_t st);

// Stage kernels, in place on the SoA layout (reference call_* semantics).
cudaError_t launch_zgehrd(Geom g, double *rA, double *iA, double *rtau, double *itau, cudaStream_t st);
cudaError_t launch_zunghr(Geom g, double *rA, double *iA, const double *rtau, const double *itau, cudaStream_t st);
cudaError_t launch_hessenberg(Geom g, double *rA, double *iA, double *rQ, double *iQ, double *rtau, double *itau,
                              cudaStream_t st);
cudaError_t launch_zlahqr(Geom g, double *rE, double *iE, double *rH, double *iH, double *rZ, double *iZ,
                          int *status, int max_its, cudaStream_t st);
cudaError_t launch_ztrevc(Geom g, double *rT, double *iT, double *rR, double *iR, double *rwork, double *iwork,
                          cudaStream_t st);
cudaError_t launch_zgemv(Geom g, bool herm, const double *rA, const double *iA, const double *rx, const double *ix,
                         double rbeta, double ibeta, double *ry, double *iy, cudaStream_t st);
cudaError_t launch_backsubs(Geom g, const double *rT, const double *iT, double *rx, double *ix, cudaStream_t st);

// The FP64 fused kernel on a caller-chosen grid of `blocks` x 4 warps; the
// workspace must hold blocks * 4 warp slots.
cudaError_t launch_fused_fp64_blocks(const FusedArgs &a, int blocks, cudaStream_t st);

// Learned-shift polish pre-pass (n <= 32): predictions (rS, iS) refined by
// Aberth steps on the FP32 Hessenberg form, written to (rP, iP); NaN = dropped.
cudaError_t launch_polish32(Geom g, const double *rA, const double *iA, const double *rS, const double *iS,
                            double *rP, double *iP, int steps, unsigned long long *work, cudaStream_t st);

// Eigenvalues only (no Q, no Schur vectors), companion-matrix roots, and the
// SoA <-> interleaved-complex transposes.
size_t eigvals_workspace_bytes(int n, long long N, int blocks_per_sm);
cudaError_t launch_eigvals(Geom g, const double *rA, const double *iA, double *rE, double *iE, int *status,
                           int *sweeps, void *ws, int max_its, int blocks_per_sm, cudaStream_t st);
cudaError_t launch_polyroots(Geom g, const double *rC, const double *iC, double *rR, double *iR, int *status,
                             void *ws, int max_its, cudaStream_t st);
cudaError_t launch_transpose(bool to_soa, const double *src_re, const double *src_im, double *dst_re, double *dst_im,
                             const double *z_in, double *z_out, long long N, int n, long long len, int tc,
                             bool row_major, cudaStream_t st);

// Mixed-size (packed) batches: binned by order, one persistent solve.
size_t varsize_workspace_bytes(long long count, int max_dim, int blocks_per_sm);
cudaError_t launch_varsize(long long count, int max_dim, const int *dims, const double *rA, const double *iA,
                           double *rE, double *iE, double *rV, double *iV, int *status, int *sweeps, void *ws,
                           int max_its, int vnorm, int blocks_per_sm, int order, cudaStream_t st);

// BF16 GEMM on tcgen05 (C = A * B, Bt = B transposed, both K-major), bias and
// GELU (act = 1) fused; C (BF16) and/or Cf (FP32) written.
cudaError_t launch_gemm_bf16(int M, int N, int K, const void *A, int lda, const void *Bt, int ldb, const float *bias,
                             int act, void *C, float *Cf, int ldc, int *err, cudaStream_t st);

// The drop-in bodies (ves_api.cu) behind the C names of ves.h and the C++
// names of the reference host API (ves_dropin_cxx.cpp).
void dropin_eigensolver(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rE, double *iE, double *rV, double *iV);
void dropin_hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ);
void dropin_call_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau);
void dropin_call_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau);
void dropin_call_zlahqr_new(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM, double *rS, double *iS);
void dropin_call_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR);
void dropin_call_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, double *rM, double *iM, double *rx, double *ix, double *ry, double *iy, double rbeta, double ibeta);
void dropin_call_backsubstitution(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rb, double *ib);
void dropin_repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out);
void dropin_repVectorSoA(int dim, int block_cnt, int thread_cnt, double *vec, double *out);
void dropin_rearrangeMatrices(int dim, int block_cnt, int thread_cnt, double *in, double *out);
void dropin_arrangeMatricesAoS(int dim, int block_cnt, int thread_cnt, double *in, double *out);

// Record the calling thread's message for ves_last_error().
void set_error_message(const char *msg);

// Measured FP64 / FP32 FMA throughput of this GPU (2 flops per FMA).
cudaError_t fp64_fma_rate(double *flops_per_s, cudaStream_t st);
cudaError_t fp32_fma_rate(double *flops_per_s, cudaStream_t st);

// Work counters of ves_options.work_counts (device, accumulated with atomics).
enum { WORK_RES64 = 0, WORK_CORR32 = 1, WORK_RESFF = 2, WORK_POLISH = 3 };

// CUDA loads a kernel lazily, at its first launch, by default, so where a
// kernel's code lands depends on what the process loaded before.  Kernels that
// run at the same time on one SM (the FP32+refine form's Schur and refinement
// stages) measured up to 9% slower when loaded late in a long process than
// when loaded early.  load_kernels() loads every kernel of the library, in
// one fixed order, the first time it is called for the current device; each
// file's list below is in that order.
void load_kernels();
void load_mixed_kernels();
void load_fused_kernels();
void load_varsize_kernels();
void load_extras_kernels();
void load_shiftnet_kernels();
template <typename K> inline void load_kernel(K *k)
{
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, k);  // forces the load; errors are cleared by load_kernels()
}

}  // namespace ves
