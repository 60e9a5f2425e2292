// ves_extras.cu -- the entry points around the solver path:
//
//  * eigenvalues only (LAPACK zlahqr with wantT = wantZ = false; the
//    reference's unused zlahqr_ at Toolbox.hpp:1663-1890): zgehrd, then the QR
//    iteration on the active block only, no Q, no Schur vectors, no ztrevc.
//    About a third of the full solve's QR work, and the same eigenvalues bit
//    for bit (the active block sees the same arithmetic).
//  * roots of polynomials through their companion matrices (the reference's
//    create_companion_matrices + zlahqr kernel, Toolbox.hpp:607-643 and
//    :1894-1957), on the eigenvalues-only QR.
//  * device transposes between the SoA planes and interleaved complex AoS
//    batches (NumPy complex128 (N, n, n), C or Fortran order), replacing the
//    host-side rearrangeMatrices / arrangeMatricesAoS (utils.cpp:85-123).
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>

namespace ves {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ long long soa_off(long long m, long long len, int tc)
{
    return (m / tc) * (long long)tc * len + (m % tc);
}

// Eigenvalues only.  Workspace per warp: H (n*n) and tau (n), double2.
__global__ void __launch_bounds__(kThreads) eigvals_fp64_kernel(const Geom g, const double *rA, const double *iA,
                                                                double *rE, double *iE, int *status_out,
                                                                int *sweeps_out, void *ws, int max_its)
{
    const int n = g.n, tc = g.tc, lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    const long long nslots = (long long)gridDim.x * (kThreads / 32);
    const long long ngroups = (g.N + 31) / 32;
    double2 *base = reinterpret_cast<double2 *>(ws) + slot * ((long long)n * n + n) * 32 + lane;
    const MatIlv<double> H{base, n};
    const VecIlv<double> W{base + (long long)n * n * 32};
    for (long long gr = slot; gr < ngroups; gr += nslots) {
        const long long m = gr * 32 + lane;
        const bool valid = m < g.N;
        const long long mo = valid ? soa_off(m, (long long)n * n, tc) : 0;
        const long long vo = valid ? soa_off(m, n, tc) : 0;
        int status = 0, sweeps = 0;
        if (valid) {
            const MatSoA<double> A{const_cast<double *>(rA) + mo, const_cast<double *>(iA) + mo, tc, n};
            bool bad = false;
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) {
                    const cx<double> v = A.ld(i, j);
                    bad |= nonfinite(v.r) | nonfinite(v.i);
                    H.st(i, j, v);
                }
            if (bad) status |= ST_NONFINITE;
            zgehrd_lane<double>(n, H, W);
            clear_below_subdiag_lane<double>(n, H);
        }
        zlahqr_warp<double, false>(n, H, H, valid && !(status & ST_NONFINITE), max_its, sweeps, status);
        if (valid) {
            const VecSoA<double> E{rE + vo, iE + vo, tc};
            for (int k = 1; k <= n; ++k) E.st(k, H.ld(k, k));
            if (status_out) status_out[m] = status;
            if (sweeps_out) sweeps_out[m] = sweeps;
        }
    }
}

// Roots of sum_{i=0..n} c_i x^i: the companion matrix with ones on the
// subdiagonal and -c_{i-1}/c_n in the last column (create_companion_matrices,
// Toolbox.hpp:607-643, normalising by the leading coefficient with the same
// Smith division), already upper Hessenberg, then the eigenvalues-only QR.
// Coefficients are SoA vectors of length n+1, roots SoA vectors of length n.
__global__ void __launch_bounds__(kThreads) polyroots_kernel(const Geom g, const double *rC, const double *iC,
                                                             double *rR, double *iR, int *status_out, void *ws,
                                                             int max_its)
{
    const int n = g.n, tc = g.tc, lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    const long long nslots = (long long)gridDim.x * (kThreads / 32);
    const long long ngroups = (g.N + 31) / 32;
    double2 *base = reinterpret_cast<double2 *>(ws) + slot * ((long long)n * n + n) * 32 + lane;
    const MatIlv<double> H{base, n};
    for (long long gr = slot; gr < ngroups; gr += nslots) {
        const long long m = gr * 32 + lane;
        const bool valid = m < g.N;
        int status = 0, sweeps = 0;
        if (valid) {
            const long long co = soa_off(m, n + 1, tc);
            const VecSoA<double> C{const_cast<double *>(rC) + co, const_cast<double *>(iC) + co, tc};
            const cx<double> lead = C.ld(n + 1);
            bool bad = nonfinite(lead.r) | nonfinite(lead.i) | (lead.r == 0.0 && lead.i == 0.0);
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) H.st(i, j, mk(i == j + 1 ? 1.0 : 0.0, 0.0));
            for (int i = 1; i <= n; ++i) {
                const cx<double> c = C.ld(i);
                bad |= nonfinite(c.r) | nonfinite(c.i);
                const cx<double> q = cdiv(c, lead);
                H.st(i, n, mk(-q.r, -q.i));
            }
            if (bad) status |= ST_NONFINITE;
        }
        zlahqr_warp<double, false>(n, H, H, valid && !(status & ST_NONFINITE), max_its, sweeps, status);
        if (valid) {
            const long long ro = soa_off(m, n, tc);
            const VecSoA<double> Rt{rR + ro, iR + ro, tc};
            for (int k = 1; k <= n; ++k) Rt.st(k, status & ST_NONFINITE ? mk(nan(""), nan("")) : H.ld(k, k));
            if (status_out) status_out[m] = status;
        }
    }
}

// Transposes.  Z is interleaved complex, matrix m occupying len consecutive
// complex numbers; element e' of Z's matrix maps to element e of the SoA
// matrix (e = e' for column-major data and vectors, the transpose index for
// row-major n x n data).  Tiles of 32 matrices x 32 elements through shared
// memory: reads of Z are contiguous in e', writes of the planes contiguous in
// the matrix index (t).
__device__ __forceinline__ long long perm_index(long long ep, int n, bool row_major)
{
    if (!row_major) return ep;
    const long long i = ep / n, j = ep % n;  // row-major (i, j)
    return i + j * n;                        // column-major index
}

__global__ void aos_to_soa_kernel(const double2 *Z, double *re, double *im, long long N, int n, long long len, int tc,
                                  bool row_major)
{
    __shared__ double2 tile[32][33];
    const long long m0 = (long long)blockIdx.x * 32, e0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const long long m = m0 + r, ep = e0 + tx;
        if (m < N && ep < len) tile[r][tx] = Z[m * len + ep];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const long long ep = e0 + r, m = m0 + tx;
        if (m < N && ep < len) {
            const long long e = perm_index(ep, n, row_major);
            const long long o = (m / tc) * (long long)tc * len + e * tc + (m % tc);
            const double2 v = tile[tx][r];
            re[o] = v.x;
            im[o] = v.y;
        }
    }
}

__global__ void soa_to_aos_kernel(const double *re, const double *im, double2 *Z, long long N, int n, long long len,
                                  int tc, bool row_major)
{
    __shared__ double2 tile[32][33];
    const long long m0 = (long long)blockIdx.x * 32, e0 = (long long)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        const long long ep = e0 + r, m = m0 + tx;
        if (m < N && ep < len) {
            const long long e = perm_index(ep, n, row_major);
            const long long o = (m / tc) * (long long)tc * len + e * tc + (m % tc);
            tile[tx][r] = make_double2(re[o], im[o]);
        }
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const long long m = m0 + r, ep = e0 + tx;
        if (m < N && ep < len) Z[m * len + ep] = tile[r][tx];
    }
}

// Persistent grid of the eigenvalues-only and polynomial-root kernels: blocks
// of 4 warps per SM, default by order as measured on GB300 (eigenvalues only,
// 2 -> 3 -> 4 -> 5 blocks): n=16 3.07 3.14 3.08 3.06 M/s, n=32 0.473 0.519
// 0.542 0.501 M/s.  The workspace size and the launch use the same count.
long long persistent_blocks(int n, long long N, int blocks_per_sm)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    const long long groups = (N + 31) / 32;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : (n <= 20 ? 3 : 4);
    return std::max<long long>(1, std::min<long long>((groups + 3) / 4, (long long)sms * bps));
}

}  // namespace

size_t eigvals_workspace_bytes(int n, long long N, int blocks_per_sm)
{
    return (size_t)persistent_blocks(n, N, blocks_per_sm) * 4 * ((size_t)n * n + n) * 32 * sizeof(double2);
}

cudaError_t launch_eigvals(Geom g, const double *rA, const double *iA, double *rE, double *iE, int *status,
                           int *sweeps, void *ws, int max_its, int blocks_per_sm, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    eigvals_fp64_kernel<<<(unsigned)persistent_blocks(g.n, g.N, blocks_per_sm), kThreads, 0, st>>>(g, rA, iA, rE, iE,
                                                                                              status, sweeps, ws,
                                                                               max_its);
    return cudaGetLastError();
}

cudaError_t launch_polyroots(Geom g, const double *rC, const double *iC, double *rR, double *iR, int *status,
                             void *ws, int max_its, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    polyroots_kernel<<<(unsigned)persistent_blocks(g.n, g.N, 0), kThreads, 0, st>>>(g, rC, iC, rR, iR, status, ws,
                                                                                 max_its);
    return cudaGetLastError();
}

cudaError_t launch_transpose(bool to_soa, const double *src_re, const double *src_im, double *dst_re, double *dst_im,
                             const double *z_in, double *z_out, long long N, int n, long long len, int tc,
                             bool row_major, cudaStream_t st)
{
    if (N <= 0 || len <= 0) return cudaSuccess;
    const dim3 block(32, 8);
    const long long gx = (N + 31) / 32, gy = (len + 31) / 32;  // matrix tiles on x (2^31-1), element tiles on y
    if (gx > 0x7fffffffLL || gy > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)gx, (unsigned)gy);
    if (to_soa)
        aos_to_soa_kernel<<<grid, block, 0, st>>>(reinterpret_cast<const double2 *>(z_in), dst_re, dst_im, N, n, len,
                                                 tc, row_major);
    else
        soa_to_aos_kernel<<<grid, block, 0, st>>>(src_re, src_im, reinterpret_cast<double2 *>(z_out), N, n, len, tc,
                                                 row_major);
    return cudaGetLastError();
}

void load_extras_kernels()
{
    load_kernel(eigvals_fp64_kernel);
    load_kernel(polyroots_kernel);
    load_kernel(aos_to_soa_kernel);
    load_kernel(soa_to_aos_kernel);
}

}  // namespace ves
