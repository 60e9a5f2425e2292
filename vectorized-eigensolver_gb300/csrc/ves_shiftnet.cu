// ves_shiftnet.cu -- the learned-shift network: a small BF16 MLP whose
// forward GEMMs run on the tcgen05 tensor cores (ves_tc.cuh), trained with
// hand-written kernels, that maps cheap per-matrix features to estimates of
// the eigenvalues; the solver uses them as first QR shifts.
//
//   features  f = [family parameters (P), Re diag A (n), Im diag A (n)],
//             standardised with the training set's mean / std, zero-padded to
//             Kin (a multiple of 32), BF16
//   network   Kin -> H -> H -> H -> Nout, GELU after the hidden layers,
//             BF16 weights and activations, FP32 accumulation (in TMEM)
//   targets   the eigenvalues the plain solver computed, as [Re (n), Im (n)]
//             (sorted by real part, which only seeds the output order), shifted
//             by the mean real / imaginary part and divided by one common
//             standard deviation, zero-padded to Nout (multiple of 16)
//   training  the loss is the symmetric Chamfer distance between the predicted
//             set and the eigenvalue set, (1/2n) [sum_i min_j |y_i - l_j|^2 +
//             sum_j min_i |y_i - l_j|^2]: an eigenvalue set has no canonical
//             order that is continuous in the matrix (any order by real part
//             jumps where two real parts cross), and the solver only needs
//             every eigenvalue to have a prediction nearby.  Backward pass and
//             Adam (cosine learning-rate decay to 1/50) in FP32 on CUDA cores
//             (the batch GEMMs of the backward pass are a few MFLOP)
//   inference one forward pass per matrix, denormalised to n complex shifts
#include "ves.h"
#include "ves_device.cuh"
#include "ves_internal.h"
#include "ves_tc.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

namespace ves {

namespace {

template <int NT>
cudaError_t launch_persistent(int M, int N, int K, const __nv_bfloat16 *a, int lda, const __nv_bfloat16 *b, int ldb,
                              const float *bias, int act, __nv_bfloat16 *c, float *cf, int ldc, int *err,
                              cudaStream_t st)
{
    const int smem = (tc::kM + NT) * K * 2;
    // per call (per device, thread safe; microseconds next to the kernel)
    cudaError_t e = cudaFuncSetAttribute(tc::gemm_bf16_persistent_kernel<NT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (tc::kM + NT) * 256 * 2);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    constexpr int kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
    const int per_sm = std::max(1, std::min(512 / kCols, (220 * 1024) / smem));
    const int mtiles = (M + tc::kM - 1) / tc::kM;
    const unsigned gx = (unsigned)std::max(1, std::min(mtiles, std::max(sms, 1) * per_sm));
    tc::gemm_bf16_persistent_kernel<NT><<<dim3(gx, (N + NT - 1) / NT), 128, smem, st>>>(a, lda, b, ldb, M, N, K, bias,
                                                                                      act, c, cf, ldc, err);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// Tensor map of a row-major rows x K BF16 matrix (leading dimension ld) read
// in boxes of 8 elements (16 bytes) x box_rows; false if the driver rejects it
// (base not 16-byte aligned, ld * 2 not a multiple of 16, ...).
bool bf16_box_map(CUtensorMap *map, const void *base, int rows, int K, int ld, int box_rows)
{
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || ((uintptr_t)base & 15) != 0 || (ld % 8) != 0 || K < 8 || rows < 1 || box_rows > 256) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The persistent GEMM with TMA operand loads; cudaErrorNotSupported when a
// tensor map cannot be made for these operands (the caller then uses cp.async).
template <int NT>
cudaError_t launch_persistent_tma(int M, int N, int K, const __nv_bfloat16 *a, int lda, const __nv_bfloat16 *b,
                                  int ldb, const float *bias, int act, __nv_bfloat16 *c, float *cf, int ldc, int *err,
                                  cudaStream_t st)
{
    CUtensorMap ta, tb;
    if (!bf16_box_map(&ta, a, M, K, lda, tc::kM) || !bf16_box_map(&tb, b, N, K, ldb, NT)) return cudaErrorNotSupported;
    const int smem = (tc::kM + NT) * K * 2;
    cudaError_t e = cudaFuncSetAttribute(tc::gemm_bf16_tma_kernel<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (tc::kM + NT) * 256 * 2);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    constexpr int kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
    const int per_sm = std::max(1, std::min(512 / kCols, (220 * 1024) / smem));
    const int mtiles = (M + tc::kM - 1) / tc::kM;
    const unsigned gx = (unsigned)std::max(1, std::min(mtiles, std::max(sms, 1) * per_sm));
    tc::gemm_bf16_tma_kernel<NT><<<dim3(gx, (N + NT - 1) / NT), 128, smem, st>>>(ta, tb, M, N, K, bias, act, c, cf,
                                                                               ldc, err);
    return cudaGetLastError();
}

// The persistent GEMM: TMA operand loads for more than 16 row tiles, cp.async
// for fewer (a training batch) or where no tensor map can be made.  GB300,
// 256 x 256 weights, GELU: M = 1,048,576 0.835 ms with TMA against 1.043 ms
// (165 against 132 TFLOP/s), M = 262,144 0.226 against 0.282 ms; M = 1,024
// about the same either way.  VES_GEMM_TMA=1 / 0 forces TMA / cp.async.
template <int NT>
cudaError_t launch_persistent_any(int M, int N, int K, const __nv_bfloat16 *a, int lda, const __nv_bfloat16 *b,
                                  int ldb, const float *bias, int act, __nv_bfloat16 *c, float *cf, int ldc, int *err,
                                  cudaStream_t st)
{
    const char *e = getenv("VES_GEMM_TMA");
    const bool tma = e && (e[0] == '0' || e[0] == '1') ? e[0] == '1' : (M + tc::kM - 1) / tc::kM > 16;
    if (tma) {
        const cudaError_t r = launch_persistent_tma<NT>(M, N, K, a, lda, b, ldb, bias, act, c, cf, ldc, err, st);
        if (r != cudaErrorNotSupported) return r;
    }
    return launch_persistent<NT>(M, N, K, a, lda, b, ldb, bias, act, c, cf, ldc, err, st);
}

}  // namespace

// The persistent kernel when K <= 256 and the shapes allow 16-byte vector
// stores; the K-chunked kernel otherwise.
cudaError_t launch_gemm_bf16(int M, int N, int K, const void *A, int lda, const void *Bt, int ldb, const float *bias,
                             int act, void *C, float *Cf, int ldc, int *err, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
    const auto *a = static_cast<const __nv_bfloat16 *>(A);
    const auto *b = static_cast<const __nv_bfloat16 *>(Bt);
    auto *c = static_cast<__nv_bfloat16 *>(C);
    const bool vec_ok = (N % 16) == 0 && (ldc % 8) == 0 && ((uintptr_t)C & 15) == 0 && ((uintptr_t)Cf & 15) == 0;
    if (K % 16 == 0 && K <= 256 && vec_ok) {
        // few row tiles (a training batch): narrower column tiles give more CTAs
        // (M = 1,024, N = 256: 32 instead of 8)
        if ((M + tc::kM - 1) / tc::kM <= 16 && N > 64 && N % 64 == 0)
            return launch_persistent_any<64>(M, N, K, a, lda, b, ldb, bias, act, c, Cf, ldc, err, st);
        if (N > 128) return launch_persistent_any<256>(M, N, K, a, lda, b, ldb, bias, act, c, Cf, ldc, err, st);
        if (N > 64) return launch_persistent_any<128>(M, N, K, a, lda, b, ldb, bias, act, c, Cf, ldc, err, st);
        return launch_persistent_any<64>(M, N, K, a, lda, b, ldb, bias, act, c, Cf, ldc, err, st);
    }
    const unsigned gx = (unsigned)((M + tc::kM - 1) / tc::kM);
    if (N > 64) {
        tc::gemm_bf16_kernel<256><<<dim3(gx, (N + 255) / 256), 128, 0, st>>>(a, lda, b, ldb, M, N, K, bias, act, c,
                                                                             Cf, ldc, err);
    } else {
        tc::gemm_bf16_kernel<64><<<dim3(gx, (N + 63) / 64), 128, 0, st>>>(a, lda, b, ldb, M, N, K, bias, act, c, Cf,
                                                                         ldc, err);
    }
    return cudaGetLastError();
}

// Split-K product for the weight gradients (K = the batch): S partial FP32
// products part[z] = A[:, Kz] * B[Kz, :] (z-th K range), M x N each with
// leading dimension ldc, one after the other; the caller sums them.
cudaError_t launch_gemm_bf16_splitk(int M, int N, int K, const void *A, int lda, const void *Bt, int ldb, float *part,
                                    int ldc, int S, int *err, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || K <= 0 || S < 1) return cudaSuccess;
    const auto *a = static_cast<const __nv_bfloat16 *>(A);
    const auto *b = static_cast<const __nv_bfloat16 *>(Bt);
    const unsigned gx = (unsigned)((M + tc::kM - 1) / tc::kM);
    const long long zs = (long long)M * ldc;
    if (N > 64)
        tc::gemm_bf16_kernel<256><<<dim3(gx, (N + 255) / 256, S), 128, 0, st>>>(a, lda, b, ldb, M, N, K, nullptr, 0,
                                                                                nullptr, part, ldc, err, zs);
    else
        tc::gemm_bf16_kernel<64><<<dim3(gx, (N + 63) / 64, S), 128, 0, st>>>(a, lda, b, ldb, M, N, K, nullptr, 0,
                                                                              nullptr, part, ldc, err, zs);
    return cudaGetLastError();
}

namespace {

constexpr int kMaxDimNet = 64;
constexpr int kMaxLayers = 6;  // hidden layers
typedef __nv_bfloat16 bf16;

__device__ __forceinline__ long long soa_off_s(long long m, long long len, int tc)
{
    return (m / tc) * (long long)tc * len + (m % tc);
}

constexpr int kMaxFourier = 64;  // n_params * fourier

// feature c (unnormalised) of matrix m; the row is [parameters (P), sin / cos
// ((pi/2) k p) for k = 1..F per parameter, Re diag A (n), Im diag A (n), and
// with S = 1 the 2-norms of the n - 1 subdiagonals of A (how far A is from
// upper triangular, diagonal by diagonal)]
__device__ __forceinline__ float one_feature(long long m, int c, int n, int P, int F, int tc, const double *params,
                                             const double *rA, const double *iA)
{
    if (c < P) return params ? (float)params[m * P + c] : 0.f;
    const int o = P + 2 * P * F;
    if (c < o) {
        const int idx = c - P, q = idx / (2 * F), k = (idx % (2 * F)) / 2 + 1;
        const float x = params ? (float)params[m * P + q] : 0.f;
        float sn, cs;
        sincospif(0.5f * (float)k * x, &sn, &cs);
        return (idx & 1) ? cs : sn;
    }
    const long long mo = soa_off_s(m, (long long)n * n, tc);
    if (c < o + 2 * n) {
        const int i = (c - o) % n;
        const long long k = mo + (long long)(i + i * n) * tc;
        return c < o + n ? (float)rA[k] : (float)iA[k];
    }
    const int d = c - o - 2 * n + 1;  // subdiagonal d: elements (i + d, i)
    double s2 = 0.0;
    for (int i = 0; i + d < n; ++i) {
        const long long k = mo + (long long)(i + d + i * n) * tc;
        s2 = fma(rA[k], rA[k], fma(iA[k], iA[k], s2));
    }
    return (float)sqrt(s2);
}

// features -> standardised BF16 rows [count x kin_pad]: one warp per row, the
// lanes take the row's features c = lane, lane + 32, ... (coalesced stores)
__global__ void features_kernel(long long count, int n, int P, int F, int S, int tc, const double *params, const double *rA,
                                const double *iA, const float *mean, const float *stdv, int kin, int kin_pad, bf16 *X,
                                const int *rows)
{
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= count) return;
    const long long m = rows ? rows[r] : r;
    for (int c = lane; c < kin_pad; c += 32) {
        float v = 0.f;
        if (c < kin) {
            const float f = one_feature(m, c, n, P, F, tc, params, rA, iA);
            v = mean ? (f - mean[c]) / stdv[c] : f;
        }
        X[r * kin_pad + c] = __float2bfloat16(v);
    }
}

// standardised targets [count x nout_pad]: the eigenvalues in canonical order
// (real parts ascending, ties in index order), real parts then imaginary
// parts.  One warp per row; lane i holds eigenvalues i and i + 32 and finds
// each one's place in that order by counting
__global__ void targets_kernel(long long count, int n, int tc, const double *rE, const double *iE, const float *mean,
                               const float *stdv, int nout_pad, float *T, const int *rows)
{
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= count) return;
    const long long m = rows ? rows[r] : r;
    const long long vo = soa_off_s(m, n, tc);
    float re[2], im[2];
    int rank[2] = {0, 0};
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        re[h] = i < n ? (float)rE[vo + (long long)i * tc] : 0.f;
        im[h] = i < n ? (float)iE[vo + (long long)i * tc] : 0.f;
    }
    for (int j = 0; j < n; ++j) {
        const float v0 = __shfl_sync(FULL, re[0], j & 31), v1 = __shfl_sync(FULL, re[1], j & 31);
        const float rj = j < 32 ? v0 : v1;
        for (int h = 0; h < 2; ++h) rank[h] += (rj < re[h]) || (rj == re[h] && j < lane + 32 * h);
    }
    float *t = T + r * nout_pad;
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        if (i >= n) continue;
        const int c = rank[h];
        t[c] = mean ? (re[h] - mean[c]) / stdv[c] : re[h];
        t[n + c] = mean ? (im[h] - mean[n + c]) / stdv[n + c] : im[h];
    }
    for (int c = 2 * n + lane; c < nout_pad; c += 32) t[c] = 0.f;
}

// column mean and standard deviation of the BF16 feature table, one thread per column
__global__ void colstats_bf16_kernel(long long count, int cols, int ld, const bf16 *X, float *mean, float *stdv)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    double s = 0.0, s2 = 0.0;
    for (long long r = 0; r < count; ++r) {
        const double v = __bfloat162float(X[r * ld + c]);
        s += v;
        s2 += v * v;
    }
    const double mu = s / (double)count;
    const double var = s2 / (double)count - mu * mu;
    mean[c] = (float)mu;
    stdv[c] = (float)(var > 1e-12 ? sqrt(var) : 1.0);
}

// Target normalisation: mean of the real parts, mean of the imaginary parts,
// one common standard deviation (distances stay isotropic in the complex
// plane).  One block; T holds raw targets [count x ld].
__global__ void target_stats_kernel(long long count, int n, int ld, int nout_pad, const float *T, float *mean,
                                    float *stdv)
{
    __shared__ double red[4][256];
    double sr = 0.0, si = 0.0, sr2 = 0.0, si2 = 0.0;
    const long long total = count * n;
    for (long long e = threadIdx.x; e < total; e += blockDim.x) {
        const long long r = e / n;
        const int i = (int)(e % n);
        const double vr = T[r * ld + i], vi = T[r * ld + n + i];
        sr += vr;
        sr2 += vr * vr;
        si += vi;
        si2 += vi * vi;
    }
    red[0][threadIdx.x] = sr;
    red[1][threadIdx.x] = si;
    red[2][threadIdx.x] = sr2;
    red[3][threadIdx.x] = si2;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double c = (double)total;
        const double mr = red[0][0] / c, mi = red[1][0] / c;
        const double var = 0.5 * ((red[2][0] / c - mr * mr) + (red[3][0] / c - mi * mi));
        const float sd = (float)(var > 1e-24 ? sqrt(var) : 1.0);
        for (int k = 0; k < nout_pad; ++k) {
            mean[k] = k < n ? (float)mr : (k < 2 * n ? (float)mi : 0.f);
            stdv[k] = k < 2 * n ? sd : 1.f;
        }
    }
}

// ---- training kernels (FP32, CUDA cores) -----------------------------------
// Symmetric Chamfer loss between the predicted set y and the eigenvalue set t
// of each sample (rows of Y, T: [Re (n), Im (n), padding]) and its gradient
// dY; one thread per sample.  Every prediction is matched to its nearest
// eigenvalue and every eigenvalue to its nearest prediction; a matched pair at
// squared distance d2 costs d2 (kind 0) or sqrt(d2 + delta^2) - delta (kind 1,
// robust: the rare far pairs near colliding eigenvalues do not dominate).
// loss += batch mean of (1/2n) sum of the costs.
__device__ __forceinline__ float pair_cost(int kind, float d2, float delta, float &gscale)
{
    if (kind == 0) { gscale = 2.f; return d2; }
    const float r = sqrtf(d2 + delta * delta);
    gscale = 1.f / r;
    return r - delta;
}

__global__ void chamfer_kernel(int B, int n, int ld, const float *Y, const float *T, float *dY, float *loss, int kind,
                               float delta)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (b < B) {
        float yr[kMaxDimNet], yi[kMaxDimNet], tr[kMaxDimNet], ti[kMaxDimNet], gr[kMaxDimNet], gi[kMaxDimNet];
        const float *y = Y + (long long)b * ld, *t = T + (long long)b * ld;
        for (int i = 0; i < n; ++i) {
            yr[i] = y[i]; yi[i] = y[n + i];
            tr[i] = t[i]; ti[i] = t[n + i];
            gr[i] = 0.f; gi[i] = 0.f;
        }
        const float w = 1.f / (2.f * (float)n * (float)B);
        for (int i = 0; i < n; ++i) {  // each prediction to its nearest eigenvalue
            float best = 0.f;
            int bj = -1;
            for (int j = 0; j < n; ++j) {
                const float dr = yr[i] - tr[j], di = yi[i] - ti[j];
                const float d = dr * dr + di * di;
                if (bj < 0 || d < best) { best = d; bj = j; }
            }
            float gs;
            l += pair_cost(kind, best, delta, gs);
            gr[i] += gs * w * (yr[i] - tr[bj]);
            gi[i] += gs * w * (yi[i] - ti[bj]);
        }
        for (int j = 0; j < n; ++j) {  // each eigenvalue to its nearest prediction
            float best = 0.f;
            int bi = -1;
            for (int i = 0; i < n; ++i) {
                const float dr = yr[i] - tr[j], di = yi[i] - ti[j];
                const float d = dr * dr + di * di;
                if (bi < 0 || d < best) { best = d; bi = i; }
            }
            float gs;
            l += pair_cost(kind, best, delta, gs);
            gr[bi] += gs * w * (yr[bi] - tr[j]);
            gi[bi] += gs * w * (yi[bi] - ti[j]);
        }
        float *g = dY + (long long)b * ld;
        for (int i = 0; i < n; ++i) { g[i] = gr[i]; g[n + i] = gi[i]; }
        for (int c = 2 * n; c < ld; ++c) g[c] = 0.f;
        l *= w;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(FULL, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    const float u = k0 * (x + k1 * x * x * x);
    const float th = tanhf(u);
    return 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * k0 * (1.f + 3.f * k1 * x * x);
}

// dZ = dH * GELU'(Z)
__global__ void gelu_bwd_kernel(long long total, const float *dH, const float *Z, float *dZ)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) dZ[i] = dH[i] * gelu_grad(Z[i]);
}

__device__ __forceinline__ float to_f32(bf16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float to_f32(float x) { return x; }

// FP32 activations of the last hidden layer: Hf = GELU(Z)
__global__ void gelu_f32_kernel(long long total, const float *Z, float *Hf)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) Hf[i] = tc::gelu(Z[i]);
}

// Output layer in FP32 on CUDA cores (no BF16 rounding of the last hidden
// activations or of the output weights): Y[r][o] = b[o] + sum_i W[o][i]
// GELU(Z[r][i]).  A block of (32, 8) threads takes a 32-row x 32-output tile:
// GELU(Z) and W are staged through shared memory 32 columns of the sum at a
// time, each thread accumulates four outputs, starting from the bias and
// adding the terms in index order.
__global__ void __launch_bounds__(256) dense_out_kernel(int rows, int out, int in, const float *Z, const float *W,
                                                        const float *b, float *Y)
{
    __shared__ float As[32][33], Ws[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int r0 = blockIdx.y * 32, o0 = blockIdx.x * 32;
    float acc[4];
    for (int q = 0; q < 4; ++q) acc[q] = o0 + tx < out ? b[o0 + tx] : 0.f;
    for (int k0 = 0; k0 < in; k0 += 32) {
        for (int q = 0; q < 4; ++q) {
            const int rr = ty + 8 * q, k = k0 + tx;
            As[rr][tx] = (r0 + rr < rows && k < in) ? tc::gelu(Z[(long long)(r0 + rr) * in + k]) : 0.f;
            Ws[rr][tx] = (o0 + rr < out && k < in) ? W[(long long)(o0 + rr) * in + k] : 0.f;
        }
        __syncthreads();
        const int kmax = min(32, in - k0);
        for (int kk = 0; kk < kmax; ++kk) {
            const float w = Ws[tx][kk];
            for (int q = 0; q < 4; ++q) acc[q] = fmaf(w, As[ty + 8 * q][kk], acc[q]);
        }
        __syncthreads();
    }
    for (int q = 0; q < 4; ++q) {
        const int r = r0 + ty + 8 * q, o = o0 + tx;
        if (r < rows && o < out) Y[(long long)r * out + o] = acc[q];
    }
}

// dH[b][i] = sum_o dZ[b][o] * W[o][i]
__global__ void dh_kernel(int B, int out, int in, const float *dZ, const float *W, float *dH)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= in || b >= B) return;
    float acc = 0.f;
    for (int o = 0; o < out; ++o) acc = fmaf(dZ[(long long)b * out + o], W[(long long)o * in + i], acc);
    dH[(long long)b * in + i] = acc;
}

// out[c][r] = in[r][c] as BF16 (in: R x C row-major, leading dimension ldi;
// out: C x R, leading dimension ldo), through 32 x 32 shared-memory tiles;
// block (32, 8).  Makes the K-major operands of the backward GEMMs, whose K is
// the batch.
template <class T>
__global__ void transpose_bf16_kernel(int R, int C, const T *in, int ldi, bf16 *out, int ldo)
{
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        tile[y][threadIdx.x] = (r < R && c < C) ? to_f32(in[(long long)r * ldi + c]) : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (c < C && r < R) out[(long long)c * ldo + r] = __float2bfloat16(tile[threadIdx.x][y]);
    }
}

// out[e] = sum_z part[z * zs + e]: the partial products of a split-K GEMM
__global__ void sum_splits_kernel(long long n, int S, long long zs, const float *part, float *out)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    float acc = 0.f;
    for (int z = 0; z < S; ++z) acc += part[z * zs + e];
    out[e] = acc;
}

// db[o] = sum_b dZ[b][o]: a block of 32 x 32 threads takes 32 columns, thread
// (x, y) sums rows y, y + 32, ... of column x (coalesced), then the 32 partial
// sums of a column are added in shared memory
__global__ void __launch_bounds__(1024) colsum_kernel(int B, int out, const float *dZ, float *db)
{
    __shared__ float part[32][33];
    const int o = blockIdx.x * 32 + threadIdx.x;
    float acc = 0.f;
    if (o < out)
        for (int b = threadIdx.y; b < B; b += 32) acc += dZ[(long long)b * out + o];
    part[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && o < out) {
        float s = 0.f;
        for (int y = 0; y < 32; ++y) s += part[y][threadIdx.x];
        db[o] = s;
    }
}

// The FP32 output layer's weight gradient, part[z][o][i] = sum over the z-th
// range of the batch of dY[b][o] Hf[b][i] (dY: B x M, Hf: B x N, row-major):
// 32 x 32 output tiles staged through shared memory, the batch split over the
// grid's z dimension; the caller sums the partials.  Block (32, 8), four
// outputs per thread.
__global__ void __launch_bounds__(256) sgemm_tn_splitk_kernel(int M, int N, int K, const float *A, int lda,
                                                              const float *Bm, int ldb, float *part, int kz)
{
    __shared__ float As[32][33], Bs[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int m0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
    const int kb = blockIdx.z * kz, ke = min(K, kb + kz);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = kb; k0 < ke; k0 += 32) {
        for (int q = 0; q < 4; ++q) {
            const int kk = ty + 8 * q, k = k0 + kk;
            As[kk][tx] = (k < ke && m0 + tx < M) ? A[(long long)k * lda + m0 + tx] : 0.f;
            Bs[kk][tx] = (k < ke && n0 + tx < N) ? Bm[(long long)k * ldb + n0 + tx] : 0.f;
        }
        __syncthreads();
        for (int kk = 0; kk < 32; ++kk) {
            const float bv = Bs[kk][tx];
            for (int q = 0; q < 4; ++q) acc[q] = fmaf(As[kk][ty + 8 * q], bv, acc[q]);
        }
        __syncthreads();
    }
    float *p = part + (long long)blockIdx.z * M * N;
    for (int q = 0; q < 4; ++q) {
        const int mm = m0 + ty + 8 * q, nn = n0 + tx;
        if (mm < M && nn < N) p[(long long)mm * N + nn] = acc[q];
    }
}

__global__ void adam_kernel(long long n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2,
                            float eps, float c1, float c2, bf16 *pb)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16(pi);
}

__global__ void to_bf16_kernel(long long n, const float *p, bf16 *pb)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pb[i] = __float2bfloat16(p[i]);
}

// network output -> n complex shifts per matrix (SoA vectors)
__global__ void shifts_out_kernel(long long count, int n, int tc, int nout_pad, const float *Y, const float *mean,
                                  const float *stdv, double *rS, double *iS)
{
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= count) return;
    const long long vo = soa_off_s(m, n, tc);
    for (int i = 0; i < n; ++i) {
        const float re = Y[m * nout_pad + i] * stdv[i] + mean[i];
        const float im = Y[m * nout_pad + n + i] * stdv[n + i] + mean[n + i];
        rS[vo + (long long)i * tc] = re;
        iS[vo + (long long)i * tc] = im;
    }
}

inline unsigned nb(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void load_shiftnet_kernels()
{
    load_kernel(tc::gemm_bf16_persistent_kernel<64>);
    load_kernel(tc::gemm_bf16_persistent_kernel<128>);
    load_kernel(tc::gemm_bf16_persistent_kernel<256>);
    load_kernel(tc::gemm_bf16_tma_kernel<64>);
    load_kernel(tc::gemm_bf16_tma_kernel<128>);
    load_kernel(tc::gemm_bf16_tma_kernel<256>);
    load_kernel(tc::gemm_bf16_kernel<64>);
    load_kernel(tc::gemm_bf16_kernel<256>);
    load_kernel(features_kernel);
    load_kernel(targets_kernel);
    load_kernel(colstats_bf16_kernel);
    load_kernel(target_stats_kernel);
    load_kernel(chamfer_kernel);
    load_kernel(gelu_bwd_kernel);
    load_kernel(sgemm_tn_splitk_kernel);
    load_kernel(transpose_bf16_kernel<float>);
    load_kernel(transpose_bf16_kernel<bf16>);
    load_kernel(sum_splits_kernel);
    load_kernel(colsum_kernel);
    load_kernel(gelu_f32_kernel);
    load_kernel(dense_out_kernel);
    load_kernel(dh_kernel);
    load_kernel(adam_kernel);
    load_kernel(to_bf16_kernel);
    load_kernel(shifts_out_kernel);
}

}  // namespace ves

// ---------------------------------------------------------------------------
// The network object and its C ABI.
// ---------------------------------------------------------------------------
struct ves_shiftnet {
    ves_shiftnet_config cfg{};
    int n = 0, P = 0, H = 0, L = 0, F = 0, S = 0, kin = 0, kin_pad = 0, nout = 0, nout_pad = 0;
    // layers 0..L-1: hidden (tcgen05, BF16 in, FP32 accumulate, GELU);
    // layer L: output (FP32, CUDA cores)
    int in[ves::kMaxLayers + 1] = {}, out[ves::kMaxLayers + 1] = {};
    float *W[ves::kMaxLayers + 1] = {}, *b[ves::kMaxLayers + 1] = {};
    float *mW[ves::kMaxLayers + 1] = {}, *vW[ves::kMaxLayers + 1] = {};
    float *mb[ves::kMaxLayers + 1] = {}, *vb[ves::kMaxLayers + 1] = {};
    ves::bf16 *Wb[ves::kMaxLayers] = {};
    float *fmean = nullptr, *fstd = nullptr, *tmean = nullptr, *tstd = nullptr;
    long long step = 0;
    int dev = 0;
};

namespace {

void net_free(ves_shiftnet *t)
{
    for (int l = 0; l <= t->L; ++l) {
        cudaFree(t->W[l]); cudaFree(t->b[l]); cudaFree(t->mW[l]); cudaFree(t->vW[l]);
        cudaFree(t->mb[l]); cudaFree(t->vb[l]);
        if (l < t->L) cudaFree(t->Wb[l]);
    }
    cudaFree(t->fmean); cudaFree(t->fstd); cudaFree(t->tmean); cudaFree(t->tstd);
}

bool net_alloc(ves_shiftnet *t)
{
    bool ok = true;
    for (int l = 0; l <= t->L && ok; ++l) {
        const size_t nw = (size_t)t->out[l] * t->in[l];
        ok &= cudaMalloc(&t->W[l], nw * 4) == cudaSuccess;
        ok &= cudaMalloc(&t->b[l], t->out[l] * 4) == cudaSuccess;
        ok &= cudaMalloc(&t->mW[l], nw * 4) == cudaSuccess;
        ok &= cudaMalloc(&t->vW[l], nw * 4) == cudaSuccess;
        ok &= cudaMalloc(&t->mb[l], t->out[l] * 4) == cudaSuccess;
        ok &= cudaMalloc(&t->vb[l], t->out[l] * 4) == cudaSuccess;
        if (l < t->L) ok &= cudaMalloc(&t->Wb[l], nw * 2) == cudaSuccess;
        if (!ok) break;
        cudaMemset(t->mW[l], 0, nw * 4);
        cudaMemset(t->vW[l], 0, nw * 4);
        cudaMemset(t->mb[l], 0, t->out[l] * 4);
        cudaMemset(t->vb[l], 0, t->out[l] * 4);
    }
    ok &= cudaMalloc(&t->fmean, t->kin_pad * 4) == cudaSuccess && cudaMalloc(&t->fstd, t->kin_pad * 4) == cudaSuccess;
    ok &= cudaMalloc(&t->tmean, t->nout_pad * 4) == cudaSuccess && cudaMalloc(&t->tstd, t->nout_pad * 4) == cudaSuccess;
    return ok;
}

bool config_ok(const ves_shiftnet_config &c)
{
    return c.dim >= 1 && c.dim <= ves::kMaxDimNet && c.n_params >= 0 && c.n_params <= 64 && c.hidden >= 16 &&
           c.hidden <= 256 && (c.hidden % 16) == 0 && c.layers >= 1 && c.layers <= ves::kMaxLayers &&
           c.fourier >= 0 && c.n_params * c.fourier <= ves::kMaxFourier && (c.loss == 0 || c.loss == 1) &&
           c.delta > 0.f && c.delta < 1e3f && (c.subdiag == 0 || c.subdiag == 1);
}

void set_geometry(ves_shiftnet *t, const ves_shiftnet_config &c)
{
    t->cfg = c;
    t->n = c.dim; t->P = c.n_params; t->H = c.hidden; t->L = c.layers; t->F = c.fourier; t->S = c.subdiag ? 1 : 0;
    t->kin = t->P + 2 * t->P * t->F + 2 * t->n + t->S * (t->n - 1);
    t->kin_pad = (t->kin + 31) / 32 * 32;
    t->nout = 2 * t->n;
    t->nout_pad = (t->nout + 15) / 16 * 16;
    for (int l = 0; l <= t->L; ++l) {
        t->in[l] = l == 0 ? t->kin_pad : t->H;
        t->out[l] = l == t->L ? t->nout_pad : t->H;
    }
}

// Activation buffers of a forward pass over `rows` rows.
struct Acts {
    float *Z[ves::kMaxLayers] = {};     // FP32 pre-activations of the hidden layers [rows x H]
    ves::bf16 *Hs[ves::kMaxLayers] = {};  // BF16 activations of the hidden layers [rows x H]
    float *Hf = nullptr;                  // FP32 activations of the last hidden layer
    float *Y = nullptr;                   // output [rows x nout_pad]
};

size_t acts_bytes(const ves_shiftnet *t, size_t rows)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    return t->L * (al(rows * t->H * 4) + al(rows * t->H * 2)) + al(rows * t->H * 4) + al(rows * t->nout_pad * 4);
}

Acts carve_acts(const ves_shiftnet *t, size_t rows, char *&w)
{
    auto take = [&](size_t bytes) { char *p = w; w += (bytes + 255) & ~(size_t)255; return p; };
    Acts a;
    for (int l = 0; l < t->L; ++l) {
        a.Z[l] = reinterpret_cast<float *>(take(rows * t->H * 4));
        a.Hs[l] = reinterpret_cast<ves::bf16 *>(take(rows * t->H * 2));
    }
    a.Hf = reinterpret_cast<float *>(take(rows * t->H * 4));
    a.Y = reinterpret_cast<float *>(take(rows * t->nout_pad * 4));
    return a;
}

// forward over `rows` rows of X (BF16 [rows x kin_pad]); training keeps every
// hidden layer's FP32 pre-activation for the backward pass, inference only the
// last one (the FP32 output layer's input)
cudaError_t forward(const ves_shiftnet *t, int rows, const ves::bf16 *X, const Acts &a, int *err, cudaStream_t st,
                    bool training)
{
    const void *in = X;
    int ld = t->kin_pad;
    for (int l = 0; l < t->L; ++l) {
        float *zf = (training || l == t->L - 1) ? a.Z[l] : nullptr;
        cudaError_t e = ves::launch_gemm_bf16(rows, t->H, t->in[l], in, ld, t->Wb[l], t->in[l], t->b[l], 1, a.Hs[l],
                                              zf, t->H, err, st);
        if (e != cudaSuccess) return e;
        in = a.Hs[l];
        ld = t->H;
    }
    if (training) {  // FP32 activations of the last hidden layer, for the output layer's weight gradient
        const long long nh = (long long)rows * t->H;
        ves::gelu_f32_kernel<<<ves::nb(nh), 256, 0, st>>>(nh, a.Z[t->L - 1], a.Hf);
    }
    ves::dense_out_kernel<<<dim3(ves::nb(t->nout_pad, 32), ves::nb(rows, 32)), dim3(32, 8), 0, st>>>(rows, t->nout_pad, t->H, a.Z[t->L - 1],
                                                                         t->W[t->L], t->b[t->L], a.Y);
    return cudaGetLastError();
}

// Record a message for ves_last_error() and return the code.
int fail(int code, const char *msg)
{
    ves::set_error_message(msg);
    return code;
}

int create_from_config(ves_shiftnet **out, const ves_shiftnet_config &c)
{
    ves::set_error_message("");
    if (!out || !config_ok(c)) return fail(VES_ERR_ARG, "shiftnet: bad configuration");
    ves_shiftnet *t = new ves_shiftnet();
    cudaGetDevice(&t->dev);
    set_geometry(t, c);
    if (!net_alloc(t)) { net_free(t); delete t; return fail(VES_ERR_NOMEM, "shiftnet: device allocation failed"); }
    // He-style initialisation from a fixed seed (host), zero biases, identity normalisation
    std::mt19937_64 rng(c.seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int l = 0; l <= t->L; ++l) {
        const int fan_in = l == 0 ? t->kin : t->in[l];
        std::vector<float> w((size_t)t->out[l] * t->in[l], 0.f);
        const float sc = std::sqrt((l == t->L ? 1.f : 2.f) / (float)fan_in);
        for (int o = 0; o < t->out[l]; ++o)
            for (int i = 0; i < t->in[l]; ++i)
                if ((l != 0 || i < t->kin) && (l != t->L || o < t->nout)) w[(size_t)o * t->in[l] + i] = nd(rng) * sc;
        cudaMemcpy(t->W[l], w.data(), w.size() * 4, cudaMemcpyHostToDevice);
        cudaMemset(t->b[l], 0, t->out[l] * 4);
        if (l < t->L) ves::to_bf16_kernel<<<ves::nb((long long)w.size()), 256>>>((long long)w.size(), t->W[l], t->Wb[l]);
    }
    std::vector<float> zero(512, 0.f), one(512, 1.f);
    cudaMemcpy(t->fmean, zero.data(), t->kin_pad * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(t->fstd, one.data(), t->kin_pad * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(t->tmean, zero.data(), t->nout_pad * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(t->tstd, one.data(), t->nout_pad * 4, cudaMemcpyHostToDevice);
    if (cudaDeviceSynchronize() != cudaSuccess) { net_free(t); delete t; return fail(VES_ERR_CUDA, "shiftnet: initialisation failed"); }
    *out = t;
    return VES_OK;
}

// Gradient buffers of one training step over `batch` rows.
struct GradBufs {
    float *gW[ves::kMaxLayers + 1] = {}, *gb[ves::kMaxLayers + 1] = {};
    float *dA = nullptr, *dB = nullptr;  // FP32 [batch x max(H, nout_pad)]: dY, then dH / dZ of the hidden layers
    ves::bf16 *dZ16 = nullptr;            // dZ as BF16 [batch x H]: A operand of dH = dZ W
    ves::bf16 *dZt = nullptr;             // dZ transposed [H x batch]: A operand of dW = dZ^T Hin
    ves::bf16 *HinT = nullptr;            // the layer input transposed [max(kin_pad, H) x batch]
    ves::bf16 *WbT = nullptr;             // BF16 weights transposed [H x H]: B operand of dH
    float *part = nullptr;                // split-K partials [splits x max(H, nout_pad) x max(kin_pad, H)]
    int splits = 1;
};

// split-K factor of the weight-gradient GEMMs: K = batch in ranges of >= 64
int grad_splits(int batch) { return std::max(1, std::min(16, batch / 64)); }

bool grad_alloc(const ves_shiftnet *t, int batch, GradBufs &g)
{
    const int H = t->H, wmax = std::max(H, t->nout_pad), imax = std::max(t->kin_pad, H);
    g.splits = grad_splits(batch);
    bool ok = cudaMalloc(&g.dA, (size_t)batch * wmax * 4) == cudaSuccess &&
              cudaMalloc(&g.dB, (size_t)batch * wmax * 4) == cudaSuccess &&
              cudaMalloc(&g.dZ16, (size_t)batch * H * 2) == cudaSuccess &&
              cudaMalloc(&g.dZt, (size_t)batch * H * 2) == cudaSuccess &&
              cudaMalloc(&g.HinT, (size_t)batch * imax * 2) == cudaSuccess &&
              cudaMalloc(&g.WbT, (size_t)H * H * 2) == cudaSuccess &&
              cudaMalloc(&g.part, (size_t)g.splits * std::max(H, t->nout_pad) * imax * 4) == cudaSuccess;
    for (int l = 0; l <= t->L && ok; ++l) {
        ok &= cudaMalloc(&g.gW[l], (size_t)t->out[l] * t->in[l] * 4) == cudaSuccess;
        ok &= cudaMalloc(&g.gb[l], (size_t)t->out[l] * 4) == cudaSuccess;
    }
    return ok;
}

void grad_free(const ves_shiftnet *t, GradBufs &g)
{
    cudaFree(g.dA); cudaFree(g.dB); cudaFree(g.dZ16); cudaFree(g.dZt); cudaFree(g.HinT); cudaFree(g.WbT);
    cudaFree(g.part);
    for (int l = 0; l <= t->L; ++l) { cudaFree(g.gW[l]); cudaFree(g.gb[l]); }
}

// Loss and parameter gradients of one batch (features Xb, standardised
// targets Tb), into g.gW / g.gb; the batch loss is added to *loss.
//   output layer (FP32 on CUDA cores, like its forward): dW = dY^T Hf, dH = dY W
//   hidden layers (tcgen05): dW = dZ^T Hin as a split-K BF16 GEMM over the
//   batch (FP32 partials summed), dH = dZ W as a BF16 GEMM with W transposed;
//   db = column sums of dZ; then dZ of the layer below = dH * GELU'(Z).
// dZ is rounded to BF16 for the tensor cores and accumulated in FP32.
void step_gradients(const ves_shiftnet *t, int batch, const ves::bf16 *Xb, const float *Tb, const Acts &a,
                    GradBufs &g, float *loss, int *err, cudaStream_t st)
{
    const int n = t->n, H = t->H, L = t->L;
    forward(t, batch, Xb, a, err, st, true);
    ves::chamfer_kernel<<<ves::nb(batch, 128), 128, 0, st>>>(batch, n, t->nout_pad, a.Y, Tb, g.dA, loss, t->cfg.loss,
                                                             t->cfg.delta);
    {  // output layer: dW = dY^T Hf (FP32, split over the batch), db = column sums of dY
        const int kz = (batch + g.splits - 1) / g.splits;
        ves::sgemm_tn_splitk_kernel<<<dim3(ves::nb(H, 32), ves::nb(t->nout_pad, 32), g.splits), dim3(32, 8), 0, st>>>(
            t->nout_pad, H, batch, g.dA, t->nout_pad, a.Hf, H, g.part, kz);
        const long long nw = (long long)t->nout_pad * H;
        ves::sum_splits_kernel<<<ves::nb(nw), 256, 0, st>>>(nw, g.splits, nw, g.part, g.gW[L]);
        ves::colsum_kernel<<<ves::nb(t->nout_pad, 32), dim3(32, 32), 0, st>>>(batch, t->nout_pad, g.dA, g.gb[L]);
    }
    ves::dh_kernel<<<dim3(ves::nb(H, 128), batch), 128, 0, st>>>(batch, t->nout_pad, H, g.dA, t->W[L], g.dB);
    ves::gelu_bwd_kernel<<<ves::nb((long long)batch * H), 256, 0, st>>>((long long)batch * H, g.dB, a.Z[L - 1], g.dB);
    float *dZ = g.dB, *dH = g.dA;
    const dim3 tb(32, 8);
    for (int l = L - 1; l >= 0; --l) {
        const ves::bf16 *Hin = l == 0 ? Xb : a.Hs[l - 1];
        const int in = t->in[l];  // kin_pad for the first layer, H otherwise (= the leading dimension of Hin)
        const long long nz = (long long)batch * H;
        ves::transpose_bf16_kernel<float><<<dim3(ves::nb(H, 32), ves::nb(batch, 32)), tb, 0, st>>>(batch, H, dZ, H,
                                                                                                  g.dZt, batch);
        ves::transpose_bf16_kernel<ves::bf16><<<dim3(ves::nb(in, 32), ves::nb(batch, 32)), tb, 0, st>>>(
            batch, in, Hin, in, g.HinT, batch);
        ves::launch_gemm_bf16_splitk(H, in, batch, g.dZt, batch, g.HinT, batch, g.part, in, g.splits, err, st);
        ves::sum_splits_kernel<<<ves::nb((long long)H * in), 256, 0, st>>>((long long)H * in, g.splits,
                                                                          (long long)H * in, g.part, g.gW[l]);
        ves::colsum_kernel<<<ves::nb(H, 32), dim3(32, 32), 0, st>>>(batch, H, dZ, g.gb[l]);
        if (l > 0) {
            ves::to_bf16_kernel<<<ves::nb(nz), 256, 0, st>>>(nz, dZ, g.dZ16);
            ves::transpose_bf16_kernel<ves::bf16><<<dim3(ves::nb(H, 32), ves::nb(H, 32)), tb, 0, st>>>(
                H, H, t->Wb[l], H, g.WbT, H);
            ves::launch_gemm_bf16(batch, H, H, g.dZ16, H, g.WbT, H, nullptr, 0, nullptr, dH, H, err, st);
            ves::gelu_bwd_kernel<<<ves::nb(nz), 256, 0, st>>>(nz, dH, a.Z[l - 1], dH);
            float *tmp = dZ; dZ = dH; dH = tmp;
        }
    }
}

}  // namespace

extern "C" {

void ves_shiftnet_default_config(ves_shiftnet_config *c)
{
    if (!c) return;
    c->dim = 16;
    c->n_params = 0;
    c->hidden = 256;
    c->layers = 3;
    c->fourier = 0;
    c->loss = VES_SHIFTNET_LOSS_CHAMFER;
    c->delta = 0.01f;
    c->seed = 0;
    c->subdiag = 0;
}

int ves_shiftnet_create_config(ves_shiftnet **out, const ves_shiftnet_config *cfg)
{
    if (!cfg) return fail(VES_ERR_ARG, "shiftnet: null configuration");
    return create_from_config(out, *cfg);
}

int ves_shiftnet_create(ves_shiftnet **out, int dim, int n_params, int hidden, unsigned long long seed)
{
    ves_shiftnet_config c;
    ves_shiftnet_default_config(&c);
    c.dim = dim;
    c.n_params = n_params;
    c.hidden = hidden;
    c.seed = seed;
    return create_from_config(out, c);
}

void ves_shiftnet_destroy(ves_shiftnet *t)
{
    if (!t) return;
    net_free(t);
    delete t;
}

int ves_shiftnet_train(ves_shiftnet *t, long long count, int thread_cnt, const double *params, const double *rA,
                       const double *iA, const double *rE, const double *iE, int epochs, int batch, float lr,
                       unsigned long long seed, float *loss_per_epoch, void *stream)
{
    if (!t || count < 1 || count > 0x7fffffffLL || thread_cnt < 1 || (count % thread_cnt) || !rA || !iA || !rE ||
        !iE || epochs < 0 || batch < 32 || batch > 65536 || !(lr > 0.f))
        return fail(VES_ERR_ARG, "shiftnet train: bad arguments (count a multiple of thread_cnt, 32 <= batch <= 65536)");
    if (t->P > 0 && !params) return fail(VES_ERR_ARG, "shiftnet train: the network needs family parameters");
    ves::set_error_message("");
    cudaStream_t st = (cudaStream_t)stream;
    const int n = t->n, L = t->L;
    ves::bf16 *Xall = nullptr, *Xb = nullptr;
    float *Tall = nullptr, *Tb = nullptr, *loss = nullptr;
    GradBufs g;
    int *rows = nullptr, *err = nullptr;
    char *actbuf = nullptr;
    bool ok = cudaMalloc(&Xall, (size_t)count * t->kin_pad * 2) == cudaSuccess &&
              cudaMalloc(&Tall, (size_t)count * t->nout_pad * 4) == cudaSuccess &&
              cudaMalloc(&Xb, (size_t)batch * t->kin_pad * 2) == cudaSuccess &&
              cudaMalloc(&Tb, (size_t)batch * t->nout_pad * 4) == cudaSuccess &&
              cudaMalloc(&loss, 4 * 2) == cudaSuccess && cudaMalloc(&rows, (size_t)count * 4) == cudaSuccess &&
              cudaMalloc(&err, 4) == cudaSuccess && cudaMalloc(&actbuf, acts_bytes(t, batch)) == cudaSuccess &&
              grad_alloc(t, batch, g);
    int rc = ok ? VES_OK : VES_ERR_NOMEM;
    if (rc == VES_OK) {
        char *w = actbuf;
        const Acts a = carve_acts(t, batch, w);
        cudaMemsetAsync(err, 0, 4, st);
        // standardisation statistics over the whole training set
        ves::features_kernel<<<ves::nb(count * 32, 256), 256, 0, st>>>(count, n, t->P, t->F, t->S, thread_cnt, params, rA, iA,
                                                             nullptr, nullptr, t->kin, t->kin_pad, Xall, nullptr);
        ves::colstats_bf16_kernel<<<ves::nb(t->kin_pad), 256, 0, st>>>(count, t->kin_pad, t->kin_pad, Xall, t->fmean,
                                                                      t->fstd);
        ves::features_kernel<<<ves::nb(count * 32, 256), 256, 0, st>>>(count, n, t->P, t->F, t->S, thread_cnt, params, rA, iA,
                                                             t->fmean, t->fstd, t->kin, t->kin_pad, Xall, nullptr);
        ves::targets_kernel<<<ves::nb(count * 32, 256), 256, 0, st>>>(count, n, thread_cnt, rE, iE, nullptr, nullptr,
                                                            t->nout_pad, Tall, nullptr);
        ves::target_stats_kernel<<<1, 256, 0, st>>>(count, n, t->nout_pad, t->nout_pad, Tall, t->tmean, t->tstd);
        ves::targets_kernel<<<ves::nb(count * 32, 256), 256, 0, st>>>(count, n, thread_cnt, rE, iE, t->tmean, t->tstd,
                                                            t->nout_pad, Tall, nullptr);
        std::mt19937_64 rng(seed);
        std::vector<int> perm(count);
        for (long long i = 0; i < count; ++i) perm[i] = (int)i;
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        const long long steps_per_epoch = count / batch;
        const double total_steps = (double)std::max<long long>(1, steps_per_epoch * epochs);
        long long k = 0;  // step within this call: cosine decay from lr to lr / 50
        for (int ep = 0; ep < epochs && rc == VES_OK; ++ep) {
            std::shuffle(perm.begin(), perm.end(), rng);
            cudaMemcpyAsync(rows, perm.data(), (size_t)count * 4, cudaMemcpyHostToDevice, st);
            cudaMemsetAsync(loss, 0, 4, st);
            for (long long s = 0; s < steps_per_epoch; ++s) {
                const int *r = rows + s * batch;
                ves::features_kernel<<<ves::nb(batch * 32, 256), 256, 0, st>>>(batch, n, t->P, t->F, t->S, thread_cnt, params,
                                                                     rA, iA, t->fmean, t->fstd, t->kin, t->kin_pad,
                                                                     Xb, r);
                ves::targets_kernel<<<ves::nb(batch * 32, 256), 256, 0, st>>>(batch, n, thread_cnt, rE, iE, t->tmean, t->tstd,
                                                                    t->nout_pad, Tb, r);
                step_gradients(t, batch, Xb, Tb, a, g, loss, err, st);
                ++t->step;
                const float lr_k = (float)(lr * (0.02 + 0.49 * (1.0 + std::cos(3.141592653589793 * (double)k++ /
                                                                                 total_steps))));
                const float c1 = 1.f - std::pow(b1, (float)t->step), c2 = 1.f - std::pow(b2, (float)t->step);
                for (int l = 0; l <= L; ++l) {
                    const long long nw = (long long)t->out[l] * t->in[l];
                    ves::adam_kernel<<<ves::nb(nw), 256, 0, st>>>(nw, t->W[l], g.gW[l], t->mW[l], t->vW[l], lr_k, b1,
                                                                 b2, eps, c1, c2, l < L ? t->Wb[l] : nullptr);
                    ves::adam_kernel<<<ves::nb(t->out[l]), 256, 0, st>>>(t->out[l], t->b[l], g.gb[l], t->mb[l],
                                                                        t->vb[l], lr_k, b1, b2, eps, c1, c2, nullptr);
                }
            }
            float lh = 0.f;
            cudaMemcpyAsync(&lh, loss, 4, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) { rc = VES_ERR_CUDA; break; }
            if (loss_per_epoch) loss_per_epoch[ep] = steps_per_epoch ? lh / (float)steps_per_epoch : 0.f;
        }
        int he = 0;
        cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost);
        if (he) rc = VES_ERR_CUDA;
        if (cudaDeviceSynchronize() != cudaSuccess) rc = VES_ERR_CUDA;
    }
    cudaFree(Xall); cudaFree(Tall); cudaFree(Xb); cudaFree(Tb); cudaFree(loss);
    cudaFree(rows); cudaFree(err); cudaFree(actbuf);
    grad_free(t, g);
    if (rc == VES_ERR_NOMEM) return fail(rc, "shiftnet train: device allocation failed");
    if (rc != VES_OK) return fail(rc, "shiftnet train: a kernel failed or a tensor-core wait timed out");
    return rc;
}

size_t ves_shiftnet_param_count(const ves_shiftnet *t)
{
    if (!t) return 0;
    size_t c = 0;
    for (int l = 0; l <= t->L; ++l) c += (size_t)t->out[l] * t->in[l] + t->out[l];
    return c;
}

int ves_shiftnet_gradient(const ves_shiftnet *t, long long count, int thread_cnt, const double *params,
                          const double *rA, const double *iA, const double *rE, const double *iE, float *grad,
                          float *loss, void *stream)
{
    if (!t || count < 32 || count > 65536 || thread_cnt < 1 || (count % thread_cnt) || !rA || !iA || !rE || !iE ||
        !grad || !loss)
        return fail(VES_ERR_ARG, "shiftnet gradient: bad arguments (32 <= count <= 65536, a multiple of thread_cnt)");
    if (t->P > 0 && !params) return fail(VES_ERR_ARG, "shiftnet gradient: the network needs family parameters");
    ves::set_error_message("");
    cudaStream_t st = (cudaStream_t)stream;
    const int batch = (int)count;
    ves::bf16 *X = nullptr;
    float *T = nullptr;
    int *err = nullptr;
    char *actbuf = nullptr;
    GradBufs g;
    bool ok = cudaMalloc(&X, (size_t)batch * t->kin_pad * 2) == cudaSuccess &&
              cudaMalloc(&T, (size_t)batch * t->nout_pad * 4) == cudaSuccess && cudaMalloc(&err, 4) == cudaSuccess &&
              cudaMalloc(&actbuf, acts_bytes(t, batch)) == cudaSuccess && grad_alloc(t, batch, g);
    int rc = ok ? VES_OK : VES_ERR_NOMEM;
    if (rc == VES_OK) {
        char *w = actbuf;
        const Acts a = carve_acts(t, batch, w);
        cudaMemsetAsync(err, 0, 4, st);
        cudaMemsetAsync(loss, 0, 4, st);
        ves::features_kernel<<<ves::nb(batch * 32, 256), 256, 0, st>>>(batch, t->n, t->P, t->F, t->S, thread_cnt, params, rA, iA,
                                                             t->fmean, t->fstd, t->kin, t->kin_pad, X, nullptr);
        ves::targets_kernel<<<ves::nb(batch * 32, 256), 256, 0, st>>>(batch, t->n, thread_cnt, rE, iE, t->tmean, t->tstd,
                                                            t->nout_pad, T, nullptr);
        step_gradients(t, batch, X, T, a, g, loss, err, st);
        size_t off = 0;
        for (int l = 0; l <= t->L; ++l) {
            const size_t nw = (size_t)t->out[l] * t->in[l];
            cudaMemcpyAsync(grad + off, g.gW[l], nw * 4, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(grad + off + nw, g.gb[l], t->out[l] * 4, cudaMemcpyDeviceToDevice, st);
            off += nw + t->out[l];
        }
        int he = 0;
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = VES_ERR_CUDA;
        cudaMemcpy(&he, err, 4, cudaMemcpyDeviceToHost);
        if (he) rc = VES_ERR_CUDA;
    }
    cudaFree(X); cudaFree(T); cudaFree(err); cudaFree(actbuf);
    grad_free(t, g);
    if (rc == VES_ERR_NOMEM) return fail(rc, "shiftnet gradient: device allocation failed");
    if (rc != VES_OK) return fail(rc, "shiftnet gradient: a kernel failed or a tensor-core wait timed out");
    return rc;
}

size_t ves_shiftnet_predict_workspace_size(const ves_shiftnet *t, long long count)
{
    if (!t || count < 0) return 0;
    const size_t rows = (size_t)count;
    return ((rows * t->kin_pad * 2 + 255) & ~(size_t)255) + acts_bytes(t, rows) + 256;
}

int ves_shiftnet_predict(const ves_shiftnet *t, long long count, int thread_cnt, const double *params,
                         const double *rA, const double *iA, double *rS, double *iS, void *workspace,
                         size_t workspace_bytes, void *stream)
{
    if (!t || count < 0 || count > 0x7fffffffLL || thread_cnt < 1 || (count % thread_cnt) || !rA || !iA || !rS ||
        !iS)
        return fail(VES_ERR_ARG, "shiftnet predict: bad arguments");
    if (t->P > 0 && !params) return fail(VES_ERR_ARG, "shiftnet predict: the network needs family parameters");
    ves::set_error_message("");
    if (count == 0) return VES_OK;
    if (!workspace || workspace_bytes < ves_shiftnet_predict_workspace_size(t, count))
        return fail(VES_ERR_ARG, "shiftnet predict: workspace missing or too small");
    cudaStream_t st = (cudaStream_t)stream;
    char *w = static_cast<char *>(workspace);
    ves::bf16 *X = reinterpret_cast<ves::bf16 *>(w);
    w += ((size_t)count * t->kin_pad * 2 + 255) & ~(size_t)255;
    const Acts a = carve_acts(t, (size_t)count, w);
    int *err = nullptr;  // a GEMM wait that gives up leaves its tile unwritten; training checks the flag
    ves::features_kernel<<<ves::nb(count * 32, 256), 256, 0, st>>>(count, t->n, t->P, t->F, t->S, thread_cnt, params, rA, iA,
                                                         t->fmean, t->fstd, t->kin, t->kin_pad, X, nullptr);
    if (forward(t, (int)count, X, a, err, st, false) != cudaSuccess) return fail(VES_ERR_CUDA, "shiftnet predict: launch failed");
    ves::shifts_out_kernel<<<ves::nb(count), 256, 0, st>>>(count, t->n, thread_cnt, t->nout_pad, a.Y, t->tmean,
                                                           t->tstd, rS, iS);
    return cudaGetLastError() == cudaSuccess ? VES_OK : VES_ERR_CUDA;
}

// Flat binary checkpoint: header {magic, version 2, n, P, H, L, F, loss, step},
// delta (float), seed (u64), then per layer W and b (FP32), then the four
// normalisation vectors.
int ves_shiftnet_save(const ves_shiftnet *t, const char *path)
{
    if (!t || !path) return fail(VES_ERR_ARG, "shiftnet save: null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(VES_ERR_ARG, "shiftnet save: cannot open the file");
    const int hdr[10] = {0x56455353, 3, t->n, t->P, t->H, t->L, t->F, t->cfg.loss, (int)t->step, t->S};
    bool ok = fwrite(hdr, sizeof hdr, 1, f) == 1 && fwrite(&t->cfg.delta, 4, 1, f) == 1 &&
              fwrite(&t->cfg.seed, 8, 1, f) == 1;
    auto put = [&](const float *d, size_t cnt) {
        std::vector<float> h(cnt);
        ok = ok && cudaMemcpy(h.data(), d, cnt * 4, cudaMemcpyDeviceToHost) == cudaSuccess &&
             fwrite(h.data(), 4, cnt, f) == cnt;
    };
    for (int l = 0; l <= t->L; ++l) {
        put(t->W[l], (size_t)t->out[l] * t->in[l]);
        put(t->b[l], t->out[l]);
    }
    put(t->fmean, t->kin_pad); put(t->fstd, t->kin_pad); put(t->tmean, t->nout_pad); put(t->tstd, t->nout_pad);
    fclose(f);
    return ok ? VES_OK : VES_ERR_CUDA;
}

int ves_shiftnet_load(ves_shiftnet **out, const char *path)
{
    if (!out || !path) return fail(VES_ERR_ARG, "shiftnet load: null argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(VES_ERR_ARG, "shiftnet load: cannot open the file");
    // version 2: 9 header ints; version 3 adds the subdiagonal-feature flag
    int hdr[10] = {};
    ves_shiftnet_config c;
    ves_shiftnet_default_config(&c);
    bool hok = fread(hdr, sizeof(int), 9, f) == 9 && hdr[0] == 0x56455353 && (hdr[1] == 2 || hdr[1] == 3);
    if (hok && hdr[1] == 3) hok = fread(hdr + 9, sizeof(int), 1, f) == 1;
    if (!hok || fread(&c.delta, 4, 1, f) != 1 || fread(&c.seed, 8, 1, f) != 1) {
        fclose(f);
        return fail(VES_ERR_ARG, "shiftnet load: not a version-2 or version-3 shift network checkpoint");
    }
    c.dim = hdr[2]; c.n_params = hdr[3]; c.hidden = hdr[4]; c.layers = hdr[5]; c.fourier = hdr[6]; c.loss = hdr[7];
    c.subdiag = hdr[9];
    ves_shiftnet *t = nullptr;
    int rc = create_from_config(&t, c);
    if (rc != VES_OK) { fclose(f); return rc; }
    t->step = hdr[8];
    bool ok = true;
    auto get = [&](float *d, size_t cnt) {
        std::vector<float> h(cnt);
        ok = ok && fread(h.data(), 4, cnt, f) == cnt &&
             cudaMemcpy(d, h.data(), cnt * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    for (int l = 0; l <= t->L; ++l) {
        get(t->W[l], (size_t)t->out[l] * t->in[l]);
        get(t->b[l], t->out[l]);
        const long long nw = (long long)t->out[l] * t->in[l];
        if (l < t->L) ves::to_bf16_kernel<<<ves::nb(nw), 256>>>(nw, t->W[l], t->Wb[l]);
    }
    get(t->fmean, t->kin_pad); get(t->fstd, t->kin_pad); get(t->tmean, t->nout_pad); get(t->tstd, t->nout_pad);
    fclose(f);
    if (!ok || cudaDeviceSynchronize() != cudaSuccess) {
        ves_shiftnet_destroy(t);
        return fail(VES_ERR_CUDA, "shiftnet load: truncated file or device error");
    }
    *out = t;
    return VES_OK;
}

}  // extern "C"
