// ves_mixed.cu -- mixed-precision form of the eigensolver: the whole
// reference path (zgehrd -> zunghr -> zlahqr -> ztrevc back substitution) in
// complex FP32, then every eigenpair refined by Newton's method with the
// residual in FP64.
//
// Why: on GB300 the FP32 pipe retires ~58x the FP64 pipe's FMAs, so the
// O(90 n^3) flops of the reduction and the QR sweeps are cheap in FP32; the
// FP64 work shrinks to the residuals r = A v - lambda v (4 n^2 FMAs per pair
// and step).
//
// Two kernels:
//  schur32  one matrix per lane (the lockstep routines of ves_device.cuh in
//           float): T, Z and the T-eigenvectors X of each matrix are left in an
//           HBM buffer laid out [group of 32][element][lane].  Matrices whose
//           data are non-finite or beyond FP32 range, or whose FP32 QR hit the
//           sweep cap, are put on the FP64 list here.
//  refine   one EIGENPAIR per lane: the lanes of one matrix read the same A, T,
//           Z, X elements (one broadcast transaction each) and every FP64
//           instruction works on 32 pairs.
//
// Refinement of pair k (Newton on (A - lambda I) v = 0 with the component of v
// along the k-th Schur vector held fixed; Dongarra, Moler & Wilkinson,
// "Improving the accuracy of computed eigenvalues and eigenvectors", SIAM J.
// Numer. Anal. 20 (1983)).  With the FP32 Schur form A ~ Z T Z^H and the
// T-eigenvector x (x_i = 0 for i > k):
//     r    = A v - lambda v                    FP64
//     r'   = Z^H r                             FP32
//     (T - lambda I) dx - dlambda x = -r', dx_k = 0:
//        rows i > k : back substitution for dx_i
//        row  k     : dlambda x_k = r'_k + sum_{j>k} T_kj dx_j
//        rows i < k : back substitution including + dlambda x_i
//     v += Z dx, lambda += dlambda             FP64 update
// until ||r|| <= tol ||A||_F ||v|| (the final residual, FP64).  A pair that is
// not certified after `max_steps` corrections sends its matrix to the FP64
// solver (the caller's second launch over the list).
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>
#include <cstdlib>

namespace ves {

namespace {

constexpr int kSchurThreads = 128;
constexpr int kRefineThreads = 64;

__device__ __forceinline__ long long soa_off_m(long long m, long long len, int tc)
{
    return (m / tc) * (long long)tc * len + (m % tc);
}

// float2 elements per group of 32 matrices: T, Z, X (n*n each), work (n).
__host__ __device__ __forceinline__ long long group_elems(int n) { return 3LL * n * n + n; }

// T-eigenvectors: column k of X solves (T(1:k-1,1:k-1) - T(k,k) I) x = -T(1:k-1,k)
// with the unit entry at k (the reference's ztrevc back substitution,
// Toolbox.hpp:1204-1262), zeros below; X(k,k) = s < 1 only where the overflow
// guard of trevc_solve had to scale the column.
template <class R, class MT>
__device__ void trevc_x_lane(const int n, const MT &T, typename vec2<R>::T *pX)
{
    const R ulp = lim<R>::eps();
    const R smlnum = lim<R>::tiny() * (R(n) / ulp);
    for (int ki = n; ki >= 1; --ki) {
        const VecIlv<R> xc{pX + (long long)(ki - 1) * n * 32};
        const cx<R> tkk = T.ld(ki, ki);
        const R smin = fmax(ulp * cabs1(tkk), smlnum);
        const R s = ki > 1 ? trevc_solve<R>(ki, T, xc, smin, tkk) : R(1);
        xc.st(ki, mk(s, R(0)));
        for (int i = ki + 1; i <= n; ++i) xc.st(i, mk(R(0), R(0)));
    }
}

__device__ __forceinline__ cx<double> up(cx<float> z) { return mk((double)z.r, (double)z.i); }
__device__ __forceinline__ cx<float> down(cx<double> z) { return mk((float)z.r, (float)z.i); }

__device__ __forceinline__ void to_fp64_list(const MixedArgs &a, int *flags, long long m)
{
    // the first pair (or the Schur kernel) to give up on matrix m puts it on the list
    if ((atomicOr(&flags[m], 2) & 2) == 0) a.fb_list[atomicAdd(a.fb_count, 1)] = (int)m;
}

__global__ void __launch_bounds__(kSchurThreads) schur32_kernel(const MixedArgs a, float2 *buf, int *flags)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long N = a.g.N;
    const int lane = threadIdx.x & 31;
    const long long warp = (long long)blockIdx.x * (kSchurThreads / 32) + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * (kSchurThreads / 32);
    const long long ngroups = (N + 31) / 32;
    const long long nn = (long long)n * n;
    for (long long g = warp; g < ngroups; g += nwarps) {
        float2 *pT = buf + g * group_elems(n) * 32 + lane;
        float2 *pZ = pT + 32 * nn, *pX = pZ + 32 * nn, *pW = pX + 32 * nn;
        const MatIlv<float> T{pT, n}, Z{pZ, n};
        const VecIlv<float> W{pW};
        const long long m = g * 32 + lane;
        const bool valid = m < N;
        int status = 0, sweeps = 0;
        bool fb = false;
        float nA2 = 0.f;
        if (valid) {
            const long long mo = soa_off_m(m, nn, tc);
            const MatSoA<double> A{const_cast<double *>(a.rA) + mo, const_cast<double *>(a.iA) + mo, tc, n};
            bool bad = false;
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) {
                    const cx<double> v = A.ld(i, j);
                    bad |= nonfinite(v.r) | nonfinite(v.i);
                    const cx<float> f = down(v);
                    nA2 = fma(f.i, f.i, fma(f.r, f.r, nA2));
                    T.st(i, j, f);
                }
            fb = bad || !(nA2 < 1e36f);  // beyond FP32 range: FP64
            zgehrd_lane<float>(n, T, W);
            zunghr_lane<float>(n, T, Z, W);
            clear_below_subdiag_lane<float>(n, T);
        }
        zlahqr_warp<float>(n, T, Z, valid && !fb, a.max_its, sweeps, status);
        if (status & ST_ITCAP) fb = true;
        if (valid) {
            if (!fb) trevc_x_lane<float>(n, T, pX);
            W.st(1, mk(nA2, 0.f));  // ||A||_F^2 for the refinement's tolerance
            flags[m] = fb ? 1 : 0;
            if (fb) to_fp64_list(a, flags, m);
            if (a.status) a.status[m] = status;
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
    }
}

// One eigenpair per lane.  MAXN bounds n (per-lane vectors live in local
// memory, indexed uniformly across the warp).
template <int MAXN>
__global__ void __launch_bounds__(kRefineThreads) refine_kernel(const MixedArgs a, const float2 *buf, int *flags)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long N = a.g.N;
    const long long p = (long long)blockIdx.x * kRefineThreads + threadIdx.x;
    const bool valid = p < N * n;
    const long long m = valid ? p / n : 0;
    const int k = valid ? (int)(p % n) + 1 : 1;
    bool act = valid && flags[m] == 0;
    if (!__any_sync(FULL, act)) return;

    const long long nn = (long long)n * n;
    float2 *pT = const_cast<float2 *>(buf) + (m / 32) * group_elems(n) * 32 + (m % 32);
    const MatIlv<float> T{pT, n}, Z{pT + 32 * nn, n}, X{pT + 64 * nn, n};
    const float nA2 = pT[96 * nn].x;
    const long long mo = soa_off_m(m, nn, tc);
    const MatSoA<double> A{const_cast<double *>(a.rA) + mo, const_cast<double *>(a.iA) + mo, tc, n};

    cx<double> v[MAXN];
    cx<float> r32[MAXN], dx[MAXN];
    cx<double> lam = mk(0.0, 0.0);
    if (act) {
        lam = up(T.ld(k, k));
        for (int i = 1; i <= n; ++i) {  // v = Z X(:,k), X upper triangular
            cx<float> acc = mk(0.f, 0.f);
            for (int j = 1; j <= k; ++j) acc = cmac(acc, Z.ld(i, j), X.ld(j, k));
            v[i - 1] = up(acc);
        }
    }
    const double tol2 = a.tol * a.tol;
    const float xkk = act ? X.ld(k, k).r : 1.f;
    bool fail = false;
    for (int step = 0; step <= a.max_steps; ++step) {
        if (!__any_sync(FULL, act)) break;
        if (!act) continue;
        // FP64 residual
        double rn2 = 0.0, vn2 = 0.0;
        for (int i = 1; i <= n; ++i) {
            const cx<double> vi = v[i - 1];
            cx<double> acc = mk(-(lam.r * vi.r - lam.i * vi.i), -(lam.r * vi.i + lam.i * vi.r));
            for (int j = 1; j <= n; ++j) acc = cmac(acc, A.ld(i, j), v[j - 1]);
            rn2 = fma(acc.i, acc.i, fma(acc.r, acc.r, rn2));
            vn2 = fma(vi.i, vi.i, fma(vi.r, vi.r, vn2));
            r32[i - 1] = down(acc);
        }
        if (rn2 <= tol2 * (double)nA2 * vn2) { act = false; continue; }
        if (step == a.max_steps) { fail = true; act = false; continue; }
        // FP32 correction through the Schur form: r' = Z^H r kept in dx
        for (int i = 1; i <= n; ++i) {
            cx<float> s = mk(0.f, 0.f);
            for (int j = 1; j <= n; ++j) s = cjmac(s, Z.ld(j, i), r32[j - 1]);
            dx[i - 1] = s;
        }
        const cx<float> l32 = down(lam);
        const float smin = fmax(lim<float>::eps() * cabs1(l32), lim<float>::tiny() * (float(n) / lim<float>::eps()));
        cx<float> dl = mk(0.f, 0.f);
        for (int i = n; i >= 1; --i) {
            cx<float> s = mk(-dx[i - 1].r, -dx[i - 1].i);
            for (int j = i + 1; j <= n; ++j) s = cnmac(s, T.ld(i, j), dx[j - 1]);
            if (i == k) {  // dlambda x_k = r'_k + sum_{j>k} T_kj dx_j = -s
                dl = cscal(mk(-s.r, -s.i), 1.f / xkk);
                dx[i - 1] = mk(0.f, 0.f);
                continue;
            }
            if (i < k) s = cmac(s, dl, X.ld(i, k));
            cx<float> d = csub(T.ld(i, i), l32);
            if (cabs1(d) < smin) d = mk(smin, 0.f);
            dx[i - 1] = cdiv(s, d);
        }
        for (int i = 1; i <= n; ++i) {
            cx<float> s = mk(0.f, 0.f);
            for (int j = 1; j <= n; ++j) s = cmac(s, Z.ld(i, j), dx[j - 1]);
            v[i - 1] = cadd(v[i - 1], up(s));
        }
        lam = cadd(lam, up(dl));
    }
    if (!valid || flags[m] != 0) return;
    if (fail) {
        to_fp64_list(a, flags, m);
        return;
    }
    const long long vo = soa_off_m(m, n, tc);
    const VecSoA<double> E{a.rE + vo, a.iE + vo, tc};
    E.st(k, lam);
    double scale = 1.0;
    if (a.vnorm == 1) {
        double mx = 0.0;
        for (int i = 0; i < n; ++i) mx = fmax(mx, cabs1(v[i]));
        scale = mx > 0.0 ? 1.0 / mx : 1.0;
    } else if (a.vnorm == 2) {
        double s2 = 0.0;
        for (int i = 0; i < n; ++i) s2 = fma(v[i].i, v[i].i, fma(v[i].r, v[i].r, s2));
        scale = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
    }
    const MatSoA<double> Vo{a.rV + mo, a.iV + mo, tc, n};
    for (int i = 1; i <= n; ++i) Vo.st(i, k, cscal(v[i - 1], scale));
}

int g_schur_blocks_per_sm = 8;

long long schur_blocks(long long N, int blocks_per_sm)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    static bool env_read = false;
    if (!env_read) {
        env_read = true;
        if (const char *e = getenv("VES_MIXED_BLOCKS_PER_SM")) {
            int v = atoi(e);
            if (v >= 1 && v <= 16) g_schur_blocks_per_sm = v;
        }
    }
    const long long groups = (N + 31) / 32;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : g_schur_blocks_per_sm;
    return std::max<long long>(1, std::min<long long>((groups + 3) / 4, (long long)sms * bps));
}

}  // namespace

size_t mixed_workspace_bytes(int n, long long N, int blocks_per_sm, int *out_blocks, int *out_threads)
{
    const long long groups = (N + 31) / 32;
    if (out_blocks) *out_blocks = (int)schur_blocks(N, blocks_per_sm);
    if (out_threads) *out_threads = kSchurThreads;
    const size_t bufb = (size_t)groups * group_elems(n) * 32 * sizeof(float2);
    const size_t flagb = ((size_t)N * sizeof(int) + 255) & ~(size_t)255;
    return bufb + flagb;
}

cudaError_t launch_mixed(const MixedArgs &a, cudaStream_t st)
{
    if (a.g.N <= 0) return cudaSuccess;
    const int n = a.g.n;
    if (n > 64) return cudaErrorInvalidValue;  // the refinement keeps per-pair vectors of at most 64 entries
    const long long groups = (a.g.N + 31) / 32;
    float2 *buf = static_cast<float2 *>(a.ws);
    int *flags = reinterpret_cast<int *>(static_cast<char *>(a.ws) +
                                         (size_t)groups * group_elems(n) * 32 * sizeof(float2));
    schur32_kernel<<<(unsigned)schur_blocks(a.g.N, a.blocks_per_sm), kSchurThreads, 0, st>>>(a, buf, flags);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long pairs = a.g.N * n;
    const unsigned rb = (unsigned)((pairs + kRefineThreads - 1) / kRefineThreads);
    if (n <= 16)
        refine_kernel<16><<<rb, kRefineThreads, 0, st>>>(a, buf, flags);
    else if (n <= 32)
        refine_kernel<32><<<rb, kRefineThreads, 0, st>>>(a, buf, flags);
    else
        refine_kernel<64><<<rb, kRefineThreads, 0, st>>>(a, buf, flags);
    return cudaGetLastError();
}

}  // namespace ves
