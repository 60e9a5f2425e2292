// ves_kernels.cu -- sm_103a kernels of the batched eigensolver.
//
// fused_fp64_kernel: the whole path of the reference's eigensolver()
// (utils.cpp:578-698: test_zgehrd -> copy -> test_zunghr -> zlahqr_new ->
// test_ztrevc, Toolbox.hpp:2150/2179/1984/2060) in one launch.  Each warp is
// persistent and takes groups of 32 consecutive matrices; lane l of a group
// owns matrix 32*g + l.  The input is read once from the SoA layout, the
// working H and Z live in a per-warp workspace laid out so that the 32 lanes'
// copies of one element are contiguous (one 512-byte access per warp), and
// eigenvalues / eigenvectors are written once.
//
// The stage kernels implement the reference's per-stage entry points
// (call_zgehrd, call_zunghr, hessenberg, call_zlahqr_new, call_ztrevc,
// call_zgemv, call_backsubstitution) in place on the SoA layout, one matrix
// per lane.
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace ves {

namespace {

constexpr int kFusedThreads = 128;  // 4 warps per block

// double2 elements per lane of one fused-kernel slot: H, Z (n^2 each), a work
// vector (n); the shift-seeded kernel adds an FP32 copy of H (n^2 float2 =
// ceil(n^2 / 2) double2), the n predictions and an FP32 vector (n float2).
__host__ __device__ __forceinline__ long long fused_slot_elems(int n, bool learned)
{
    const long long nn = (long long)n * n;
    return 2 * nn + n + (learned ? (nn + 1) / 2 + n + (n + 1) / 2 : 0);
}

__device__ __forceinline__ long long soa_mat_off(long long m, int n, int tc)
{
    return (m / tc) * (long long)tc * n * n + (m % tc);
}
__device__ __forceinline__ long long soa_vec_off(long long m, int n, int tc)
{
    return (m / tc) * (long long)tc * n + (m % tc);
}

// Eigenvector column scaling: 0 = as the reference leaves it (the T-eigenvector
// has a unit entry at position k), 1 = largest |re|+|im| equal to 1 (LAPACK
// ztrevc), 2 = unit 2-norm.
template <class R, class MZ>
__device__ __forceinline__ R vector_scale(const int n, const MZ &Z, const int j, const int vnorm)
{
    R scale = R(1);
    if (vnorm == 1) {
        R mx = R(0);
        for (int i = 1; i <= n; ++i) mx = fmax(mx, cabs1(Z.ld(i, j)));
        scale = mx > R(0) ? R(1) / mx : R(1);
    } else if (vnorm == 2) {
        R s2 = R(0);
        for (int i = 1; i <= n; ++i) { const cx<R> z = Z.ld(i, j); s2 += fma(z.r, z.r, z.i * z.i); }
        scale = s2 > R(0) ? R(1) / sqrt(s2) : R(1);
    }
    return scale;
}

template <class R, class MZ>
__device__ void write_vectors(const int n, const MZ &Z, const MatSoA<R> &V, const int vnorm)
{
    for (int j = 1; j <= n; ++j) {
        const R scale = vector_scale<R>(n, Z, j, vnorm);
        for (int i = 1; i <= n; ++i) V.st(i, j, cscal(Z.ld(i, j), scale));
    }
}

template <bool kLearned>
__global__ void __launch_bounds__(kFusedThreads) fused_fp64_kernel(const FusedArgs a)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long N = a.g.N;
    const int lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * (kFusedThreads / 32) + (threadIdx.x >> 5);
    const long long nslots = (long long)gridDim.x * (kFusedThreads / 32);
    const long long Nw = a.list ? (long long)*a.list_count - a.list_split : N;
    const long long ngroups = (Nw + 31) / 32;
    const long long per_lane = fused_slot_elems(n, kLearned);  // H, Z, work vector (+ FP32 H, predictions)

    double2 *base = reinterpret_cast<double2 *>(a.ws) + slot * per_lane * 32 + lane;
    const MatIlv<double> H{base, n};
    const MatIlv<double> Z{base + (long long)n * n * 32, n};
    const VecIlv<double> W{base + 2LL * n * n * 32};

    for (long long g = slot; g < ngroups; g += nslots) {
        const long long idx = g * 32 + lane;
        const bool valid = idx < Nw;
        const long long m = valid ? (a.list ? (long long)a.list[a.list_split + idx] : idx) : 0;
        const long long mo = valid ? soa_mat_off(m, n, tc) : 0;
        const long long vo = valid ? soa_vec_off(m, n, tc) : 0;
        int status = 0, sweeps = 0;
        double fro2 = 0.0;  // ||A||_F^2: scale of the learned-shift gate

        if (valid) {
            const MatSoA<double> A{const_cast<double *>(a.rA) + mo, const_cast<double *>(a.iA) + mo, tc, n};
            bool bad = false;
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) {
                    const cx<double> v = A.ld(i, j);
                    bad |= nonfinite(v.r) | nonfinite(v.i);
                    if (kLearned) fro2 = fma(v.i, v.i, fma(v.r, v.r, fro2));
                    H.st(i, j, v);
                }
            if (bad) status |= ST_NONFINITE;
            zgehrd_lane<double>(n, H, W);
            zunghr_lane<double>(n, H, Z, W);
            clear_below_subdiag_lane<double>(n, H);
        }
        ShiftPredictions sp{};
        if (kLearned) {
            // predictions into the slot, optionally polished on H in FP32
            const VecIlv<double> S{base + (2LL * n * n + n + ((long long)n * n + 1) / 2) * 32};
            const double scale = sqrt(fro2 / (double)n);
            if (valid) {
                for (int k = 1; k <= n; ++k)
                    S.st(k, mk(a.rS[vo + (long long)(k - 1) * tc], a.iS[vo + (long long)(k - 1) * tc]));
            }
            // FP32 copy of the Hessenberg matrix (for the in-kernel polish and the
            // FP64 step's derivative): lane l's element e at float2 index e * 32 + l
            // of the region after H, Z and the work vector
            float2 *region = reinterpret_cast<float2 *>(base - lane + (2LL * n * n + n) * 32);
            const MatIlv<float> Hf{region + lane, n};
            if ((a.shift_polish > 0 || a.shift_newton64) && valid && !(status & ST_NONFINITE))
                for (int j = 1; j <= n; ++j)
                    for (int i = 1; i <= (j + 1 < n ? j + 1 : n); ++i) {
                        const cx<double> h = H.ld(i, j);
                        Hf.st(i, j, mk((float)h.r, (float)h.i));
                    }
            if (a.shift_polish > 0) {
                const bool go = valid && !(status & ST_NONFINITE);
                // stop below 1e-6 of the eigenvalue scale (FP32 resolution); keep
                // a prediction whose last step was below 1e-3 of it
                const float tol = (float)(1e-6 * scale), keep = (float)(1e-3 * scale), dup = (float)(1e-5 * scale);
                if (go) {
                    if (n <= 16)
                        polish_shifts_lane<16>(n, Hf, S, a.shift_polish, tol, keep, dup);
                    else if (n <= 32)
                        polish_shifts_lane<32>(n, Hf, S, a.shift_polish, tol, keep, dup);
                    else
                        polish_shifts_lane<64>(n, Hf, S, a.shift_polish, tol, keep, dup);
                }
            }
            if (a.shift_newton64 && valid && !(status & ST_NONFINITE) && n >= 2) {
                // x in the work vector, x' (FP32) after the predictions
                float2 *dregion = reinterpret_cast<float2 *>(
                    base - lane + (2LL * n * n + n + ((long long)n * n + 1) / 2 + n) * 32);
                const VecIlv<float> DX{dregion + lane};
                for (int st = 0; st < a.shift_newton64; ++st) newton64_shifts_lane(n, H, Hf, S, W, DX, 1e-4 * scale);
            }
            sp.S = S;
            sp.n = n;
            sp.sweeps = a.shift_sweeps;
            sp.gate = (double)a.shift_gate * sqrt(fro2 / (double)n);
            sp.used = 0;
            sp.current = -1;
            sp.fallbacks = 0;
            zlahqr_warp<double, true>(n, H, Z, valid && !(status & ST_NONFINITE), a.max_its, sweeps, status, &sp);
            if (sp.fallbacks) status |= ST_SHIFT_FALLBACK;
        } else {
            zlahqr_warp<double>(n, H, Z, valid && !(status & ST_NONFINITE), a.max_its, sweeps, status);
        }
        if (valid) {
            if (kLearned && a.fallbacks) a.fallbacks[m] = sp.fallbacks;
            const VecSoA<double> E{a.rE + vo, a.iE + vo, tc};
            for (int k = 1; k <= n; ++k) E.st(k, H.ld(k, k));
            if (a.rT) {
                const MatSoA<double> T{a.rT + mo, a.iT + mo, tc, n};
                for (int j = 1; j <= n; ++j)
                    for (int i = 1; i <= n; ++i) T.st(i, j, i <= j ? H.ld(i, j) : mk(0.0, 0.0));
            }
            ztrevc_lane<double>(n, H, Z, W);
            const MatSoA<double> V{a.rV + mo, a.iV + mo, tc, n};
            write_vectors<double>(n, Z, V, a.vnorm);
            if (a.status) a.status[m] = status | (a.list ? ST_REFINE_FALLBACK : 0);
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
    }
}

// ---------------------------------------------------------------------------
// fp64_warp_kernel: the fused kernel's FP64 solve (no learned shifts) for
// n <= 64 with one matrix per warp, H, Z and the T-eigenvectors X in shared
// memory (197 KB at n = 64); for the few matrices on a device list (those the FP32+refine form
// hands back to FP64).  The lane kernel solves such a list in one or two
// lanes of one warp, and an FP64 warp instruction costs the same with one
// active lane as with 32: 11 ms at n = 16 and 72 ms at n = 32 on GB300 for
// one or two matrices.  Here lane l owns rows l + 1 and l + 33 of a column
// operation and the same columns of a row operation, and each
// element goes through the same operations in the same order as in the lane
// routines (zgehrd_lane, zunghr_lane, clear_below_subdiag_lane,
// make_subdiag_real_lane, zlahqr_warp, ztrevc_lane, write_vectors), the
// reflector norms summed sequentially as there: the results are the lane
// kernel's bit for bit.  Scalar steps run redundantly on every lane from
// shared values.  One warp per block.
// ---------------------------------------------------------------------------
struct SmemMat64 {
    double2 *p;
    int lda;
    __device__ __forceinline__ cx<double> ld(int i, int j) const
    {
        VES_CHECK_IJ(i, j, lda - 1);
        const double2 v = p[(i - 1) + (j - 1) * lda];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, int j, cx<double> v) const
    {
        VES_CHECK_IJ(i, j, lda - 1);
        p[(i - 1) + (j - 1) * lda] = make_double2(v.r, v.i);
    }
};
struct SmemCol64 {
    double2 *p;
    __device__ __forceinline__ cx<double> ld(int i) const
    {
        VES_CHECK_I(i);
        const double2 v = p[i - 1];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, cx<double> v) const
    {
        VES_CHECK_I(i);
        p[i - 1] = make_double2(v.r, v.i);
    }
};

// double2 elements of shared memory: H, Z, X (n (n + 1) each), tau, scales
__host__ __device__ __forceinline__ size_t fp64_warp_smem(int n) { return ((size_t)3 * n * (n + 1) + 2 * n) * sizeof(double2); }

__global__ void __launch_bounds__(32) fp64_warp_kernel(const FusedArgs a)
{
    extern __shared__ double2 fsm[];
    const int n = a.g.n, tc = a.g.tc;
    const int lane = threadIdx.x;  // owns rows / columns lane + 1 and lane + 33 (n <= 64)
    const int lda = n + 1;
    const SmemMat64 H{fsm, lda}, Z{fsm + n * lda, lda}, X{fsm + 2 * n * lda, lda};
    double2 *sTau = fsm + 3 * n * lda, *sS = sTau + n;
    const double ulp = lim<double>::eps();
    const double smlnum = lim<double>::tiny() * ((double)n / ulp);
    const long long count = a.list ? (long long)min(*a.list_count, (int)a.list_split) : a.g.N;

    for (long long w = blockIdx.x; w < count; w += gridDim.x) {
        const long long m = a.list ? (long long)a.list[w] : w;
        const long long mo = soa_mat_off(m, n, tc), vo = soa_vec_off(m, n, tc);
        int status = 0, sweeps = 0;
        bool bad = false;
        for (int e = lane; e < n * n; e += 32) {
            const long long k = mo + (long long)e * tc;
            const double re = a.rA[k], im = a.iA[k];
            bad |= nonfinite(re) | nonfinite(im);
            H.st(e % n + 1, e / n + 1, mk(re, im));
        }
        if (__any_sync(FULL, bad)) status |= ST_NONFINITE;
        __syncwarp();

        // ---- zgehrd (zgehd2): reflector i from column i, applied right then left
        for (int i = 1; i <= n - 1; ++i) {
            const int mm = n - i;
            const cx<double> alpha = H.ld(i + 1, i);
            double xnorm2 = 0.0;
            for (int k = i + 2; k <= n; ++k) {
                const cx<double> x = H.ld(k, i);
                xnorm2 = fma(x.i, x.i, fma(x.r, x.r, xnorm2));
            }
            const bool trivial = (xnorm2 == 0.0) && (alpha.i == 0.0);
            const double beta = trivial ? alpha.r : -copysign(sqrt(fma(alpha.r, alpha.r, fma(alpha.i, alpha.i, xnorm2))), alpha.r);
            cx<double> t = mk(0.0, 0.0), scale = mk(0.0, 0.0);
            if (!trivial) {
                const double rb = 1.0 / beta;
                t = mk((beta - alpha.r) * rb, -alpha.i * rb);
                scale = cinv(mk(alpha.r - beta, alpha.i));
            }
            __syncwarp();  // every lane has read column i
            for (int j = lane + 1; j <= n; j += 32) if (j >= i + 2 && j <= n) H.st(j, i, cmul(H.ld(j, i), scale));
            if (lane == 0) sTau[i - 1] = make_double2(t.r, t.i);
            __syncwarp();
            for (int j = lane + 1; j <= n; j += 32) if (j <= n) {  // right: row j of A(1:n, i+1:n) -= tau (A v)_j v^H
                cx<double> sacc = H.ld(j, i + 1);
                for (int q = 2; q <= mm; ++q) sacc = cmac(sacc, H.ld(j, i + q), H.ld(i + q, i));
                const cx<double> ts = cmul(t, sacc);
                H.st(j, i + 1, csub(H.ld(j, i + 1), ts));
                for (int q = 2; q <= mm; ++q) H.st(j, i + q, cnmacc(H.ld(j, i + q), ts, H.ld(i + q, i)));
            }
            __syncwarp();
            for (int j = lane + 1; j <= n; j += 32) if (j >= i + 1 && j <= n) {  // left: column j of A(i+1:n, i+1:n) -= conj(tau) v (v^H A)_j
                const cx<double> tcj = conj(t);
                cx<double> sacc = H.ld(i + 1, j);
                for (int q = 2; q <= mm; ++q) sacc = cjmac(sacc, H.ld(i + q, i), H.ld(i + q, j));
                const cx<double> ts = cmul(tcj, sacc);
                H.st(i + 1, j, csub(H.ld(i + 1, j), ts));
                for (int q = 2; q <= mm; ++q) H.st(i + q, j, cnmac(H.ld(i + q, j), H.ld(i + q, i), ts));
            }
            __syncwarp();
            if (lane == 0) H.st(i + 1, i, mk(beta, 0.0));
            __syncwarp();
        }
        // ---- zunghr (zung2r): Z = Q, last reflector first
        for (int i = n - 1; i >= 1; --i) {
            const cx<double> t = mk(sTau[i - 1].x, sTau[i - 1].y);
            const int c = i + 1;
            for (int j = lane + 1; j <= n; j += 32) if (j >= c + 1 && j <= n) {
                cx<double> sacc = Z.ld(c, j);
                for (int k = c + 1; k <= n; ++k) sacc = cjmac(sacc, H.ld(k, i), Z.ld(k, j));
                const cx<double> ts = cmul(t, sacc);
                Z.st(c, j, csub(Z.ld(c, j), ts));
                for (int k = c + 1; k <= n; ++k) Z.st(k, j, cnmac(Z.ld(k, j), H.ld(k, i), ts));
            }
            __syncwarp();
            const cx<double> mt = mk(-t.r, -t.i);
            for (int j = lane + 1; j <= n; j += 32) if (j >= c + 1 && j <= n) Z.st(j, c, cmul(H.ld(j, i), mt));
            for (int j = lane + 1; j <= n; j += 32) if (j == c) Z.st(c, c, mk(1.0 - t.r, -t.i));
            for (int j = lane + 1; j <= n; j += 32) if (j >= 2 && j <= c - 1) Z.st(j, c, mk(0.0, 0.0));
            __syncwarp();
        }
        for (int j = lane + 1; j <= n; j += 32) if (j <= n) {
            Z.st(j, 1, mk(j == 1 ? 1.0 : 0.0, 0.0));
            if (j > 1) Z.st(1, j, mk(0.0, 0.0));
        }
        for (int j = lane + 1; j <= n; j += 32) if (j <= n)  // clear below the subdiagonal
            for (int k = j + 2; k <= n; ++k) H.st(k, j, mk(0.0, 0.0));
        __syncwarp();

        if (!(status & ST_NONFINITE)) {
            // ---- make the subdiagonal real
            for (int i = 2; i <= n; ++i) {
                const cx<double> h = H.ld(i, i - 1);
                if (h.i != 0.0) {
                    cx<double> sc = cscal(h, 1.0 / cabs1(h));
                    sc = cscal(conj(sc), 1.0 / cabs(sc));
                    __syncwarp();
                    if (lane == 0) H.st(i, i - 1, mk(cabs(h), 0.0));
                    for (int j = lane + 1; j <= n; j += 32) if (j >= i && j <= n) H.st(i, j, cmul(H.ld(i, j), sc));
                    __syncwarp();
                    const int re = (i + 1) < n ? (i + 1) : n;
                    for (int j = lane + 1; j <= n; j += 32) if (j <= re) H.st(j, i, cmulc(H.ld(j, i), sc));
                    for (int j = lane + 1; j <= n; j += 32) if (j <= n) Z.st(j, i, cmulc(Z.ld(j, i), sc));
                }
                __syncwarp();
            }
            // ---- single-shift QR
            int I = n, L = 1, its = 0;
            while (I > 1) {
                if (its > a.max_its) { status |= ST_ITCAP; --I; L = 1; its = 0; continue; }
                L = deflation_scan<double>(I, L, H, n, ulp, smlnum);
                __syncwarp();
                if (L > 1 && lane == 0) H.st(L, L - 1, mk(0.0, 0.0));
                __syncwarp();
                if (L >= I) { --I; L = 1; its = 0; continue; }
                const cx<double> t = qr_shift<double>(I, L, its, H);
                const cx<double> h11s = csub(H.ld(L, L), t);
                const double h21 = H.ld(L + 1, L).r;
                const double rs = 1.0 / (cabs1(h11s) + fabs(h21));
                const cx<double> v0 = cscal(h11s, rs), v1 = mk(h21 * rs, 0.0);
                ++its;
                ++sweeps;
                for (int K = L; K <= I - 1; ++K) {
                    cx<double> a0 = v0, a1 = v1, t1;
                    if (K > L) { a0 = H.ld(K, K - 1); a1 = H.ld(K + 1, K - 1); }
                    zlarfg2<double>(a0, a1, t1);
                    __syncwarp();
                    if (K > L && lane == 0) { H.st(K, K - 1, a0); H.st(K + 1, K - 1, mk(0.0, 0.0)); }
                    const cx<double> w1 = a1, c1 = conj(t1), cw = conj(w1);
                    const double t2 = fma(t1.r, w1.r, -(t1.i * w1.i));
                    for (int j = lane + 1; j <= n; j += 32) if (j <= n) {  // Schur vectors: row j of columns K, K+1; H: rows K, K+1 of column j >= K
                        cx<double> z1 = Z.ld(j, K), z2 = Z.ld(j, K + 1);
                        rot_pair(z1, z2, t1, t2, cw);
                        Z.st(j, K, z1);
                        Z.st(j, K + 1, z2);
                        if (j >= K) {
                            cx<double> h1 = H.ld(K, j), h2 = H.ld(K + 1, j);
                            rot_pair(h1, h2, c1, t2, w1);
                            H.st(K, j, h1);
                            H.st(K + 1, j, h2);
                        }
                    }
                    __syncwarp();
                    const int je = (K + 2) < I ? (K + 2) : I;
                    for (int j = lane + 1; j <= n; j += 32) if (j <= je) {  // columns K, K+1, row j
                        cx<double> h1 = H.ld(j, K), h2 = H.ld(j, K + 1);
                        rot_pair(h1, h2, t1, t2, cw);
                        H.st(j, K, h1);
                        H.st(j, K + 1, h2);
                    }
                    __syncwarp();
                }
                // make H(I, I-1) real
                const cx<double> h = H.ld(I, I - 1);
                if (h.i != 0.0) {
                    const double d = cabs(h);
                    const cx<double> z = conj(cscal(h, 1.0 / d));
                    __syncwarp();
                    if (lane == 0) H.st(I, I - 1, mk(d, 0.0));
                    for (int j = lane + 1; j <= n; j += 32) if (j >= I + 1 && j <= n) H.st(I, j, cmul(H.ld(I, j), z));
                    for (int j = lane + 1; j <= n; j += 32) if (j <= I - 1) H.st(j, I, cmulc(H.ld(j, I), z));
                    for (int j = lane + 1; j <= n; j += 32) if (j <= n) Z.st(j, I, cmulc(Z.ld(j, I), z));
                }
                __syncwarp();
            }
        }

        // ---- eigenvalues, Schur form, eigenvectors
        const VecSoA<double> E{a.rE + vo, a.iE + vo, a.g.tc};
        for (int j = lane + 1; j <= n; j += 32) if (j <= n) E.st(j, H.ld(j, j));
        if (a.rT) {
            const MatSoA<double> T{a.rT + mo, a.iT + mo, tc, n};
            for (int j = lane + 1; j <= n; j += 32) if (j <= n)
                for (int i = 1; i <= n; ++i) T.st(i, j, i <= j ? H.ld(i, j) : mk(0.0, 0.0));
        }
        for (int j = lane + 1; j <= n; j += 32) if (j >= 2 && j <= n) {  // T-eigenvector j (back substitution) into column j of X
            const cx<double> tkk = H.ld(j, j);
            const double smin = fmax(ulp * cabs1(tkk), smlnum);
            const double s = trevc_solve<double>(j, H, SmemCol64{fsm + 2 * n * lda + (j - 1) * lda}, smin, tkk);
            sS[j - 1] = make_double2(s, 0.0);
        }
        __syncwarp();
        for (int j = lane + 1; j <= n; j += 32) if (j <= n) {  // row j of Z := Z [x; s; 0], columns n down to 2 (Z(j, 1:ki-1) still Q's)
            for (int ki = n; ki >= 2; --ki) {
                cx<double> acc = Z.ld(j, ki);
                const double s = sS[ki - 1].x;
                if (s != 1.0) acc = cscal(acc, s);
                for (int q = 1; q <= ki - 1; ++q) acc = cmac(acc, Z.ld(j, q), X.ld(q, ki));
                Z.st(j, ki, acc);
            }
        }
        __syncwarp();
        for (int j = lane + 1; j <= n; j += 32) if (j <= n) {
            const MatSoA<double> V{a.rV + mo, a.iV + mo, tc, n};
            const double scale = vector_scale<double>(n, Z, j, a.vnorm);
            for (int i = 1; i <= n; ++i) V.st(i, j, cscal(Z.ld(i, j), scale));
        }
        if (lane == 0) {
            if (a.status) a.status[m] = status | (a.list ? ST_REFINE_FALLBACK : 0);
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Learned-shift polish pre-pass for n <= 32: one matrix per warp in shared
// memory, FP32.  The warp reduces its matrix to Hessenberg form (hess32_warp;
// FP32 rounding moves the eigenvalues by ~1e-7 relative, far below what the
// shifts need), then lane k takes prediction k through up to `steps` steps on
// det(H - sI): the Newton correction by Hyman's recurrence (as in
// polish_shifts_lane, with every lane's x and x' in shared memory and H read
// as broadcasts), turned into Aberth's correction with the other lanes'
// current predictions (all lanes step together, Jacobi order; `aberth` = 0
// keeps plain Newton).  A prediction is kept only if its last step was below
// 1e-3 of the eigenvalue scale ||A||_F / sqrt(n) and no lower lane landed
// within 1e-5 of it; dropped predictions are NaN.  Output: rP, iP in the SoA
// vector layout.
// ---------------------------------------------------------------------------
constexpr int kPolishThreads = 128;  // 4 matrices per block

__host__ __device__ __forceinline__ size_t polish_warp_elems(int n)
{
    return (size_t)n * (n + 1) + n + 2 * (size_t)n * 32;  // H, tau, x and x' of 32 lanes
}

__global__ void __launch_bounds__(kPolishThreads) polish32_warp_kernel(const Geom g, const double *rA,
                                                                       const double *iA, const double *rS,
                                                                       const double *iS, double *rP, double *iP,
                                                                       int steps, int aberth,
                                                                       unsigned long long *work)
{
    extern __shared__ float2 psm[];
    const int n = g.n, tc = g.tc;
    const long long N = g.N;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int lda = n + 1;
    float2 *sH = psm + (size_t)wib * polish_warp_elems(n);
    float2 *sTau = sH + n * lda, *xs = sTau + n, *dxs = xs + n * 32;
    const SmemMat H{sH, lda};
    const long long nn = (long long)n * n;
    const long long gw = (long long)blockIdx.x * (kPolishThreads / 32) + wib;
    const long long nw = (long long)gridDim.x * (kPolishThreads / 32);
    const float nanf_ = __int_as_float(0x7fc00000);
    for (long long m = gw; m < N; m += nw) {
        const long long mo = soa_mat_off(m, n, tc), vo = soa_vec_off(m, n, tc);
        bool bad = false;
        float s2 = 0.f;
        for (int e = lane; e < nn; e += 32) {
            const long long q = mo + (long long)e * tc;
            const double re = rA[q], im = iA[q];
            bad |= nonfinite(re) | nonfinite(im);
            const float fr = (float)re, fi = (float)im;
            s2 = fmaf(fi, fi, fmaf(fr, fr, s2));
            sH[(e % n) + (e / n) * lda] = make_float2(fr, fi);
        }
        const float nA2 = warp_sum(s2);
        const bool skip = __any_sync(FULL, bad) || !(nA2 < 1e36f) || n < 2;
        cx<float> s = mk(0.f, 0.f);
        if (lane < n) s = mk((float)rS[vo + (long long)lane * tc], (float)iS[vo + (long long)lane * tc]);
        __syncwarp();
        if (skip) {  // leave such matrices to the solver's own checks, predictions as given
            if (lane < n) { rP[vo + (long long)lane * tc] = s.r; iP[vo + (long long)lane * tc] = s.i; }
            continue;
        }
        hess32_warp(n, H, sTau, lane);
        const float scale = sqrtf(nA2 / (float)n);
        const float tol = 1e-6f * scale, keep = 1e-3f * scale, dup = 1e-5f * scale;
        bool ok = lane < n && !nonfinite(s.r) && !nonfinite(s.i);
        float last = 3.0e38f;
        int nsteps = 0;  // Newton steps this lane's prediction took (work counter)
        for (int it = 0; it < steps; ++it) {
            const bool act = ok && last > tol;
            if (!__any_sync(FULL, act)) break;
            nsteps += act;
            xs[(n - 1) * 32 + lane] = make_float2(1.f, 0.f);
            dxs[(n - 1) * 32 + lane] = make_float2(0.f, 0.f);
            bool broke = false;
            for (int i = n; i >= 2; --i) {
                const cx<float> d = csub(H.ld(i, i), s);
                const float2 xi = xs[(i - 1) * 32 + lane], dxi = dxs[(i - 1) * 32 + lane];
                cx<float> acc = cmul(d, mk(xi.x, xi.y));
                cx<float> dacc = csub(cmul(d, mk(dxi.x, dxi.y)), mk(xi.x, xi.y));
                for (int q = i + 1; q <= n; ++q) {
                    const cx<float> h = H.ld(i, q);
                    const float2 xq = xs[(q - 1) * 32 + lane], dxq = dxs[(q - 1) * 32 + lane];
                    acc = cmac(acc, h, mk(xq.x, xq.y));
                    dacc = cmac(dacc, h, mk(dxq.x, dxq.y));
                }
                const cx<float> sub = H.ld(i, i - 1);
                if (sub.r == 0.f && sub.i == 0.f) { broke = true; break; }  // uniform: H is shared
                cx<float> xn = cdiv(mk(-acc.r, -acc.i), sub), dxn = cdiv(mk(-dacc.r, -dacc.i), sub);
                if (cabs1(xn) > 1e18f) {  // rescale x, x' together (the Newton ratio is scale free)
                    for (int q = i; q <= n; ++q) {
                        const float2 a0 = xs[(q - 1) * 32 + lane], a1 = dxs[(q - 1) * 32 + lane];
                        xs[(q - 1) * 32 + lane] = make_float2(a0.x * 1e-18f, a0.y * 1e-18f);
                        dxs[(q - 1) * 32 + lane] = make_float2(a1.x * 1e-18f, a1.y * 1e-18f);
                    }
                    xn = cscal(xn, 1e-18f);
                    dxn = cscal(dxn, 1e-18f);
                }
                xs[(i - 2) * 32 + lane] = make_float2(xn.r, xn.i);
                dxs[(i - 2) * 32 + lane] = make_float2(dxn.r, dxn.i);
            }
            if (broke) { ok = false; break; }
            const cx<float> d1 = csub(H.ld(1, 1), s);
            const float2 x1 = xs[lane], dx1 = dxs[lane];
            cx<float> r = cmul(d1, mk(x1.x, x1.y));
            cx<float> rp = csub(cmul(d1, mk(dx1.x, dx1.y)), mk(x1.x, x1.y));
            for (int q = 2; q <= n; ++q) {
                const cx<float> h = H.ld(1, q);
                const float2 xq = xs[(q - 1) * 32 + lane], dxq = dxs[(q - 1) * 32 + lane];
                r = cmac(r, h, mk(xq.x, xq.y));
                rp = cmac(rp, h, mk(dxq.x, dxq.y));
            }
            cx<float> delta = act ? cdiv(r, rp) : mk(0.f, 0.f);
            if (aberth) {
                // w = sum over the other live approximations s_q of 1 / (s - s_q),
                // taken before any lane moves (all lanes step together)
                const unsigned live = __ballot_sync(FULL, ok);
                cx<float> w = mk(0.f, 0.f);
                for (int q = 0; q < n; ++q) {
                    const float qr = __shfl_sync(FULL, s.r, q), qi = __shfl_sync(FULL, s.i, q);
                    const cx<float> d = mk(s.r - qr, s.i - qi);
                    if (q != lane && ((live >> q) & 1u) && (d.r != 0.f || d.i != 0.f)) w = cadd(w, cinv(d));
                }
                // Aberth-Ehrlich: the Newton step on p(s) / prod_q (s - s_q)
                const cx<float> ab = cdiv(delta, csub(mk(1.f, 0.f), cmul(delta, w)));
                if (act && !nonfinite(ab.r) && !nonfinite(ab.i)) delta = ab;
            }
            if (act) {
                if (nonfinite(delta.r) || nonfinite(delta.i)) {
                    ok = false;
                } else {
                    s = csub(s, delta);
                    last = cabs1(delta);
                }
            }
        }
        cx<float> res = ok && last <= keep ? s : mk(nanf_, nanf_);
        // drop a prediction that a lower lane also converged to
        bool dupl = false;
        for (int q = 0; q < n; ++q) {
            const float orr = __shfl_sync(FULL, res.r, q), oi = __shfl_sync(FULL, res.i, q);
            if (q < lane && orr == orr && fabsf(orr - res.r) + fabsf(oi - res.i) <= dup) dupl = true;
        }
        if (dupl) res = mk(nanf_, nanf_);
        if (lane < n) {
            rP[vo + (long long)lane * tc] = res.r;
            iP[vo + (long long)lane * tc] = res.i;
        }
        if (work) {
            const int tot = __reduce_add_sync(FULL, nsteps);
            if (lane == 0 && tot) atomicAdd(work + WORK_POLISH, (unsigned long long)tot);
        }
        __syncwarp();
    }
}

size_t polish_smem_bytes(int n) { return (kPolishThreads / 32) * polish_warp_elems(n) * sizeof(float2); }

// ---------------------------------------------------------------------------
// Stage kernels: one lane per matrix, in place on the SoA layout.
// ---------------------------------------------------------------------------
struct Lane {
    long long m;
    bool valid;
    long long mo, vo;
};
__device__ __forceinline__ Lane lane_of(const Geom &g)
{
    Lane l;
    l.m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    l.valid = l.m < g.N;
    l.mo = l.valid ? soa_mat_off(l.m, g.n, g.tc) : 0;
    l.vo = l.valid ? soa_vec_off(l.m, g.n, g.tc) : 0;
    return l;
}

__global__ void zgehrd_kernel(const Geom g, double *rA, double *iA, double *rtau, double *itau)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> A{rA + l.mo, iA + l.mo, g.tc, g.n};
    const VecSoA<double> tau{rtau + l.vo, itau + l.vo, g.tc};
    zgehrd_lane<double>(g.n, A, tau);
}

__global__ void zunghr_kernel(const Geom g, double *rA, double *iA, const double *rtau, const double *itau)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> A{rA + l.mo, iA + l.mo, g.tc, g.n};
    const VecSoA<double> tau{const_cast<double *>(rtau) + l.vo, const_cast<double *>(itau) + l.vo, g.tc};
    zunghr_lane<double>(g.n, A, A, tau);
}

// hessenberg(): A -> H (reflectors below the subdiagonal, as the reference
// leaves them), Q formed in a separate matrix.
__global__ void hessenberg_kernel(const Geom g, double *rA, double *iA, double *rQ, double *iQ, double *rtau,
                                  double *itau)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> A{rA + l.mo, iA + l.mo, g.tc, g.n};
    const MatSoA<double> Q{rQ + l.mo, iQ + l.mo, g.tc, g.n};
    const VecSoA<double> tau{rtau + l.vo, itau + l.vo, g.tc};
    zgehrd_lane<double>(g.n, A, tau);
    zunghr_lane<double>(g.n, A, Q, tau);
}

// call_zlahqr_new(): Z := I, H (cleared below the subdiagonal) -> T, E = diag(T).
__global__ void zlahqr_kernel(const Geom g, double *rE, double *iE, double *rH, double *iH, double *rZ, double *iZ,
                              int *status_out, int max_its)
{
    const Lane l = lane_of(g);
    const MatSoA<double> H{rH + l.mo, iH + l.mo, g.tc, g.n};
    const MatSoA<double> Z{rZ + l.mo, iZ + l.mo, g.tc, g.n};
    int status = 0, sweeps = 0;
    if (l.valid) {
        set_identity_lane<double>(g.n, Z);
        clear_below_subdiag_lane<double>(g.n, H);
    }
    zlahqr_warp<double>(g.n, H, Z, l.valid, max_its, sweeps, status);
    if (l.valid) {
        const VecSoA<double> E{rE + l.vo, iE + l.vo, g.tc};
        for (int k = 1; k <= g.n; ++k) E.st(k, H.ld(k, k));
        if (status_out) status_out[l.m] = status;
    }
}

__global__ void ztrevc_kernel(const Geom g, double *rT, double *iT, double *rR, double *iR, double *rw, double *iw)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> T{rT + l.mo, iT + l.mo, g.tc, g.n};
    const MatSoA<double> Rm{rR + l.mo, iR + l.mo, g.tc, g.n};
    const VecSoA<double> x{rw + l.vo, iw + l.vo, g.tc};
    ztrevc_lane<double>(g.n, T, Rm, x);
}

__global__ void zgemv_kernel(const Geom g, bool herm, const double *rA, const double *iA, const double *rx,
                             const double *ix, double rbeta, double ibeta, double *ry, double *iy)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> A{const_cast<double *>(rA) + l.mo, const_cast<double *>(iA) + l.mo, g.tc, g.n};
    const VecSoA<double> x{const_cast<double *>(rx) + l.vo, const_cast<double *>(ix) + l.vo, g.tc};
    const VecSoA<double> y{ry + l.vo, iy + l.vo, g.tc};
    zgemv_lane<double>(herm, g.n, A, x, mk(rbeta, ibeta), y);
}

__global__ void backsubs_kernel(const Geom g, const double *rT, const double *iT, double *rx, double *ix)
{
    const Lane l = lane_of(g);
    if (!l.valid) return;
    const MatSoA<double> T{const_cast<double *>(rT) + l.mo, const_cast<double *>(iT) + l.mo, g.tc, g.n};
    const VecSoA<double> x{rx + l.vo, ix + l.vo, g.tc};
    backsubs_lane<double>(g.n, T, x);
}


// FMA throughput probes: the roofline denominators of the FP64-bound solver
// and of the FP32 stages of the mixed-precision form (measured figures, as
// the HBM and tensor peaks are).  Eight independent dependent-FMA chains per
// thread.
template <class R>
__global__ void fma_probe_kernel(R *out, int iters, R b, R c)
{
    R a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

constexpr int kStageThreads = 128;
inline unsigned stage_blocks(const Geom &g) { return (unsigned)((g.N + kStageThreads - 1) / kStageThreads); }

// Blocks (4 warps) per SM of the persistent FP64 grid when the caller leaves
// it to the library; VES_FUSED_BLOCKS_PER_SM overrides.  Measured on GB300
// (eigensolves/s, 2 -> 3 -> 4 -> 5 blocks): n=8 8.88 9.07 9.19 9.30 M/s,
// n=16 1.588 1.651 1.656 1.637 M/s, n=24 0.520 0.565 0.549 0.546 M/s,
// n=32 0.230 0.248 0.251 0.232 M/s, n=48 0.063 0.060 0.068 0.068 M/s.
int fused_default_bps(int n)
{
    if (const char *e = getenv("VES_FUSED_BLOCKS_PER_SM")) {
        const int v = atoi(e);
        if (v >= 1 && v <= 16) return v;
    }
    return (n >= 21 && n <= 28) ? 3 : 4;
}

int device_sms()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

}  // namespace

size_t fused_workspace_bytes(int n, long long N, int blocks_per_sm, int *out_blocks, int *out_threads, bool learned)
{
    const int sms = device_sms();
    const long long groups = (N + 31) / 32;
    const int wpb = kFusedThreads / 32;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : fused_default_bps(n);
    long long blocks = std::min<long long>((groups + wpb - 1) / wpb, (long long)sms * bps);
    if (blocks < 1) blocks = 1;
    const size_t per_slot = (size_t)fused_slot_elems(n, learned) * 32 * sizeof(double2);
    if (out_blocks) *out_blocks = (int)blocks;
    if (out_threads) *out_threads = kFusedThreads;
    return per_slot * (size_t)blocks * wpb;
}

cudaError_t launch_fused_fp64(const FusedArgs &a, cudaStream_t st)
{
    if (a.g.N <= 0) return cudaSuccess;
    int blocks = 0, threads = 0;
    fused_workspace_bytes(a.g.n, a.g.N, a.blocks_per_sm, &blocks, &threads, a.rS != nullptr);
    if (a.rS)
        fused_fp64_kernel<true><<<blocks, threads, 0, st>>>(a);
    else
        fused_fp64_kernel<false><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_polish32(Geom g, const double *rA, const double *iA, const double *rS, const double *iS,
                            double *rP, double *iP, int steps, unsigned long long *work, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    if (g.n > 32) return cudaErrorInvalidValue;
    // per call (per device, thread safe; microseconds next to the kernel)
    cudaError_t e = cudaFuncSetAttribute(polish32_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)polish_smem_bytes(32));
    if (e != cudaSuccess) return e;
    const int sms = device_sms();
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, polish32_warp_kernel, kPolishThreads,
                                                  polish_smem_bytes(g.n));
    const long long need = (g.N + kPolishThreads / 32 - 1) / (kPolishThreads / 32);
    const long long blocks = std::max<long long>(1, std::min<long long>(need, (long long)sms * std::max(per_sm, 1)));
    // simultaneous (Aberth-Ehrlich) iteration by default; VES_POLISH_METHOD=newton
    // polishes each prediction on its own (read per launch: cheap next to a solve)
    const char *pm = getenv("VES_POLISH_METHOD");
    const int aberth = (pm && strcmp(pm, "newton") == 0) ? 0 : 1;
    polish32_warp_kernel<<<(unsigned)blocks, kPolishThreads, polish_smem_bytes(g.n), st>>>(g, rA, iA, rS, iS, rP,
                                                                                         iP, steps, aberth, work);
    return cudaGetLastError();
}

cudaError_t launch_fp64_list(FusedArgs a, cudaStream_t st)
{
    if (a.g.N <= 0) return cudaSuccess;
    a.list_split = 0;
    if (a.list && !a.rS && a.g.n <= 64) {
        // per call (per device, thread safe; microseconds next to the kernel)
        cudaError_t e = cudaFuncSetAttribute(fp64_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)fp64_warp_smem(64));
        if (e != cudaSuccess) return e;
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_warp_kernel, 32, fp64_warp_smem(a.g.n));
        const long long slots = (long long)device_sms() * std::max(per_sm, 1);
        a.list_split = std::min<long long>(a.g.N, slots);
        fp64_warp_kernel<<<(unsigned)a.list_split, 32, fp64_warp_smem(a.g.n), st>>>(a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_fused_fp64(a, st);
}

cudaError_t launch_fused_fp64_blocks(const FusedArgs &a, int blocks, cudaStream_t st)
{
    if (a.g.N <= 0) return cudaSuccess;
    fused_fp64_kernel<false><<<blocks, kFusedThreads, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_zgehrd(Geom g, double *rA, double *iA, double *rtau, double *itau, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    zgehrd_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rA, iA, rtau, itau);
    return cudaGetLastError();
}

cudaError_t launch_zunghr(Geom g, double *rA, double *iA, const double *rtau, const double *itau, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    zunghr_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rA, iA, rtau, itau);
    return cudaGetLastError();
}

cudaError_t launch_hessenberg(Geom g, double *rA, double *iA, double *rQ, double *iQ, double *rtau, double *itau,
                              cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    hessenberg_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rA, iA, rQ, iQ, rtau, itau);
    return cudaGetLastError();
}

cudaError_t launch_zlahqr(Geom g, double *rE, double *iE, double *rH, double *iH, double *rZ, double *iZ,
                          int *status, int max_its, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    zlahqr_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rE, iE, rH, iH, rZ, iZ, status, max_its);
    return cudaGetLastError();
}

cudaError_t launch_ztrevc(Geom g, double *rT, double *iT, double *rR, double *iR, double *rw, double *iw,
                          cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    ztrevc_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rT, iT, rR, iR, rw, iw);
    return cudaGetLastError();
}

cudaError_t launch_zgemv(Geom g, bool herm, const double *rA, const double *iA, const double *rx, const double *ix,
                         double rbeta, double ibeta, double *ry, double *iy, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    zgemv_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, herm, rA, iA, rx, ix, rbeta, ibeta, ry, iy);
    return cudaGetLastError();
}

cudaError_t launch_backsubs(Geom g, const double *rT, const double *iT, double *rx, double *ix, cudaStream_t st)
{
    if (g.N <= 0) return cudaSuccess;
    backsubs_kernel<<<stage_blocks(g), kStageThreads, 0, st>>>(g, rT, iT, rx, ix);
    return cudaGetLastError();
}

// threads per SM: 8 warps keep the FP64 pipe full; the FP32 pipe (about 58x
// the FP64 rate) needs 32 warps of independent chains
template <class R>
cudaError_t fma_rate(double *flops_per_s, cudaStream_t st, int threads, int iters)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    R *out = nullptr;
    cudaError_t e = cudaMallocAsync(&out, (size_t)sms * threads * sizeof(R), st);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const R b = R(1.0000001), c = R(1e-9);
    fma_probe_kernel<R><<<sms, threads, 0, st>>>(out, iters, b, c);  // warm-up
    cudaEventRecord(e0, st);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) fma_probe_kernel<R><<<sms, threads, 0, st>>>(out, iters, b, c);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    *flops_per_s = 2.0 * 8.0 * iters * (double)sms * threads * reps / (ms * 1e-3);
    return e;
}

cudaError_t fp64_fma_rate(double *flops_per_s, cudaStream_t st) { return fma_rate<double>(flops_per_s, st, 256, 4096); }
cudaError_t fp32_fma_rate(double *flops_per_s, cudaStream_t st) { return fma_rate<float>(flops_per_s, st, 1024, 16384); }

void load_fused_kernels()
{
    load_kernel(fused_fp64_kernel<false>);
    load_kernel(fused_fp64_kernel<true>);
    load_kernel(fp64_warp_kernel);
    load_kernel(polish32_warp_kernel);
    load_kernel(zgehrd_kernel);
    load_kernel(zunghr_kernel);
    load_kernel(hessenberg_kernel);
    load_kernel(zlahqr_kernel);
    load_kernel(ztrevc_kernel);
    load_kernel(zgemv_kernel);
    load_kernel(backsubs_kernel);
    load_kernel(fma_probe_kernel<double>);
    load_kernel(fma_probe_kernel<float>);
}

}  // namespace ves
