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
//     r    = A v - lambda v                    FP64 (the first one in float-float)
//     r'   = Z^H r                             FP32
//     (T - lambda I) dx - dlambda x = -r', dx_k = 0:
//        rows i > k : back substitution for dx_i
//        row  k     : dlambda x_k = r'_k + sum_{j>k} T_kj dx_j
//        rows i < k : back substitution including + dlambda x_i
//     v += Z dx, lambda += dlambda             FP64 update
// until ||r|| <= tol ||A||_F ||v|| (the final residual, FP64) and the
// correction that residual gives, |dlambda|, is <= 4 tol ||A||_F: a small
// residual bounds the eigenvalue error only up to the eigenvalue's condition
// number, while Newton's next correction estimates the error itself (the
// FP32 solve for it costs a few percent of one FP64 residual).  A pair that
// is not accepted after `max_steps` corrections sends its matrix to the FP64
// solver (the caller's second launch over the list).
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace ves {

namespace {

constexpr int kSchurThreads = 128;
constexpr int kRefineThreads = 64;

__device__ __forceinline__ long long soa_off_m(long long m, long long len, int tc)
{
    return (m / tc) * (long long)tc * len + (m % tc);
}

// float2 elements per group of 32 matrices: T, Z, X (n*n each), work (n),
// then A as two FP32 parts Ah + Al (n*n each; A - Ah - Al ~ 2^-48 |A|) for
// the refinement's first residual.
__host__ __device__ __forceinline__ long long group_elems(int n) { return 5LL * n * n + n; }

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

// Float-float accumulation (the first residual): s + p exactly as s' + e
// (TwoSum, Knuth), and s + a*b with the product's rounding error (exact, by
// fma) carried in e.  The _rn intrinsics keep the compiler from fusing these
// operations, which would void the exactness.
__device__ __forceinline__ void two_sum_acc(float &s, float &e, const float p)
{
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp)));
    s = t;
}
__device__ __forceinline__ void ff_mac(float &s, float &e, const float a, const float b)
{
    const float pr = __fmul_rn(a, b);
    const float pe = fmaf(a, b, -pr);
    two_sum_acc(s, e, pr);
    e = __fadd_rn(e, pe);
}

// One entry of an eigenvector iterate: float-float (head h, tail t with
// |t| <= ulp(h) / 2) while the residuals are float-float, FP64 (d) from the
// first FP64 residual on.  The two forms share the 16 bytes, so the per-lane
// vector costs what an FP64 one does.
union VEntry {
    cx<double> d;
    struct { cx<float> h, t; } f;
};

// (h, t) += s in float-float: TwoSum of the heads, the tail and the rounding
// error summed, then renormalised (Fast2Sum, valid as |sum| >= |tail|).
__device__ __forceinline__ void ff_add(float &h, float &t, const float s)
{
    const float sh = __fadd_rn(h, s);
    const float bp = __fsub_rn(sh, h);
    const float se = __fadd_rn(__fsub_rn(h, __fsub_rn(sh, bp)), __fsub_rn(s, bp));
    const float tt = __fadd_rn(t, se);
    h = __fadd_rn(sh, tt);
    t = __fsub_rn(tt, __fsub_rn(h, sh));
}

// r = A v - lambda v in float-float on the FP32 pipe, into r32 (rounded to
// FP32).  A = Ah + Al (two FP32 parts), v = vh + vl (the heads and tails of
// v's float-float entries) and lambda = lh + ll (kLo = false: the tails are
// zero).  The head products Ah vh and lh vh split exactly into rounded
// products and their errors (fma), the rounded products are summed by TwoSum,
// and the errors, Ah vl, Al vh, lh vl and ll vh are summed in FP32 beside
// them; Al vl and ll vl (~2^-48 of the terms) are dropped.  Error ~ 2^-48
// ||A|| ||v||.
template <int MAXN, bool kLo, class MB>
__device__ __forceinline__ void ff_residual(const int n, const MB &Ah, const MB &Al, const VEntry *v,
                                            const cx<float> lh, const cx<float> ll, cx<float> *r32)
{
    for (int i = 1; i <= n; ++i) {
        const cx<float> vi = v[i - 1].f.h;
        float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f;
        ff_mac(sr, er, -lh.r, vi.r);
        ff_mac(sr, er, lh.i, vi.i);
        ff_mac(si, ei, -lh.r, vi.i);
        ff_mac(si, ei, -lh.i, vi.r);
        if (kLo) {
            const cx<float> wi = v[i - 1].f.t;
            er = fmaf(lh.i, wi.i, fmaf(-lh.r, wi.r, fmaf(ll.i, vi.i, fmaf(-ll.r, vi.r, er))));
            ei = fmaf(-lh.i, wi.r, fmaf(-lh.r, wi.i, fmaf(-ll.i, vi.r, fmaf(-ll.r, vi.i, ei))));
        }
        for (int j = 1; j <= n; ++j) {
            const cx<float> ah = Ah.ld(i, j), al = Al.ld(i, j), vj = v[j - 1].f.h;
            ff_mac(sr, er, ah.r, vj.r);
            ff_mac(sr, er, -ah.i, vj.i);
            ff_mac(si, ei, ah.r, vj.i);
            ff_mac(si, ei, ah.i, vj.r);
            er = fmaf(-al.i, vj.i, fmaf(al.r, vj.r, er));
            ei = fmaf(al.i, vj.r, fmaf(al.r, vj.i, ei));
            if (kLo) {
                const cx<float> wj = v[j - 1].f.t;
                er = fmaf(-ah.i, wj.i, fmaf(ah.r, wj.r, er));
                ei = fmaf(ah.i, wj.r, fmaf(ah.r, wj.i, ei));
            }
        }
        r32[i - 1] = mk(__fadd_rn(sr, er), __fadd_rn(si, ei));
    }
}

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
    const long long g_end = (a.m_end + 31) / 32;
    const long long nn = (long long)n * n;
    for (long long g = a.m_begin / 32 + warp; g < g_end; g += nwarps) {
        float2 *pT = buf + g * group_elems(n) * 32 + lane;
        float2 *pZ = pT + 32 * nn, *pX = pZ + 32 * nn, *pW = pX + 32 * nn;
        const MatIlv<float> T{pT, n}, Z{pZ, n};
        const VecIlv<float> W{pW};
        const MatIlv<float> Ah{pW + 32 * n, n}, Al{pW + 32 * (n + nn), n};
        const long long m = g * 32 + lane;
        const bool valid = m >= a.m_begin && m < a.m_end;
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
                    Ah.st(i, j, f);
                    Al.st(i, j, down(csub(v, up(f))));
                }
            fb = bad || !(nA2 < 1e36f);  // beyond FP32 range: FP64
            zgehrd_lane<float>(n, T, W);
            zunghr_lane<float>(n, T, Z, W);
            clear_below_subdiag_lane<float>(n, T);
        }
        zlahqr_warp<float, true, true>(n, T, Z, valid && !fb, a.max_its, sweeps, status);
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

// ---------------------------------------------------------------------------
// schur32_warp_kernel<G>: the same FP32 Schur stage with one matrix per group
// of G lanes: a warp (G = 32, n <= 32) or half a warp (G = 16, n <= 16, two
// matrices per warp).  H and Z live in shared memory (column-major, leading
// dimension n + 1: a row sweep and a column sweep are both free of bank
// conflicts); lane l of a group owns row l + 1 in column operations and
// column l + 1 in row operations; the scalar steps (reflectors, shifts,
// deflation tests) run redundantly on all lanes of the group from shared
// values, so control flow is uniform within a group and H, Z never leave the
// SM.  The two halves of a warp synchronise only within themselves (group
// masks on every shuffle, vote and __syncwarp), so each runs its own sweep
// sequence; where they branch apart the warp runs the two paths in turn.
// Same algorithm and operation order per element as the lane routines
// (zgehd2, zung2r, zlahqr single shift, ztrevc back substitution); T, Z and
// the T-eigenvectors X go to the per-matrix buffer layout read by
// refine_kernel.
// ---------------------------------------------------------------------------
constexpr int kWarpSchurThreads = 128;  // 4 warps per block

// per-matrix buffer layout: T, Z, X (n*n float2 each, column-major), a work
// vector whose first entry holds ||A||_F^2, then Ah and Al (n*n each)
__host__ __device__ __forceinline__ long long mat_elems(int n) { return 5LL * n * n + n; }

__host__ __device__ __forceinline__ size_t warp_schur_smem(int n, int G)
{
    return (size_t)(kWarpSchurThreads / G) * (2 * n * (n + 1) + n) * sizeof(float2);
}

template <int G>
__global__ void __launch_bounds__(kWarpSchurThreads) schur32_warp_kernel(const MixedArgs a, float2 *buf, int *flags)
{
    extern __shared__ float2 wsm[];
    const int n = a.g.n, tc = a.g.tc;
    const long long N = a.g.N;
    const int gl = threadIdx.x & (G - 1), wib = threadIdx.x / G;  // lane in group, group in block
    const unsigned gmask = group_mask<G>(threadIdx.x & 31);
    const int lda = n + 1;
    float2 *sH = wsm + (size_t)wib * (2 * n * lda + n);
    float2 *sZ = sH + n * lda, *sTau = sZ + n * lda;
    const SmemMat H{sH, lda}, Z{sZ, lda};
    const long long nn = (long long)n * n;
    const long long gw = (long long)blockIdx.x * (kWarpSchurThreads / G) + wib;
    const long long nw = (long long)gridDim.x * (kWarpSchurThreads / G);
    const int j = gl + 1;  // the row / column this lane owns
    const float ulp = lim<float>::eps();
    const float smlnum = lim<float>::tiny() * ((float)n / ulp);

    for (long long m = a.m_begin + gw; m < a.m_end; m += nw) {
        // ---- load A (FP64 SoA) into H as FP32; non-finite / out-of-range check
        const long long mo = soa_off_m(m, nn, tc);
        float2 *oA = buf + m * mat_elems(n) + 3 * nn + n;  // Ah, Al of the per-matrix layout
        bool bad = false;
        float s2 = 0.f;
        for (int e = gl; e < nn; e += G) {
            const long long k = mo + (long long)e * tc;
            const double re = a.rA[k], im = a.iA[k];
            bad |= nonfinite(re) | nonfinite(im);
            const float fr = (float)re, fi = (float)im;
            s2 = fmaf(fi, fi, fmaf(fr, fr, s2));
            sH[(e % n) + (e / n) * lda] = make_float2(fr, fi);
            oA[e] = make_float2(fr, fi);
            oA[nn + e] = make_float2((float)(re - (double)fr), (float)(im - (double)fi));
        }
        const float nA2 = group_sum<G>(s2, gmask);
        bool fb = __any_sync(gmask, bad) || !(nA2 < 1e36f);
        int status = 0, sweeps = 0;
        __syncwarp(gmask);
        if (!fb) {
            hess_group<G>(n, H, sTau, gl, gmask);
            // ---- zung2r: Z = Q from the reflectors, last reflector first
            for (int i = n - 1; i >= 1; --i) {
                const cx<float> t = mk(sTau[i - 1].x, sTau[i - 1].y);
                const int c = i + 1;
                if (j >= c + 1 && j <= n) {
                    cx<float> sacc = Z.ld(c, j);
                    for (int k = c + 1; k <= n; ++k) sacc = cjmac(sacc, H.ld(k, i), Z.ld(k, j));
                    const cx<float> ts = cmul(t, sacc);
                    Z.st(c, j, csub(Z.ld(c, j), ts));
                    for (int k = c + 1; k <= n; ++k) Z.st(k, j, cnmac(Z.ld(k, j), H.ld(k, i), ts));
                }
                __syncwarp(gmask);
                if (j >= c + 1 && j <= n) Z.st(j, c, cmul(H.ld(j, i), mk(-t.r, -t.i)));
                if (j == c) Z.st(c, c, mk(1.f - t.r, -t.i));
                if (j >= 2 && j <= c - 1) Z.st(j, c, mk(0.f, 0.f));
                __syncwarp(gmask);
            }
            if (j <= n) {
                Z.st(j, 1, mk(j == 1 ? 1.f : 0.f, 0.f));
                if (j > 1) Z.st(1, j, mk(0.f, 0.f));
            }
            // clear below the subdiagonal: column j, rows j+2..n
            if (j <= n)
                for (int k = j + 2; k <= n; ++k) H.st(k, j, mk(0.f, 0.f));
            __syncwarp(gmask);
            // ---- make the subdiagonal real
            for (int i = 2; i <= n; ++i) {
                const cx<float> h = H.ld(i, i - 1);
                if (h.i != 0.f) {
                    cx<float> sc = cscal(h, frcp<float>(cabs1(h)));
                    sc = cscal(conj(sc), frcp<float>(cabs(sc)));
                    __syncwarp(gmask);
                    if (gl == 0) H.st(i, i - 1, mk(cabs(h), 0.f));
                    if (j >= i && j <= n) H.st(i, j, cmul(H.ld(i, j), sc));
                    __syncwarp(gmask);
                    const int re = (i + 1) < n ? (i + 1) : n;
                    if (j <= re) H.st(j, i, cmulc(H.ld(j, i), sc));
                    if (j <= n) Z.st(j, i, cmulc(Z.ld(j, i), sc));
                }
                __syncwarp(gmask);
            }
            // ---- single-shift QR, one matrix, uniform control flow
            int I = n, L = 1, its = 0;
            while (I > 1) {
                if (its > a.max_its) { status |= ST_ITCAP; --I; L = 1; its = 0; continue; }
                L = deflation_scan64(I, L, H, n, ulp, smlnum);
                __syncwarp(gmask);
                if (L > 1 && gl == 0) H.st(L, L - 1, mk(0.f, 0.f));
                __syncwarp(gmask);
                if (L >= I) { --I; L = 1; its = 0; continue; }
                const cx<float> t = qr_shift<float>(I, L, its, H);
                const cx<float> h11s = csub(H.ld(L, L), t);
                const float h21 = H.ld(L + 1, L).r;
                const float rs = frcp<float>(cabs1(h11s) + fabsf(h21));
                const cx<float> v0 = cscal(h11s, rs), v1 = mk(h21 * rs, 0.f);
                ++its;
                ++sweeps;
                for (int K = L; K <= I - 1; ++K) {
                    cx<float> a0 = v0, a1 = v1, t1;
                    if (K > L) { a0 = H.ld(K, K - 1); a1 = H.ld(K + 1, K - 1); }
                    zlarfg2<float>(a0, a1, t1);
                    const cx<float> w1 = a1, cw = conj(w1), c1 = conj(t1);
                    const float t2 = fmaf(t1.r, w1.r, -(t1.i * w1.i));
                    if (j >= K && j <= n) {  // rows K, K+1, column j
                        cx<float> h1 = H.ld(K, j), h2 = H.ld(K + 1, j);
                        rot_pair(h1, h2, c1, t2, w1);
                        H.st(K, j, h1);
                        H.st(K + 1, j, h2);
                    }
                    __syncwarp(gmask);
                    // the reflector's entries in column K-1, stored once every lane has
                    // read them (the row update above does not touch that column)
                    if (K > L && gl == 0) { H.st(K, K - 1, a0); H.st(K + 1, K - 1, mk(0.f, 0.f)); }
                    const int je = (K + 2) < I ? (K + 2) : I;
                    if (j <= je) {  // columns K, K+1, row j
                        cx<float> h1 = H.ld(j, K), h2 = H.ld(j, K + 1);
                        rot_pair(h1, h2, t1, t2, cw);
                        H.st(j, K, h1);
                        H.st(j, K + 1, h2);
                    }
                    if (j <= n) {  // Schur vectors, row j
                        cx<float> z1 = Z.ld(j, K), z2 = Z.ld(j, K + 1);
                        rot_pair(z1, z2, t1, t2, cw);
                        Z.st(j, K, z1);
                        Z.st(j, K + 1, z2);
                    }
                    __syncwarp(gmask);
                }
                // make H(I, I-1) real
                const cx<float> h = H.ld(I, I - 1);
                if (h.i != 0.f) {
                    const float d = cabs(h);
                    const cx<float> z = conj(cscal(h, frcp<float>(d)));
                    __syncwarp(gmask);
                    if (gl == 0) H.st(I, I - 1, mk(d, 0.f));
                    if (j >= I + 1 && j <= n) H.st(I, j, cmul(H.ld(I, j), z));
                    if (j <= I - 1) H.st(j, I, cmulc(H.ld(j, I), z));
                    if (j <= n) Z.st(j, I, cmulc(Z.ld(j, I), z));
                }
                __syncwarp(gmask);
            }
            if (status & ST_ITCAP) fb = true;
        }
        float2 *out = buf + m * mat_elems(n);
        if (!fb) {
            // T (upper triangle) and Z to the buffer, coalesced
            for (int e = gl; e < nn; e += G) {
                const int r = e % n, c = e / n;
                out[e] = r <= c ? sH[r + c * lda] : make_float2(0.f, 0.f);
                out[nn + e] = sZ[r + c * lda];
            }
            __syncwarp(gmask);
            // T-eigenvectors: lane j solves column j into sZ (Z is saved)
            if (j <= n) {
                const SmemCol xc{sZ + (j - 1) * lda};
                const cx<float> tkk = H.ld(j, j);
                const float smin = fmaxf(ulp * cabs1(tkk), smlnum);
                const float sc = j > 1 ? trevc_solve<float>(j, H, xc, smin, tkk) : 1.f;
                xc.st(j, mk(sc, 0.f));
                for (int i = j + 1; i <= n; ++i) xc.st(i, mk(0.f, 0.f));
            }
            __syncwarp(gmask);
            for (int e = gl; e < nn; e += G) out[2 * nn + e] = sZ[(e % n) + (e / n) * lda];
        }
        if (gl == 0) {
            out[3 * nn] = make_float2(nA2, 0.f);  // ||A||_F^2 for the refinement's tolerance
            flags[m] = fb ? 1 : 0;
            if (fb) to_fp64_list(a, flags, m);
            if (a.status) a.status[m] = status;
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
        __syncwarp(gmask);
    }
}

// ---------------------------------------------------------------------------
// schur32_group_kernel<G>: the FP32 Schur stage for n <= 16 with one matrix
// per group of G lanes (G = 4: eight matrices per warp; G = 8: four), H and Z
// in shared memory (4.5 KB per matrix at n = 16).
//
// Why: the lane kernel above keeps T and Z of its 32 matrices per warp in an
// HBM buffer, and its QR sweeps stream that buffer through DRAM (about 245 KB
// of traffic per matrix at n = 16 against 8.4 KB of input and output): it is
// memory-latency bound with the FP32 pipe below 10% busy.  A matrix per warp
// or half warp keeps H and Z on chip but runs every scalar step of a
// reflector on 16-32 lanes for one matrix, and its lanes idle on the short
// rows near the end of a sweep.  Here a group of G lanes owns a matrix: lane
// q of a group handles rows and columns q + 1, q + 1 + G, ... of every
// element-wise update, the scalar steps (reflector, shift, deflation test)
// run redundantly on the G lanes, and the warp's 32 / G matrices move in
// lockstep per QR sweep, as the lane kernel's 32 do: every group keeps its
// own active block [L, I] and sweep count, the bulge-chase step K is
// warp-uniform over the union of the groups' windows, and a group whose
// window does not contain K idles for that step.  Values that all lanes of a
// group write to one location (a zeroed subdiagonal, a reflector's leading
// entry) are stored by the group's first lane before a synchronisation point
// (one lane per address: several lanes storing to one shared-memory word cost
// extra wavefronts), except the zeroed subdiagonal of the deflation scan,
// which every lane of the group stores with the same value (no
// synchronisation inside the per-group scan).
//
// Same algorithm per element as the lane routines (zgehd2, zung2r, zlahqr
// single shift with the FP64 deflation test, ztrevc back substitution), in a
// different summation order for the reflector norms; the output is the
// per-matrix buffer layout of schur32_warp_kernel, read by refine_kernel.
// ---------------------------------------------------------------------------
constexpr int kGroupSchurThreads = 64;  // 2 warps per block

// float2 per matrix slot: H and Z (n (n + 1) each), tau (n), padded so that
// the slots of one warp start 4 (G = 4) or 8 (G = 8) float2 apart modulo 16:
// the lanes of a warp then touch distinct shared-memory banks when every
// group accesses the same element of its own matrix
__host__ __device__ __forceinline__ int group_slot(int n, int G)
{
    const int raw = 2 * n * (n + 1) + n, want = G == 4 ? 4 : 8;
    return raw + ((want - raw % 16) + 16) % 16;
}
__host__ __device__ __forceinline__ size_t group_schur_smem(int n, int G)
{
    return (size_t)(kGroupSchurThreads / G) * group_slot(n, G) * sizeof(float2);
}

template <int G>
__global__ void __launch_bounds__(kGroupSchurThreads) schur32_group_kernel(const MixedArgs a, float2 *buf, int *flags)
{
    extern __shared__ float2 gsm[];
    constexpr int MPW = 32 / G;  // matrices per warp
    constexpr int NPL = 16 / G;  // rows (columns) of an update per lane, n <= 16
    const int n = a.g.n, tc = a.g.tc;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), j0 = gl + 1;
    const unsigned gmask = group_mask<G>(lane);
    const int lda = n + 1;
    float2 *sH = gsm + (size_t)(threadIdx.x / G) * group_slot(n, G);
    float2 *sZ = sH + n * lda, *sTau = sZ + n * lda;
    const SmemMat H{sH, lda}, Z{sZ, lda};
    const long long nn = (long long)n * n;
    const float ulp = lim<float>::eps();
    const float smlnum = lim<float>::tiny() * ((float)n / ulp);
    const long long wg = (long long)blockIdx.x * (kGroupSchurThreads / 32) + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * (kGroupSchurThreads / 32);

    for (long long base = a.m_begin + wg * MPW; base < a.m_end; base += nw * MPW) {
        const long long m = base + (lane / G);
        const bool valid = m < a.m_end;
        // ---- load A (FP64 SoA) into H as FP32; Ah, Al to the buffer
        const long long mo = valid ? soa_off_m(m, nn, tc) : 0;
        float2 *out = buf + (valid ? m : 0) * mat_elems(n);
        bool bad = false;
        float s2 = 0.f;
        for (int e = gl; e < nn; e += G) {
            float2 h = make_float2(0.f, 0.f);
            if (valid) {
                const long long k = mo + (long long)e * tc;
                const double re = a.rA[k], im = a.iA[k];
                bad |= nonfinite(re) | nonfinite(im);
                h = make_float2((float)re, (float)im);
                s2 = fmaf(h.y, h.y, fmaf(h.x, h.x, s2));
                out[3 * nn + n + e] = h;
                out[4 * nn + n + e] = make_float2((float)(re - (double)h.x), (float)(im - (double)h.y));
            }
            sH[(e % n) + (e / n) * lda] = h;
        }
        const float nA2 = group_sum<G>(s2, gmask);
        const bool fb = valid && (__any_sync(gmask, bad) || !(nA2 < 1e36f));
        const bool run = valid && !fb;
        if (!run)  // a zero matrix: harmless arithmetic, and no sweeps
            for (int e = gl; e < nn; e += G) sH[(e % n) + (e / n) * lda] = make_float2(0.f, 0.f);
        __syncwarp();

        // ---- zgehd2: reflector i from column i, applied right then left
        for (int i = 1; i <= n - 1; ++i) {
            const int mm = n - i;
            float xs = 0.f;
            for (int k = j0; k <= n; k += G)
                if (k >= i + 2) { const cx<float> x = H.ld(k, i); xs = fmaf(x.i, x.i, fmaf(x.r, x.r, xs)); }
            const float xnorm2 = group_sum<G>(xs, gmask);
            const cx<float> alpha = H.ld(i + 1, i);
            const bool trivial = (xnorm2 == 0.f) && (alpha.i == 0.f);
            const float beta = trivial ? alpha.r : -copysignf(fsqrt<float>(fmaf(alpha.r, alpha.r, fmaf(alpha.i, alpha.i, xnorm2))), alpha.r);
            cx<float> t = mk(0.f, 0.f), scale = mk(0.f, 0.f);
            if (!trivial) {
                const float rb = frcp<float>(beta);
                t = mk((beta - alpha.r) * rb, -alpha.i * rb);
                scale = cinv(mk(alpha.r - beta, alpha.i));
            }
            __syncwarp(gmask);  // every lane has read column i
            for (int k = j0; k <= n; k += G)
                if (k >= i + 2) H.st(k, i, cmul(H.ld(k, i), scale));
            if (gl == 0) sTau[i - 1] = make_float2(t.r, t.i);
            __syncwarp(gmask);
            // the lane's rows (columns) side by side: NPL independent dot-product chains
            {  // right: row r of A(1:n, i+1:n) -= tau (A v)_r v^H
                cx<float> sacc[NPL];
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int r = j0 + u * G;
                    if (r <= n) sacc[u] = H.ld(r, i + 1);
                }
                for (int q = 2; q <= mm; ++q) {
                    const cx<float> vq = H.ld(i + q, i);
#pragma unroll
                    for (int u = 0; u < NPL; ++u) {
                        const int r = j0 + u * G;
                        if (r <= n) sacc[u] = cmac(sacc[u], H.ld(r, i + q), vq);
                    }
                }
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int r = j0 + u * G;
                    if (r > n) continue;
                    const cx<float> ts = cmul(t, sacc[u]);
                    H.st(r, i + 1, csub(H.ld(r, i + 1), ts));
                    for (int q = 2; q <= mm; ++q) H.st(r, i + q, cnmacc(H.ld(r, i + q), ts, H.ld(i + q, i)));
                }
            }
            __syncwarp(gmask);
            const cx<float> tcj = conj(t);
            {  // left: column c of A(i+1:n, i+1:n) -= conj(tau) v (v^H A)_c
                cx<float> sacc[NPL];
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int c = j0 + u * G;
                    if (c >= i + 1 && c <= n) sacc[u] = H.ld(i + 1, c);
                }
                for (int q = 2; q <= mm; ++q) {
                    const cx<float> vq = H.ld(i + q, i);
#pragma unroll
                    for (int u = 0; u < NPL; ++u) {
                        const int c = j0 + u * G;
                        if (c >= i + 1 && c <= n) sacc[u] = cjmac(sacc[u], vq, H.ld(i + q, c));
                    }
                }
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int c = j0 + u * G;
                    if (c < i + 1 || c > n) continue;
                    const cx<float> ts = cmul(tcj, sacc[u]);
                    H.st(i + 1, c, csub(H.ld(i + 1, c), ts));
                    for (int q = 2; q <= mm; ++q) H.st(i + q, c, cnmac(H.ld(i + q, c), H.ld(i + q, i), ts));
                }
            }
            __syncwarp(gmask);
            if (gl == 0) H.st(i + 1, i, mk(beta, 0.f));
            __syncwarp(gmask);
        }
        // ---- zung2r: Z = Q from the reflectors, last reflector first
        for (int e = gl; e < nn; e += G) sZ[(e % n) + (e / n) * lda] = make_float2(0.f, 0.f);
        __syncwarp(gmask);
        for (int i = n - 1; i >= 1; --i) {
            const cx<float> t = mk(sTau[i - 1].x, sTau[i - 1].y);
            const int c = i + 1;
            {
                cx<float> sacc[NPL];
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int j = j0 + u * G;
                    if (j >= c + 1 && j <= n) sacc[u] = Z.ld(c, j);
                }
                for (int k = c + 1; k <= n; ++k) {
                    const cx<float> hk = H.ld(k, i);
#pragma unroll
                    for (int u = 0; u < NPL; ++u) {
                        const int j = j0 + u * G;
                        if (j >= c + 1 && j <= n) sacc[u] = cjmac(sacc[u], hk, Z.ld(k, j));
                    }
                }
#pragma unroll
                for (int u = 0; u < NPL; ++u) {
                    const int j = j0 + u * G;
                    if (j < c + 1 || j > n) continue;
                    const cx<float> ts = cmul(t, sacc[u]);
                    Z.st(c, j, csub(Z.ld(c, j), ts));
                    for (int k = c + 1; k <= n; ++k) Z.st(k, j, cnmac(Z.ld(k, j), H.ld(k, i), ts));
                }
            }
            __syncwarp(gmask);
            for (int j = j0; j <= n; j += G) {
                if (j >= c + 1) Z.st(j, c, cmul(H.ld(j, i), mk(-t.r, -t.i)));
                if (j == c) Z.st(c, c, mk(1.f - t.r, -t.i));
                if (j >= 2 && j <= c - 1) Z.st(j, c, mk(0.f, 0.f));
            }
            __syncwarp(gmask);
        }
        for (int j = j0; j <= n; j += G) {
            Z.st(j, 1, mk(j == 1 ? 1.f : 0.f, 0.f));
            if (j > 1) Z.st(1, j, mk(0.f, 0.f));
            for (int k = j + 2; k <= n; ++k) H.st(k, j, mk(0.f, 0.f));  // clear below the subdiagonal
        }
        __syncwarp(gmask);
        // ---- make the subdiagonal real
        for (int i = 2; i <= n; ++i) {
            const cx<float> h = H.ld(i, i - 1);
            __syncwarp(gmask);
            if (h.i != 0.f) {  // the same on every lane of the group
                cx<float> sc = cscal(h, frcp<float>(cabs1(h)));
                sc = cscal(conj(sc), frcp<float>(cabs(sc)));
                if (gl == 0) H.st(i, i - 1, mk(cabs(h), 0.f));
                for (int j = j0; j <= n; j += G)
                    if (j >= i) H.st(i, j, cmul(H.ld(i, j), sc));
                __syncwarp(gmask);
                const int re = (i + 1) < n ? (i + 1) : n;
                for (int j = j0; j <= n; j += G) {  // column i, H(i, i) included (|sc| = 1)
                    if (j <= re) H.st(j, i, cmulc(H.ld(j, i), sc));
                    Z.st(j, i, cmulc(Z.ld(j, i), sc));
                }
            }
            __syncwarp(gmask);
        }
        __syncwarp();

        // ---- single-shift QR, the warp's groups in lockstep per sweep
        int I = n, L = 1, its = 0, status = 0, sweeps = 0;
        bool done = !run || n <= 1;
        for (;;) {
            bool sweep = false;
            cx<float> v0 = mk(0.f, 0.f), v1 = mk(0.f, 0.f);
            if (!done) {
                for (;;) {
                    if (I <= 1) { done = true; break; }
                    if (its > a.max_its) { status |= ST_ITCAP; --I; L = 1; its = 0; continue; }
                    L = deflation_scan64(I, L, H, n, ulp, smlnum);
                    if (L > 1) H.st(L, L - 1, mk(0.f, 0.f));  // every lane of the group: the same value
                    if (L >= I) { --I; L = 1; its = 0; continue; }
                    const cx<float> t = qr_shift<float>(I, L, its, H);
                    const cx<float> h11s = csub(H.ld(L, L), t);
                    const float h21 = H.ld(L + 1, L).r;
                    const float rs = frcp<float>(cabs1(h11s) + fabsf(h21));
                    v0 = cscal(h11s, rs);
                    v1 = mk(h21 * rs, 0.f);
                    sweep = true;
                    ++its;
                    ++sweeps;
                    break;
                }
            }
            if (!__any_sync(FULL, sweep)) break;
            const int Kmin = __reduce_min_sync(FULL, sweep ? L : INT_MAX);
            const int Kmax = __reduce_max_sync(FULL, sweep ? I - 1 : 0);
            __syncwarp();  // the scans and shifts have read H
            for (int K = Kmin; K <= Kmax; ++K) {
                const bool act = sweep && K >= L && K <= I - 1;
                cx<float> a0 = v0, a1 = v1, t1 = mk(0.f, 0.f);
                if (act) {
                    if (K > L) { a0 = H.ld(K, K - 1); a1 = H.ld(K + 1, K - 1); }
                    zlarfg2<float>(a0, a1, t1);
                }
                // (the reflector's entries in column K-1 are stored after the next
                // synchronisation: the row update below does not touch that column,
                // so no lane can still be reading them then)
                const cx<float> w1 = a1, cw = conj(w1), c1 = conj(t1);
                const float t2 = fmaf(t1.r, w1.r, -(t1.i * w1.i));
                // A lane's share of a step, n <= 16: at most NPL rows and columns;
                // the loops have a fixed trip count with predicated elements, so all
                // of a lane's loads issue before its rotations (independent chains).
                if (act) {
                    cx<float> h1[NPL], h2[NPL], z1[NPL], z2[NPL];
#pragma unroll
                    for (int t = 0; t < NPL; ++t) {
                        const int jr = K + gl + t * G, jz = j0 + t * G;
                        if (jr <= n) { h1[t] = H.ld(K, jr); h2[t] = H.ld(K + 1, jr); }  // rows K, K+1, columns K..n
                        if (jz <= n) { z1[t] = Z.ld(jz, K); z2[t] = Z.ld(jz, K + 1); }  // Schur vectors: columns K, K+1
                    }
#pragma unroll
                    for (int t = 0; t < NPL; ++t) {
                        const int jr = K + gl + t * G, jz = j0 + t * G;
                        if (jr <= n) {
                            rot_pair(h1[t], h2[t], c1, t2, w1);
                            H.st(K, jr, h1[t]);
                            H.st(K + 1, jr, h2[t]);
                        }
                        if (jz <= n) {
                            rot_pair(z1[t], z2[t], t1, t2, cw);
                            Z.st(jz, K, z1[t]);
                            Z.st(jz, K + 1, z2[t]);
                        }
                    }
                }
                __syncwarp();  // the row update is done: the column update shares the 2 x 2 block
                if (act && K > L && gl == 0) { H.st(K, K - 1, a0); H.st(K + 1, K - 1, mk(0.f, 0.f)); }
                if (act) {
                    const int je = (K + 2) < I ? (K + 2) : I;  // columns K, K+1, rows 1..min(K+2, I)
                    cx<float> h1[NPL], h2[NPL];
#pragma unroll
                    for (int t = 0; t < NPL; ++t) {
                        const int j = j0 + t * G;
                        if (j <= je) { h1[t] = H.ld(j, K); h2[t] = H.ld(j, K + 1); }
                    }
#pragma unroll
                    for (int t = 0; t < NPL; ++t) {
                        const int j = j0 + t * G;
                        if (j <= je) {
                            rot_pair(h1[t], h2[t], t1, t2, cw);
                            H.st(j, K, h1[t]);
                            H.st(j, K + 1, h2[t]);
                        }
                    }
                }
                __syncwarp();
            }
            // make H(I, I-1) real (the groups that swept)
            const cx<float> h = sweep ? H.ld(I, I - 1) : mk(0.f, 0.f);
            __syncwarp();
            if (sweep && h.i != 0.f) {
                const float d = cabs(h);
                const cx<float> z = conj(cscal(h, frcp<float>(d)));
                if (gl == 0) H.st(I, I - 1, mk(d, 0.f));
#pragma unroll
                for (int t = 0; t < NPL; ++t) {
                    const int j = j0 + t * G;
                    if (j > n) continue;
                    if (j >= I + 1) H.st(I, j, cmul(H.ld(I, j), z));
                    if (j <= I - 1) H.st(j, I, cmulc(H.ld(j, I), z));
                    Z.st(j, I, cmulc(Z.ld(j, I), z));
                }
            }
            __syncwarp();
        }
        const bool to64 = fb || (status & ST_ITCAP);
        // ---- T (upper triangle) and Z to the buffer, then the T-eigenvectors into sZ
        if (valid && !to64)
            for (int e = gl; e < nn; e += G) {
                const int r = e % n, c = e / n;
                out[e] = r <= c ? sH[r + c * lda] : make_float2(0.f, 0.f);
                out[nn + e] = sZ[r + c * lda];
            }
        __syncwarp();
        for (int j = j0; j <= n; j += G) {  // lane solves columns j0, j0 + G, ... (T read only)
            const SmemCol xc{sZ + (j - 1) * lda};
            const cx<float> tkk = H.ld(j, j);
            const float smin = fmaxf(ulp * cabs1(tkk), smlnum);
            const float sc = j > 1 ? trevc_solve<float>(j, H, xc, smin, tkk) : 1.f;
            xc.st(j, mk(sc, 0.f));
            for (int i = j + 1; i <= n; ++i) xc.st(i, mk(0.f, 0.f));
        }
        __syncwarp();
        if (valid && !to64)
            for (int e = gl; e < nn; e += G) out[2 * nn + e] = sZ[(e % n) + (e / n) * lda];
        if (valid && gl == 0) {
            out[3 * nn] = make_float2(nA2, 0.f);  // ||A||_F^2 for the refinement's tolerance
            flags[m] = to64 ? 1 : 0;
            if (to64) to_fp64_list(a, flags, m);
            if (a.status) a.status[m] = status;
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
        __syncwarp();
    }
}

// FP32 matrix in the Schur buffer, element stride S: 32 in the group layout
// of schur32_kernel, 1 in the per-matrix layout of schur32_warp_kernel.
template <int S> struct MatBuf {
    float2 *p;
    int n;
    __device__ __forceinline__ cx<float> ld(int i, int j) const
    {
        VES_CHECK_IJ(i, j, n);
        const float2 v = p[((i - 1) + (j - 1) * n) * S];
        return mk(v.x, v.y);
    }
};

// One eigenpair per lane.  MAXN bounds n (per-lane vectors live in local
// memory, indexed uniformly across the warp).  kPerMatrix: the Schur buffer
// has the per-matrix layout.
template <int MAXN, bool kPerMatrix>
__device__ __forceinline__ void refine_tile(const MixedArgs &a, const float2 *buf, int *flags, const long long tile)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long p = a.m_begin * n + tile * kRefineThreads + threadIdx.x;
    const bool valid = p < a.m_end * n;
    const long long m = valid ? p / n : 0;
    const int k = valid ? (int)(p % n) + 1 : 1;
    bool act = valid && flags[m] == 0;
    if (!__any_sync(FULL, act)) return;

    const long long nn = (long long)n * n;
    constexpr int S = kPerMatrix ? 1 : 32;
    float2 *pT = const_cast<float2 *>(buf) +
                 (kPerMatrix ? m * mat_elems(n) : (m / 32) * group_elems(n) * 32 + (m % 32));
    const MatBuf<S> T{pT, n}, Z{pT + S * nn, n}, X{pT + 2 * S * nn, n};
    const MatBuf<S> Ah{pT + S * (3 * nn + n), n}, Al{pT + S * (4 * nn + n), n};
    const float nA2 = pT[3 * S * nn].x;
    const long long mo = soa_off_m(m, nn, tc);
    const MatSoA<double> A{const_cast<double *>(a.rA) + mo, const_cast<double *>(a.iA) + mo, tc, n};

    VEntry v[MAXN];  // float-float up to the first FP64 residual, FP64 from there on
    cx<float> r32[MAXN], dx[MAXN];
    cx<double> lam = mk(0.0, 0.0);
    if (act) {
        lam = up(T.ld(k, k));
        for (int i = 1; i <= n; ++i) {  // v = Z X(:,k), X upper triangular
            cx<float> acc = mk(0.f, 0.f);
            for (int j = 1; j <= k; ++j) acc = cmac(acc, Z.ld(i, j), X.ld(j, k));
            v[i - 1].f.h = acc;
            v[i - 1].f.t = mk(0.f, 0.f);
        }
    }
    const double tol2 = a.tol * a.tol;
    // eigenvalue acceptance: the Newton correction from a certified residual
    // estimates the eigenvalue's remaining error; it must be <= 4 tol ||A||_F
    const float etol2 = (float)(16.0 * tol2);
    const float xkk = act ? X.ld(k, k).r : 1.f;
    bool fail = false;
    int n_res64 = 0, n_corr = 0, n_ff = 0;  // work counters: FP64 / float-float residuals, FP32 corrections
    const int ff_steps = a.max_steps >= 2 ? a.ff_steps : 1;  // steps whose residual is float-float
    for (int step = 0; step <= a.max_steps; ++step) {
        if (!__any_sync(FULL, act)) break;
        if (!act) continue;
        bool certified = false;
        n_res64 += step >= ff_steps;
        n_ff += step < ff_steps;
        if (step < ff_steps) {
            // The first ff_steps residuals (1 or 2) in float-float on the FP32
            // pipe (error ~ 2^-48 ||A|| ||v||); they drive the first corrections
            // and never accept a pair.  With an FP32 Jacobian each Newton step
            // gains a factor of about eps32 * cond, so most pairs reach the
            // acceptance level after the second correction: with ff_steps = 2
            // the one FP64 residual is usually the accepting one.  v is held in
            // float-float meanwhile (the corrections are added on the FP32
            // pipe); lambda is split into an FP32 head and tail.
            if (step == 0) {
                ff_residual<MAXN, false>(n, Ah, Al, v, T.ld(k, k), mk(0.f, 0.f), r32);
            } else {
                const cx<float> lh = down(lam);
                ff_residual<MAXN, true>(n, Ah, Al, v, lh, down(csub(lam, up(lh))), r32);
            }
        } else {
            // FP64 residual: the one that accepts.  The first one turns v into FP64.
            if (step == ff_steps)
                for (int i = 0; i < n; ++i) {
                    const cx<float> h = v[i].f.h, t = v[i].f.t;
                    v[i].d = cadd(up(h), up(t));
                }
            double rn2 = 0.0, vn2 = 0.0;
            for (int i = 1; i <= n; ++i) {
                const cx<double> vi = v[i - 1].d;
                cx<double> acc = mk(-(lam.r * vi.r - lam.i * vi.i), -(lam.r * vi.i + lam.i * vi.r));
                for (int j = 1; j <= n; ++j) acc = cmac(acc, A.ld(i, j), v[j - 1].d);
                rn2 = fma(acc.i, acc.i, fma(acc.r, acc.r, rn2));
                vn2 = fma(vi.i, vi.i, fma(vi.r, vi.r, vn2));
                r32[i - 1] = down(acc);
            }
            certified = rn2 <= tol2 * (double)nA2 * vn2;
        }
        if (!certified && step == a.max_steps) { fail = true; act = false; continue; }
        ++n_corr;
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
        if (certified) {
            // a small residual bounds the eigenvalue error only through its
            // condition number: accept when the next correction to lambda is
            // below 4 tol ||A||_F, else take the step and verify again
            if (dl.r * dl.r + dl.i * dl.i <= etol2 * nA2) { act = false; continue; }
            if (step == a.max_steps) { fail = true; act = false; continue; }
        }
        for (int i = 1; i <= n; ++i) {
            cx<float> s = mk(0.f, 0.f);
            for (int j = 1; j <= n; ++j) s = cmac(s, Z.ld(i, j), dx[j - 1]);
            if (step < ff_steps) {
                ff_add(v[i - 1].f.h.r, v[i - 1].f.t.r, s.r);
                ff_add(v[i - 1].f.h.i, v[i - 1].f.t.i, s.i);
            } else {
                v[i - 1].d = cadd(v[i - 1].d, up(s));
            }
        }
        lam = cadd(lam, up(dl));
    }
    if (a.work) {  // all lanes of the warp are here (the loop exits uniformly)
        const int r64 = __reduce_add_sync(FULL, n_res64), c32 = __reduce_add_sync(FULL, n_corr);
        const int ff = __reduce_add_sync(FULL, n_ff);
        if ((threadIdx.x & 31) == 0) {
            if (r64) atomicAdd(a.work + WORK_RES64, (unsigned long long)r64);
            if (c32) atomicAdd(a.work + WORK_CORR32, (unsigned long long)c32);
            if (ff) atomicAdd(a.work + WORK_RESFF, (unsigned long long)ff);
        }
    }
    if (!valid || flags[m] != 0) return;
    if (fail) {
        to_fp64_list(a, flags, m);
        return;
    }
    const long long vo = soa_off_m(m, n, tc);
    const VecSoA<double> E{a.rE + vo, a.iE + vo, tc};
    E.st(k, lam);
    // (accepted pairs passed an FP64 residual, so v is in its FP64 form)
    double scale = 1.0;
    if (a.vnorm == 1) {
        double mx = 0.0;
        for (int i = 0; i < n; ++i) mx = fmax(mx, cabs1(v[i].d));
        scale = mx > 0.0 ? 1.0 / mx : 1.0;
    } else if (a.vnorm == 2) {
        double s2 = 0.0;
        for (int i = 0; i < n; ++i) s2 = fma(v[i].d.i, v[i].d.i, fma(v[i].d.r, v[i].d.r, s2));
        scale = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
    }
    const MatSoA<double> Vo{a.rV + mo, a.iV + mo, tc, n};
    for (int i = 1; i <= n; ++i) Vo.st(i, k, cscal(v[i - 1].d, scale));
}

// Tiles of kRefineThreads pairs, block-strided: the grid is either one block
// per tile or a persistent grid whose size bounds the resident warps (the
// per-pair vectors live in local memory; fewer resident threads keep more of
// them in L1).
template <int MAXN, bool kPerMatrix>
__global__ void __launch_bounds__(kRefineThreads) refine_kernel(const MixedArgs a, const float2 *buf, int *flags)
{
    const long long ntiles = ((a.m_end - a.m_begin) * a.g.n + kRefineThreads - 1) / kRefineThreads;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
        refine_tile<MAXN, kPerMatrix>(a, buf, flags, tile);
}

// The same for n <= 16 after the lane Schur kernel (n <= 10 by default), held
// to 64 registers for 16 resident blocks per SM: n=8 measured 49.0 -> 51.4 M/s;
// the same bound on the per-matrix instances cost 2-4% at n=16 and 32.
__global__ void __launch_bounds__(kRefineThreads, 16) refine16_lane_kernel(const MixedArgs a, const float2 *buf,
                                                                           int *flags)
{
    const long long ntiles = ((a.m_end - a.m_begin) * a.g.n + kRefineThreads - 1) / kRefineThreads;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) refine_tile<16, false>(a, buf, flags, tile);
}

// Distinctness of the refined eigenvalues of each matrix.  Newton from two
// FP32 starting points can land on the same eigenpair when the FP32 Schur
// form does not resolve a cluster: both pairs pass their residual and
// correction tests, and the output holds one eigenvalue twice and misses
// another.  Every accepted eigenvalue lies within 4 tol ||A||_F of a true one,
// so two that converged to one eigenvalue are within 8 tol ||A||_F of each
// other: a matrix with two eigenvalues closer than 16 tol ||A||_F goes to the
// FP64 solver (two distinct eigenvalues that close are also left to it).  One
// thread per matrix; pairs are screened in FP32 first (the rounding of the
// FP32 copies is at most 2^-24 of each magnitude), the rest decided in FP64.
template <bool kPerMatrix>
__global__ void __launch_bounds__(128) dupcheck_kernel(const MixedArgs a, const float2 *buf, int *flags)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long m = a.m_begin + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.m_end || flags[m] != 0 || n < 2) return;
    const long long nn = (long long)n * n;
    const float2 *pT = buf + (kPerMatrix ? m * mat_elems(n) : (m / 32) * group_elems(n) * 32 + (m % 32));
    const float nA2 = pT[3 * (kPerMatrix ? 1 : 32) * nn].x;
    const double thr = 16.0 * a.tol * sqrt((double)nA2);
    const float thr_f = (float)thr;
    const long long vo = soa_off_m(m, n, tc);
    bool dup = false;
    for (int k = 1; k < n && !dup; ++k) {
        const double kr = a.rE[vo + (long long)k * tc], ki = a.iE[vo + (long long)k * tc];
        const float fkr = (float)kr, fki = (float)ki;
        for (int j = 0; j < k; ++j) {
            const double jr = a.rE[vo + (long long)j * tc], ji = a.iE[vo + (long long)j * tc];
            const float dr = fkr - (float)jr, di = fki - (float)ji;
            const float slack = 1.2e-7f * (fabsf(fkr) + fabsf(fki) + fabsf((float)jr) + fabsf((float)ji));
            if (fabsf(dr) + fabsf(di) > thr_f * 1.5f + slack) continue;  // certainly farther apart than thr
            const double er = kr - jr, ei = ki - ji;
            if (fma(er, er, ei * ei) <= thr * thr) { dup = true; break; }
        }
    }
    if (dup) to_fp64_list(a, flags, m);
}

// default blocks (4 warps each) per SM of the lane Schur kernel; VES_MIXED_BLOCKS_PER_SM overrides
int schur_default_bps()
{
    if (const char *e = getenv("VES_MIXED_BLOCKS_PER_SM")) {
        const int v = atoi(e);
        if (v >= 1 && v <= 16) return v;
    }
    return 8;
}

int device_sms()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

long long schur_blocks(long long N, int blocks_per_sm)
{
    const int sms = device_sms();
    const long long groups = (N + 31) / 32;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : schur_default_bps();
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

namespace {

// Which FP32 Schur kernel: 0 = schur32_kernel (a matrix per lane), G = 4 or
// 8 = schur32_group_kernel<G>, G = 16 or 32 = schur32_warp_kernel<G> (a
// matrix per G lanes).  With the fast FP32 division and square root, measured
// on GB300 (FP32+refine eigensolves/s, stages in sequence, two float-float
// steps): n=8 lane 47.9, group4 43.0, group8 36.1 M/s; n=12 lane 14.4,
// group4 15.4, group8 12.9 M/s; n=16 lane 6.10 (6.43 overlapped), group4
// 6.78, group8 7.04 M/s; later, with the division-free FP64 deflation test
// and unrolled lane shares: n=11 lane 17.95, group4 19.88, group8 16.44;
// n=14 8.72, 10.64, 10.16; n=16 5.95, 7.23, 7.72 M/s.  Default: the group
// kernel with G = 4 for 11 <= n <= 14 and G = 8 for n = 15, 16.  Older
// measurements, before the fast FP32 arithmetic and the group kernels:  Measured on GB300,
// FP32+refine eigensolves/s, lane -> warp (G = 32): n=16 5.34 -> 4.26 M/s,
// n=24 1.59 -> 1.63 M/s, n=32 0.66 -> 0.72 M/s (below 24 too many lanes of a
// warp idle).  Two matrices per warp (G = 16) does not recover it: with the
// Schur and refinement stages overlapped, lane -> G = 16 measured n=8 39.9 ->
// 21.0, n=12 14.1 -> 9.3, n=16 5.84 -> 4.75 M/s (its Schur stage alone at
// n=16: 90 ms per 1,048,576 matrices against about 78 for the lane kernel,
// and it leaves less of each SM to the refinement running beside it).
// Default: G = 32 for 24 <= n <= 32, the lane kernel otherwise.  Later, with
// the warp kernel's two synchronisations per step and the float-float
// refinement, stages one after the other: n=17 lane 4.88 (5.30 overlapped),
// warp 5.38 M/s; n=20 lane 3.03 (3.36), warp 3.78 M/s.  The group kernel
// generalised to n <= 32 (a matrix per 8 or 16 lanes) measured slower than
// the warp kernel at n = 17..32 (n=20 3.64 / 3.73, n=24 1.77 / 2.16, n=32
// 0.58 / 0.95 M/s against 3.78, 2.42, 1.10).  Default now: G = 32 for
// 17 <= n <= 32.
// VES_MIXED_SCHUR overrides (tests and tuning): lane; warp (G = 16 for
// n <= 16, G = 32 for n <= 32); warp16; warp32.
int schur_group(int n)
{
    const char *e = getenv("VES_MIXED_SCHUR");  // read per launch: a getenv is cheap next to a solve
    if (e && !strcmp(e, "lane")) return 0;
    if (e && !strcmp(e, "warp")) return n <= 16 ? 16 : (n <= 32 ? 32 : 0);
    if (e && !strcmp(e, "warp16")) return n <= 16 ? 16 : 0;
    if (e && !strcmp(e, "warp32")) return n <= 32 ? 32 : 0;
    if (e && !strcmp(e, "group4")) return n <= 16 ? 4 : 0;
    if (e && !strcmp(e, "group8")) return n <= 16 ? 8 : 0;
    if (n >= 11 && n <= 14) return 4;
    if (n >= 15 && n <= 16) return 8;
    return (n >= 17 && n <= 32) ? 32 : 0;
}

template <int G>
long long group_schur_blocks(int n, long long N, int blocks_per_sm)
{
    cudaFuncSetAttribute(schur32_group_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)group_schur_smem(16, G));
    const int sms = device_sms();
    int per_sm = blocks_per_sm;
    if (per_sm <= 0) {
        per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, schur32_group_kernel<G>, kGroupSchurThreads,
                                                      group_schur_smem(n, G));
        if (per_sm < 1) per_sm = 1;
    }
    const long long per_block = kGroupSchurThreads / G;
    const long long need = (N + per_block - 1) / per_block;
    return std::max<long long>(1, std::min<long long>(need, (long long)sms * per_sm));
}

template <int G>
long long warp_schur_blocks(int n, long long N, int blocks_per_sm)
{
    // per call (per device, thread safe; microseconds next to the kernel)
    cudaFuncSetAttribute(schur32_warp_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_schur_smem(G, G));
    const int sms = device_sms();
    int per_sm = blocks_per_sm;
    if (per_sm <= 0) {
        per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, schur32_warp_kernel<G>, kWarpSchurThreads,
                                                      warp_schur_smem(n, G));
        if (per_sm < 1) per_sm = 1;
    }
    const long long need = (N + kWarpSchurThreads / G - 1) / (kWarpSchurThreads / G);
    return std::max<long long>(1, std::min<long long>(need, (long long)sms * per_sm));
}

}  // namespace

namespace {

struct MixedBufs {
    float2 *buf;
    int *flags;
};
MixedBufs mixed_bufs(const MixedArgs &a)
{
    const long long groups = (a.g.N + 31) / 32;
    float2 *buf = static_cast<float2 *>(a.ws);
    int *flags = reinterpret_cast<int *>(static_cast<char *>(a.ws) +
                                         (size_t)groups * group_elems(a.g.n) * 32 * sizeof(float2));
    return {buf, flags};
}

// FP32 Schur stage of matrices [a.m_begin, a.m_end)
cudaError_t launch_schur(const MixedArgs &a, int blocks_per_sm, cudaStream_t st)
{
    const int n = a.g.n;
    const long long cnt = a.m_end - a.m_begin;
    const MixedBufs b = mixed_bufs(a);
    const int G = schur_group(n);
    if (G == 4)
        schur32_group_kernel<4><<<(unsigned)group_schur_blocks<4>(n, cnt, blocks_per_sm), kGroupSchurThreads,
                                  group_schur_smem(n, 4), st>>>(a, b.buf, b.flags);
    else if (G == 8)
        schur32_group_kernel<8><<<(unsigned)group_schur_blocks<8>(n, cnt, blocks_per_sm), kGroupSchurThreads,
                                  group_schur_smem(n, 8), st>>>(a, b.buf, b.flags);
    else if (G == 16)
        schur32_warp_kernel<16><<<(unsigned)warp_schur_blocks<16>(n, cnt, blocks_per_sm), kWarpSchurThreads,
                                  warp_schur_smem(n, 16), st>>>(a, b.buf, b.flags);
    else if (G == 32)
        schur32_warp_kernel<32><<<(unsigned)warp_schur_blocks<32>(n, cnt, blocks_per_sm), kWarpSchurThreads,
                                  warp_schur_smem(n, 32), st>>>(a, b.buf, b.flags);
    else
        schur32_kernel<<<(unsigned)schur_blocks(cnt, blocks_per_sm), kSchurThreads, 0, st>>>(a, b.buf, b.flags);
    return cudaGetLastError();
}

// FP64 refinement of the eigenpairs of matrices [a.m_begin, a.m_end)
cudaError_t launch_refine(const MixedArgs &a, cudaStream_t st)
{
    const int n = a.g.n;
    const MixedBufs b = mixed_bufs(a);
    const long long pairs = (a.m_end - a.m_begin) * n;
    long long tiles = (pairs + kRefineThreads - 1) / kRefineThreads;
    // VES_REFINE_BLOCKS_PER_SM (tuning): a persistent grid of that many blocks per SM
    if (const char *e = getenv("VES_REFINE_BLOCKS_PER_SM")) {
        const int v = atoi(e);
        if (v >= 1 && v <= 32) tiles = std::min<long long>(tiles, (long long)device_sms() * v);
    }
    const unsigned rb = (unsigned)std::max<long long>(1, tiles);
    if (schur_group(n)) {  // per-matrix buffer layout
        if (n <= 16)
            refine_kernel<16, true><<<rb, kRefineThreads, 0, st>>>(a, b.buf, b.flags);
        else
            refine_kernel<32, true><<<rb, kRefineThreads, 0, st>>>(a, b.buf, b.flags);
    } else if (n <= 16) {
        refine16_lane_kernel<<<rb, kRefineThreads, 0, st>>>(a, b.buf, b.flags);
    } else if (n <= 32) {
        refine_kernel<32, false><<<rb, kRefineThreads, 0, st>>>(a, b.buf, b.flags);
    } else {
        refine_kernel<64, false><<<rb, kRefineThreads, 0, st>>>(a, b.buf, b.flags);
    }
    return cudaGetLastError();
}

// distinctness check of the refined eigenvalues of matrices [a.m_begin, a.m_end)
cudaError_t launch_dupcheck(const MixedArgs &a, cudaStream_t st)
{
    const MixedBufs b = mixed_bufs(a);
    const unsigned blocks = (unsigned)((a.m_end - a.m_begin + 127) / 128);
    if (schur_group(a.g.n))
        dupcheck_kernel<true><<<blocks, 128, 0, st>>>(a, b.buf, b.flags);
    else
        dupcheck_kernel<false><<<blocks, 128, 0, st>>>(a, b.buf, b.flags);
    return cudaGetLastError();
}

MixedArgs whole_batch(const MixedArgs &a)
{
    MixedArgs w = a;
    if (w.m_end <= 0) {
        w.m_begin = 0;
        w.m_end = a.g.N;
    }
    return w;
}

}  // namespace

cudaError_t launch_mixed(const MixedArgs &a0, cudaStream_t st)
{
    if (a0.g.N <= 0) return cudaSuccess;
    if (a0.g.n > 64) return cudaErrorInvalidValue;  // the refinement keeps per-pair vectors of at most 64 entries
    const MixedArgs a = whole_batch(a0);
    cudaError_t e = launch_schur(a, a.blocks_per_sm, st);
    if (e == cudaSuccess) e = launch_refine(a, st);
    if (e == cudaSuccess) e = launch_dupcheck(a, st);
    return e;
}

cudaError_t launch_mixed_overlap(const MixedArgs &a0, cudaStream_t st, cudaStream_t s_schur, cudaStream_t s_refine)
{
    if (a0.g.N <= 0) return cudaSuccess;
    if (a0.g.n > 64) return cudaErrorInvalidValue;
    const MixedArgs a = whole_batch(a0);
    const long long N = a.m_end - a.m_begin;
    // chunks of whole 512-matrix units, at most 8; each chunk keeps the GPU busy on its own
    const long long unit = 512;
    long long nch = std::min<long long>(8, std::max<long long>(1, N / (32 * unit)));
    long long csz = ((N + nch - 1) / nch + unit - 1) / unit * unit;
    nch = (N + csz - 1) / csz;
    if (nch < 2) return launch_mixed(a, st);
    // the Schur kernel leaves room on each SM for refinement blocks: 4 blocks
    // per SM for the lane kernel, 6 for the warp kernel (measured on GB300,
    // FP32+refine eigensolves/s serial -> overlapped: n=8 36.1 -> 41.0 M/s,
    // n=16 5.10 -> 5.87 M/s, n=24 1.63 -> 1.72 M/s, n=32 0.726 -> 0.846 M/s);
    // VES_MIXED_OVERLAP_BLOCKS_PER_SM overrides
    // (the group kernel: as many as shared memory holds)
    const int G = schur_group(a.g.n);
    int bps = a.blocks_per_sm > 0 ? a.blocks_per_sm : (G == 4 || G == 8 ? 0 : (G ? 6 : 4));
    if (a.blocks_per_sm <= 0)
        if (const char *ev = getenv("VES_MIXED_OVERLAP_BLOCKS_PER_SM")) {
            const int v = atoi(ev);
            if (v >= 1 && v <= 16) bps = v;
        }
    cudaEvent_t fork = nullptr, join_s = nullptr, join_r = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join_s, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join_r, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(fork, st);
    if (e != cudaSuccess) {  // nothing was queued on the library streams
        if (fork) cudaEventDestroy(fork);
        if (join_s) cudaEventDestroy(join_s);
        if (join_r) cudaEventDestroy(join_r);
        return e;
    }
    e = cudaStreamWaitEvent(s_schur, fork, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s_refine, fork, 0);
    for (long long c = 0; c < nch && e == cudaSuccess; ++c) {
        MixedArgs ch = a;
        ch.m_begin = a.m_begin + c * csz;
        ch.m_end = std::min(a.m_end, ch.m_begin + csz);
        cudaEvent_t done = nullptr;
        e = launch_schur(ch, bps, s_schur);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(done, s_schur);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s_refine, done, 0);
        if (e == cudaSuccess) e = launch_refine(ch, s_refine);
        if (done) cudaEventDestroy(done);  // released once the device has passed it
    }
    // Join the library streams back into the caller's stream even after a
    // failed launch: work already queued on them writes the caller's outputs
    // and workspace, and must be ordered before anything the caller does next.
    // Where the join itself cannot be recorded, wait for the library streams.
    cudaError_t je = cudaEventRecord(join_s, s_schur);
    if (je == cudaSuccess) je = cudaStreamWaitEvent(st, join_s, 0);
    if (je != cudaSuccess) cudaStreamSynchronize(s_schur);
    cudaError_t jr = cudaEventRecord(join_r, s_refine);
    if (jr == cudaSuccess) jr = cudaStreamWaitEvent(st, join_r, 0);
    if (jr != cudaSuccess) cudaStreamSynchronize(s_refine);
    if (e == cudaSuccess) e = je != cudaSuccess ? je : jr;
    if (e == cudaSuccess) e = launch_dupcheck(a, st);
    cudaEventDestroy(fork);
    cudaEventDestroy(join_s);
    cudaEventDestroy(join_r);
    return e;
}

// The pairs that overlap come first: the lane Schur kernel with its refinement,
// then the warp Schur kernel with its refinement.
void load_mixed_kernels()
{
    load_kernel(schur32_kernel);
    load_kernel(refine16_lane_kernel);
    load_kernel(refine_kernel<32, false>);
    load_kernel(refine_kernel<64, false>);
    load_kernel(schur32_warp_kernel<32>);
    load_kernel(refine_kernel<32, true>);
    load_kernel(schur32_warp_kernel<16>);
    load_kernel(refine_kernel<16, true>);
    load_kernel(schur32_group_kernel<8>);
    load_kernel(schur32_group_kernel<4>);
    load_kernel(dupcheck_kernel<false>);
    load_kernel(dupcheck_kernel<true>);
}

}  // namespace ves
