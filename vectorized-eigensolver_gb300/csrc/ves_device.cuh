// ves_device.cuh -- per-matrix numerical routines of the batched eigensolver,
// written for one matrix per CUDA lane with the 32 lanes of a warp in lockstep.
//
// Why one matrix per lane: on GB300 the FP64 pipe retires ~1.9 lane-FMAs per
// clock per SM and a warp instruction occupies it for all 32 lanes whether or
// not they are active.  Every FP64 warp instruction must therefore carry 32
// useful operations: each lane owns one matrix, and all lanes run the same
// instruction stream.  Data-dependent control flow (QR deflation) is handled
// by keeping the K counter of a QR sweep warp-uniform while each lane keeps its
// own active window [L, I], so addresses stay coalesced and only loop bounds
// are predicated (zlahqr_warp below).
//
// Numerics follow the reference routines of kipfstuhl/vectorized-eigensolver
// (Toolbox.hpp) and LAPACK, cited per routine; indices are 1-based through the
// matrix accessors, as in both.
#pragma once

#include <cuda_runtime.h>
#include <cfloat>
#include <climits>

namespace ves {

constexpr unsigned FULL = 0xffffffffu;

// status bits, one int per matrix
constexpr int ST_ITCAP = 1;      // some eigenvalue hit the sweep cap (reference moves on silently)
constexpr int ST_NONFINITE = 2;  // input held Inf/NaN
constexpr int ST_SHIFT_FALLBACK = 4;  // learned shift abandoned for Wilkinson at least once
constexpr int ST_REFINE_FALLBACK = 8; // mixed precision: pair did not converge, solved again in FP64
constexpr int ST_BAD_DIM = 16;        // mixed-size batch: order outside the supported range, not solved

template <class R> struct cx { R r, i; };

template <class R> __device__ __forceinline__ cx<R> mk(R r, R i) { cx<R> z; z.r = r; z.i = i; return z; }
template <class R> __device__ __forceinline__ R cabs1(cx<R> z) { return fabs(z.r) + fabs(z.i); }
// Products and sums of products are written with explicit fma(): what the
// compiler would fuse on its own depends on the code around an inlined
// helper, so the same expression could round differently in two kernels.
// Written out, every kernel that inlines a helper computes the same bits
// (the lane, warp-per-matrix and eigenvalues-only FP64 solvers rely on it).
// Division, reciprocal and square root.  FP64: IEEE (the FP64 solvers give
// the reference path's results, and the lane, warp-per-matrix and
// eigenvalues-only kernels agree bit for bit).  FP32 (the Schur stage of the
// FP32 + refinement form, the learned-shift polish): the hardware's fast
// approximations (__fdividef: 2 ulp; x * rsqrtf(x): a few ulp) instead of the
// IEEE sequences, which cost several times the instructions -- Newton's
// method in FP64 corrects every FP32 eigenpair afterwards, so the FP32 stage
// only has to give a good starting point.
template <class R> __device__ __forceinline__ R fdiv(R a, R b) { return a / b; }
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) { return __fdividef(a, b); }
template <class R> __device__ __forceinline__ R frcp(R x) { return R(1) / x; }
template <> __device__ __forceinline__ float frcp<float>(float x) { return __fdividef(1.f, x); }
template <class R> __device__ __forceinline__ R fsqrt(R x) { return sqrt(x); }
template <> __device__ __forceinline__ float fsqrt<float>(float x) { return x > 0.f ? x * rsqrtf(x) : x; }

template <class R> __device__ __forceinline__ R cabs(cx<R> z) { return fsqrt<R>(fma(z.r, z.r, z.i * z.i)); }
template <class R> __device__ __forceinline__ cx<R> cmul(cx<R> a, cx<R> b) { return mk(fma(a.r, b.r, -(a.i * b.i)), fma(a.i, b.r, a.r * b.i)); }
// a * conj(b)
template <class R> __device__ __forceinline__ cx<R> cmulc(cx<R> a, cx<R> b) { return mk(fma(a.r, b.r, a.i * b.i), fma(a.i, b.r, -(a.r * b.i))); }
// conj(a) * b
template <class R> __device__ __forceinline__ cx<R> cjmul(cx<R> a, cx<R> b) { return mk(fma(a.r, b.r, a.i * b.i), fma(a.r, b.i, -(a.i * b.r))); }
template <class R> __device__ __forceinline__ cx<R> cadd(cx<R> a, cx<R> b) { return mk(a.r + b.r, a.i + b.i); }
template <class R> __device__ __forceinline__ cx<R> csub(cx<R> a, cx<R> b) { return mk(a.r - b.r, a.i - b.i); }
template <class R> __device__ __forceinline__ cx<R> cscal(cx<R> a, R d) { return mk(a.r * d, a.i * d); }
template <class R> __device__ __forceinline__ cx<R> conj(cx<R> a) { return mk(a.r, -a.i); }

// Multiply-accumulate forms written as explicit FMAs: 4 FMAs per complex
// multiply-add instead of the 6 instructions (MUL, FMA, ADD per component)
// that contraction leaves when the sum is written s + a*b.  On GB300 every
// FP64 instruction costs the same pipe time, so this is the instruction count
// that bounds the solver.
template <class R> __device__ __forceinline__ cx<R> cmac(cx<R> s, cx<R> a, cx<R> b)  // s + a*b
{
    return mk(fma(-a.i, b.i, fma(a.r, b.r, s.r)), fma(a.r, b.i, fma(a.i, b.r, s.i)));
}
template <class R> __device__ __forceinline__ cx<R> cnmac(cx<R> s, cx<R> a, cx<R> b)  // s - a*b
{
    return mk(fma(a.i, b.i, fma(-a.r, b.r, s.r)), fma(-a.r, b.i, fma(-a.i, b.r, s.i)));
}
template <class R> __device__ __forceinline__ cx<R> cmacc(cx<R> s, cx<R> a, cx<R> b)  // s + a*conj(b)
{
    return mk(fma(a.i, b.i, fma(a.r, b.r, s.r)), fma(-a.r, b.i, fma(a.i, b.r, s.i)));
}
template <class R> __device__ __forceinline__ cx<R> cnmacc(cx<R> s, cx<R> a, cx<R> b)  // s - a*conj(b)
{
    return mk(fma(-a.i, b.i, fma(-a.r, b.r, s.r)), fma(a.r, b.i, fma(-a.i, b.r, s.i)));
}
template <class R> __device__ __forceinline__ cx<R> cjmac(cx<R> s, cx<R> a, cx<R> b)  // s + conj(a)*b
{
    return mk(fma(a.i, b.i, fma(a.r, b.r, s.r)), fma(-a.i, b.r, fma(a.r, b.i, s.i)));
}
// Apply a 2-element reflector to the pair (h1, h2): z = c1*h1 + t2*h2,
// h1 -= z, h2 -= z*w (12 FP64 instructions).  Rows use c1 = conj(tau), w = v;
// columns use c1 = tau, w = conj(v).
template <class R> __device__ __forceinline__ void rot_pair(cx<R> &h1, cx<R> &h2, const cx<R> c1, const R t2, const cx<R> w)
{
    const cx<R> z = mk(fma(t2, h2.r, fma(c1.r, h1.r, -c1.i * h1.i)), fma(t2, h2.i, fma(c1.r, h1.i, c1.i * h1.r)));
    h1 = csub(h1, z);
    h2 = cnmac(h2, z, w);
}

// 1/z and a/b by Smith's method (the reference's ComplexDouble.hpp:283-353 semantics).
template <class R> __device__ __forceinline__ cx<R> cinv(cx<R> z)
{
    if (fabs(z.r) <= fabs(z.i)) {
        R ratio = fdiv<R>(z.r, z.i);
        R rden = frcp<R>(z.i * fma(ratio, ratio, R(1)));
        return mk(ratio * rden, -rden);
    } else {
        R ratio = fdiv<R>(z.i, z.r);
        R rden = frcp<R>(z.r * fma(ratio, ratio, R(1)));
        return mk(rden, -ratio * rden);
    }
}
template <class R> __device__ __forceinline__ cx<R> cdiv(cx<R> a, cx<R> b)
{
    if (fabs(b.r) <= fabs(b.i)) {
        R ratio = fdiv<R>(b.r, b.i);
        R rden = frcp<R>(b.i * fma(ratio, ratio, R(1)));
        return mk(fma(a.r, ratio, a.i) * rden, fma(a.i, ratio, -a.r) * rden);
    } else {
        R ratio = fdiv<R>(b.i, b.r);
        R rden = frcp<R>(b.r * fma(ratio, ratio, R(1)));
        return mk(fma(a.i, ratio, a.r) * rden, fma(-a.r, ratio, a.i) * rden);
    }
}
// principal square root (ComplexDouble.hpp:451-488 semantics)
template <class R> __device__ __forceinline__ cx<R> csqrt(cx<R> z)
{
    R zr = fsqrt<R>(R(0.5) * (cabs(z) + fabs(z.r)));
    R zi = (zr == R(0)) ? R(0) : fdiv<R>(fabs(z.i), R(2) * zr);
    cx<R> w = (z.r < R(0)) ? mk(zi, zr) : mk(zr, zi);
    if (z.i < R(0)) w.i = -w.i;
    return w;
}

template <class R> struct lim;
template <> struct lim<double> {
    static __device__ __forceinline__ double eps() { return DBL_EPSILON; }
    static __device__ __forceinline__ double tiny() { return DBL_MIN; }
    static __device__ __forceinline__ double huge() { return DBL_MAX; }
};
template <> struct lim<float> {
    static __device__ __forceinline__ float eps() { return FLT_EPSILON; }
    static __device__ __forceinline__ float tiny() { return FLT_MIN; }
    static __device__ __forceinline__ float huge() { return FLT_MAX; }
};

// ---------------------------------------------------------------------------
// Index checks of the bounds-checked build (-DVES_BOUNDS_CHECK; the library
// variant libves_bc.so).  Every matrix accessor below checks 1 <= i, j <= n
// and every vector accessor 1 <= i <= kMaxVecIndex; an index outside is
// counted in this translation unit's device counter and the access goes to
// the first element instead, so the kernel runs to its end and nothing is
// read or written out of bounds.  ves_bounds_violations() sums the counters
// of all translation units.  In the normal build the checks compile away.
// ---------------------------------------------------------------------------
#ifdef VES_BOUNDS_CHECK
void register_bounds_counter(unsigned long long (*read)(), void (*reset)());
namespace {
__device__ unsigned long long g_bounds_violations;
__device__ __noinline__ void bounds_hit() { atomicAdd(&g_bounds_violations, 1ULL); }
struct BoundsCounterRegistration {
    static unsigned long long read()
    {
        unsigned long long v = 0;
        cudaMemcpyFromSymbol(&v, g_bounds_violations, sizeof v);
        return v;
    }
    static void reset()
    {
        const unsigned long long z = 0;
        cudaMemcpyToSymbol(g_bounds_violations, &z, sizeof z);
    }
    BoundsCounterRegistration() { register_bounds_counter(&read, &reset); }
};
const BoundsCounterRegistration g_bounds_registration;
}  // namespace
#define VES_CHECK_IJ(i, j, n)                                                   \
    do {                                                                        \
        if ((i) < 1 || (i) > (n) || (j) < 1 || (j) > (n)) { bounds_hit(); (i) = 1; (j) = 1; } \
    } while (0)
#define VES_CHECK_I(i)                                                          \
    do {                                                                        \
        if ((i) < 1 || (i) > kMaxVecIndex) { bounds_hit(); (i) = 1; }          \
    } while (0)
#else
#define VES_CHECK_IJ(i, j, n) do { } while (0)
#define VES_CHECK_I(i) do { } while (0)
#endif
constexpr int kMaxVecIndex = 128;  // vectors hold at most 2 n entries, n <= 64

// ---------------------------------------------------------------------------
// Matrix accessors.  Indices are 1-based (i = row, j = column), column-major.
// ---------------------------------------------------------------------------

// The reference's structure-of-arrays layout: two planes, element (i,j) of a
// matrix at ((i-1) + (j-1)*n) * s from the matrix's base (s = thread_cnt).
// Bit test for Inf/NaN without touching the FP64 pipe.
__device__ __forceinline__ bool nonfinite(double v)
{
    return (__double2hiint(v) & 0x7ff00000) == 0x7ff00000;
}
__device__ __forceinline__ bool nonfinite(float v)
{
    return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u;
}

template <class R> struct MatSoA {
    R *re, *im;
    long long s;
    int n;
    __device__ __forceinline__ long long at(int i, int j) const
    {
        VES_CHECK_IJ(i, j, n);
        return ((long long)(i - 1) + (long long)(j - 1) * n) * s;
    }
    __device__ __forceinline__ cx<R> ld(int i, int j) const { long long k = at(i, j); return mk(re[k], im[k]); }
    __device__ __forceinline__ void st(int i, int j, cx<R> v) const { long long k = at(i, j); re[k] = v.r; im[k] = v.i; }
};
template <class R> struct VecSoA {
    R *re, *im;
    long long s;
    __device__ __forceinline__ cx<R> ld(int i) const
    {
        VES_CHECK_I(i);
        long long k = (long long)(i - 1) * s;
        return mk(re[k], im[k]);
    }
    __device__ __forceinline__ void st(int i, cx<R> v) const
    {
        VES_CHECK_I(i);
        long long k = (long long)(i - 1) * s;
        re[k] = v.r;
        im[k] = v.i;
    }
};

template <class R> struct vec2;
template <> struct vec2<double> { typedef double2 T; };
template <> struct vec2<float> { typedef float2 T; };

// Workspace layout: (re, im) interleaved, 32 lanes interleaved, so that a warp
// touching the same element of its 32 matrices issues one contiguous access.
template <class R> struct MatIlv {
    typename vec2<R>::T *p;  // already offset by the lane
    int n;
    __device__ __forceinline__ cx<R> ld(int i, int j) const
    {
        VES_CHECK_IJ(i, j, n);
        typename vec2<R>::T v = p[((i - 1) + (j - 1) * n) * 32];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, int j, cx<R> v) const
    {
        VES_CHECK_IJ(i, j, n);
        typename vec2<R>::T w; w.x = v.r; w.y = v.i;
        p[((i - 1) + (j - 1) * n) * 32] = w;
    }
};
template <class R> struct VecIlv {
    typename vec2<R>::T *p;
    __device__ __forceinline__ cx<R> ld(int i) const
    {
        VES_CHECK_I(i);
        typename vec2<R>::T v = p[(i - 1) * 32];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, cx<R> v) const
    {
        VES_CHECK_I(i);
        typename vec2<R>::T w; w.x = v.r; w.y = v.i;
        p[(i - 1) * 32] = w;
    }
};

// ---------------------------------------------------------------------------
// zgehrd: unblocked Householder reduction to upper Hessenberg form
// (reference Toolbox.hpp:1315-1490, LAPACK zgehd2).  The reflector sign is
// LAPACK's (beta = -sign(Re alpha) * norm), not the reference's (:1368): the
// reference's sign makes alpha - beta cancel and divides by zero on columns
// that are already reduced.  Both give unitarily similar H, so the spectrum
// and the QR iteration are unaffected.  A column with nothing to annihilate
// and real alpha gets tau = 0 (LAPACK zlarfg).
// On exit H holds the Hessenberg matrix on and above the subdiagonal and the
// reflector vectors below it; tau(i) in `tau`.
// ---------------------------------------------------------------------------
template <class R, class M, class V>
__device__ void zgehrd_lane(const int n, const M &A, const V &tau)
{
    for (int i = 1; i <= n - 1; ++i) {
        const int m = n - i;
        const cx<R> alpha = A.ld(i + 1, i);
        R xnorm2 = R(0);
        for (int k = i + 2; k <= n; ++k) {
            cx<R> x = A.ld(k, i);
            xnorm2 = fma(x.i, x.i, fma(x.r, x.r, xnorm2));
        }
        const bool trivial = (xnorm2 == R(0)) && (alpha.i == R(0));
        const R beta = trivial ? alpha.r : -copysign(fsqrt<R>(fma(alpha.r, alpha.r, fma(alpha.i, alpha.i, xnorm2))), alpha.r);
        cx<R> t = mk(R(0), R(0));
        cx<R> scale = mk(R(0), R(0));
        if (!trivial) {
            const R rb = frcp<R>(beta);
            t = mk((beta - alpha.r) * rb, -alpha.i * rb);
            scale = cinv(mk(alpha.r - beta, alpha.i));
        }
        for (int k = i + 2; k <= n; ++k) A.st(k, i, cmul(A.ld(k, i), scale));
        tau.st(i, t);
        // v = [1; A(i+2:n, i)].  Right: A(1:n, i+1:n) -= tau * (A v) v^H, row by row.
        for (int k = 1; k <= n; ++k) {
            cx<R> s = A.ld(k, i + 1);
            for (int j = 2; j <= m; ++j) s = cmac(s, A.ld(k, i + j), A.ld(i + j, i));
            const cx<R> ts = cmul(t, s);
            A.st(k, i + 1, csub(A.ld(k, i + 1), ts));
            for (int j = 2; j <= m; ++j) A.st(k, i + j, cnmacc(A.ld(k, i + j), ts, A.ld(i + j, i)));
        }
        // Left: A(i+1:n, i+1:n) -= conj(tau) * v (v^H A), column by column.
        const cx<R> tc = conj(t);
        for (int j = i + 1; j <= n; ++j) {
            cx<R> s = A.ld(i + 1, j);
            for (int k = 2; k <= m; ++k) s = cjmac(s, A.ld(i + k, i), A.ld(i + k, j));
            const cx<R> ts = cmul(tc, s);
            A.st(i + 1, j, csub(A.ld(i + 1, j), ts));
            for (int k = 2; k <= m; ++k) A.st(i + k, j, cnmac(A.ld(i + k, j), A.ld(i + k, i), ts));
        }
        A.st(i + 1, i, mk(beta, R(0)));
    }
}

// ---------------------------------------------------------------------------
// zunghr: form Q = H(1) H(2) ... H(n-1) from the reflectors that zgehrd_lane
// left below the subdiagonal of A (reference Toolbox.hpp:1492-1659, LAPACK
// zunghr + zung2r).  The reference first shifts the reflector columns one
// place right inside Q; here they are read from A directly and Q is written to
// a separate matrix, which is the same arithmetic.
// ---------------------------------------------------------------------------
//
// Q may be the same storage as A (the reference's in-place call_zunghr): step
// i reads reflector column i and writes columns i+1..n only, and the first row
// and column are written last.
template <class R, class MA, class MQ, class V>
__device__ void zunghr_lane(const int n, const MA &A, const MQ &Q, const V &tau)
{
    // zung2r on Q(2:n, 2:n), reflector i has u(i) = 1, u(i+1:n-1) = A(i+2:n, i)
    for (int i = n - 1; i >= 1; --i) {
        const cx<R> t = tau.ld(i);
        const int c = i + 1;  // global column / row of the reflector's unit entry
        // apply H(i) from the left to Q(c:n, c+1:n): Q -= tau * u (u^H Q)
        for (int j = c + 1; j <= n; ++j) {
            cx<R> s = Q.ld(c, j);
            for (int k = c + 1; k <= n; ++k) s = cjmac(s, A.ld(k, i), Q.ld(k, j));
            const cx<R> ts = cmul(t, s);
            Q.st(c, j, csub(Q.ld(c, j), ts));
            for (int k = c + 1; k <= n; ++k) Q.st(k, j, cnmac(Q.ld(k, j), A.ld(k, i), ts));
        }
        // column c: -tau * u below, 1 - tau on the diagonal, zeros above
        const cx<R> mt = mk(-t.r, -t.i);
        for (int k = c + 1; k <= n; ++k) Q.st(k, c, cmul(A.ld(k, i), mt));
        Q.st(c, c, mk(R(1) - t.r, -t.i));
        for (int k = 2; k <= c - 1; ++k) Q.st(k, c, mk(R(0), R(0)));
    }
    // first row and column of Q are those of the identity
    for (int k = 1; k <= n; ++k) {
        Q.st(k, 1, mk(R(k == 1), R(0)));
        if (k > 1) Q.st(1, k, mk(R(0), R(0)));
    }
}

// Q = identity (the reference's call_zlahqr_new starts from I, utils.cpp:167-169).
template <class R, class M>
__device__ void set_identity_lane(const int n, const M &Q)
{
    for (int j = 1; j <= n; ++j)
        for (int i = 1; i <= n; ++i) Q.st(i, j, mk(R(i == j), R(0)));
}

// Zero H(i,j) for i >= j+2 (what LAPACK zlahqr does on entry; the reference
// omits it, Toolbox.hpp:721-723).
template <class R, class M>
__device__ void clear_below_subdiag_lane(const int n, const M &H)
{
    for (int j = 1; j <= n - 2; ++j)
        for (int i = j + 2; i <= n; ++i) H.st(i, j, mk(R(0), R(0)));
}

// ---------------------------------------------------------------------------
// zlahqr, wantT = wantZ = true: single-shift complex QR with Schur vectors
// (reference Toolbox.hpp:690-1031 + single_shift_qr_schur :138-369 + scale_rc
// :14-29; LAPACK zlahqr of the 3.1 generation).  Same deflation criterion
// (Ahues-Tisseur), exceptional shifts at the 10th and 20th sweep, Wilkinson
// shift, 2-element reflector bulge chase, and at most max_its+1 sweeps per
// eigenvalue after which it moves on as the reference does (reported in
// status).  The deflation test reads Re H(K+1,K) where the reference reads
// its imaginary part (:840); subdiagonals are real here, so the reference
// term is always zero -- the difference only shows when two adjacent diagonal
// entries are exactly zero.
//
// Warp-cooperative: must be called by all 32 lanes; `valid` marks lanes that
// own a matrix.  Every lane keeps its own (I, L, its); a sweep round runs the
// K loop over the union of the lanes' windows with a warp-uniform K, so each
// matrix element access is the same offset for all lanes.
// ---------------------------------------------------------------------------
template <class R, bool kSchur = true, class MH, class MZ>
__device__ void make_subdiag_real_lane(const int n, const MH &H, const MZ &Z)
{
    for (int i = 2; i <= n; ++i) {
        const cx<R> h = H.ld(i, i - 1);
        if (h.i != R(0)) {
            cx<R> sc = cscal(h, frcp<R>(cabs1(h)));
            sc = cscal(conj(sc), frcp<R>(cabs(sc)));
            H.st(i, i - 1, mk(cabs(h), R(0)));
            for (int j = i; j <= n; ++j) H.st(i, j, cmul(H.ld(i, j), sc));
            const int re = (i + 1) < n ? (i + 1) : n;
            for (int j = 1; j <= re; ++j) H.st(j, i, cmulc(H.ld(j, i), sc));
            if (kSchur)
                for (int j = 1; j <= n; ++j) Z.st(j, i, cmulc(Z.ld(j, i), sc));
        }
    }
}

// Scan for a negligible subdiagonal in rows I..L+1 (reference :810-867).
template <class R, class MH>
__device__ __forceinline__ int deflation_scan(const int I, const int L0, const MH &H, const int n, const R ulp, const R smlnum)
{
    int K;
    for (K = I; K >= L0 + 1; --K) {
        const cx<R> hk = H.ld(K, K - 1);
        if (cabs1(hk) <= smlnum) break;
        const cx<R> hkm = H.ld(K - 1, K - 1), hkk = H.ld(K, K);
        R tst = cabs1(hkm) + cabs1(hkk);
        if (tst == R(0)) {
            if (K - 2 >= 1) tst += fabs(H.ld(K - 1, K - 2).r);
            if (K + 1 <= n) tst += fabs(H.ld(K + 1, K).r);
        }
        if (fabs(hk.r) <= ulp * tst) {
            R d2 = cabs1(hk), d3 = cabs1(H.ld(K - 1, K));
            const R ab = fmax(d2, d3), ba = fmin(d2, d3);
            d2 = cabs1(hkk);
            d3 = cabs1(csub(hkm, hkk));
            const R aa = fmax(d2, d3), bb = fmin(d2, d3);
            const R s = aa + ab;
            if (ba * (ab / s) <= fmax(smlnum, ulp * (bb * (aa / s)))) break;
        }
    }
    return K;
}

// The same deflation test evaluated in FP64 on an FP32 matrix (the FP32 +
// refinement form keeps the deflation decision in FP64; the thresholds are
// FP32's ulp and smlnum, the precision the QR runs in).  An FP32 screen
// settles every subdiagonal that is clearly not negligible -- nearly all of
// them: its sums and products round by a few 2^-24 relative, far inside the
// 2^-20 margin, so the FP64 evaluation would decide the same.  Only the
// others (the subdiagonals at or near deflation, and tst = 0) are tested in
// FP64, so the decisions are those of a full FP64 evaluation.  The
// Ahues-Tisseur comparison is the reference's multiplied through by its
// positive denominator (the same test, without divisions).
template <class MH>
__device__ __forceinline__ int deflation_scan64(const int I, const int L0, const MH &H, const int n, const float ulp,
                                                const float smlnum)
{
    const float margin = 1.0f + 0x1p-20f;
    const double ulp64 = ulp, sml64 = smlnum;
    int K;
    for (K = I; K >= L0 + 1; --K) {
        const cx<float> hkf = H.ld(K, K - 1), hkmf = H.ld(K - 1, K - 1), hkkf = H.ld(K, K);
        const float tf = cabs1(hkmf) + cabs1(hkkf);
        if (cabs1(hkf) > smlnum * margin && tf > 0.f && fabsf(hkf.r) > ulp * tf * margin) continue;
        const cx<double> hk = mk((double)hkf.r, (double)hkf.i), hkm = mk((double)hkmf.r, (double)hkmf.i),
                         hkk = mk((double)hkkf.r, (double)hkkf.i);
        if (cabs1(hk) <= sml64) break;
        double tst = cabs1(hkm) + cabs1(hkk);
        if (tst == 0.0) {
            if (K - 2 >= 1) tst += fabs((double)H.ld(K - 1, K - 2).r);
            if (K + 1 <= n) tst += fabs((double)H.ld(K + 1, K).r);
        }
        if (fabs(hk.r) <= ulp64 * tst) {
            // Ahues-Tisseur: ba (ab / s) <= max(smlnum, ulp bb (aa / s)), s = aa + ab > 0,
            // multiplied through by s: no division (two FP64 division sequences a
            // test), and on FP32 data the sums and products are exact in FP64
            const cx<float> hkuf = H.ld(K - 1, K);
            double d2 = cabs1(hk), d3 = cabs1(mk((double)hkuf.r, (double)hkuf.i));
            const double ab = fmax(d2, d3), ba = fmin(d2, d3);
            d2 = cabs1(hkk);
            d3 = cabs1(csub(hkm, hkk));
            const double aa = fmax(d2, d3), bb = fmin(d2, d3);
            const double s = aa + ab;
            if (ba * ab <= fmax(sml64 * s, ulp64 * (bb * aa))) break;
        }
    }
    return K;
}

// deflation_scan, or for kDefl64 (FP32 data only) deflation_scan64
template <class R, bool kDefl64, class MH>
__device__ __forceinline__ int deflation_scan_sel(const int I, const int L0, const MH &H, const int n, const R ulp,
                                                  const R smlnum)
{
    if constexpr (kDefl64) return deflation_scan64(I, L0, H, n, (float)ulp, (float)smlnum);
    else return deflation_scan<R>(I, L0, H, n, ulp, smlnum);
}

// Shift for sweep number `its` on the active block L..I (reference :896-990).
template <class R, class MH>
__device__ __forceinline__ cx<R> qr_shift(const int I, const int L, const int its, const MH &H)
{
    if (its == 10) { const cx<R> h = H.ld(L, L); return mk(fma(R(0.75), fabs(H.ld(L + 1, L).r), h.r), h.i); }
    if (its == 20) { const cx<R> h = H.ld(I, I); return mk(fma(R(0.75), fabs(H.ld(I, I - 1).r), h.r), h.i); }
    cx<R> t = H.ld(I, I);
    const cx<R> u = cmul(csqrt(H.ld(I - 1, I)), csqrt(H.ld(I, I - 1)));
    R s = cabs1(u);
    if (s != R(0)) {
        const cx<R> x = cscal(csub(H.ld(I - 1, I - 1), t), R(0.5));
        const R sx = cabs1(x);
        s = fmax(s, sx);
        const R rs = frcp<R>(s);
        const cx<R> xs = cscal(x, rs), us = cscal(u, rs);
        cx<R> y = cscal(csqrt(cadd(cmul(xs, xs), cmul(us, us))), s);
        if (sx > R(0)) {
            const R rsx = frcp<R>(sx);
            if (fma(x.r * rsx, y.r, (x.i * rsx) * y.i) < R(0)) y = mk(-y.r, -y.i);
        }
        t = csub(t, cmul(cdiv(u, cadd(x, y)), u));
    }
    return t;
}

// 2-element Householder reflector for (v0, v1) (reference :186-241, LAPACK
// zlarfg with n = 2).  Returns tau in t1, overwrites v1 with the scaled vector
// entry and v0 with the new leading entry.
//
// It runs once per bulge-chase step, so its divisions and square root cost
// a noticeable share of the FP64 pipe (each is a sequence of several FP64
// instructions).  When |(v0, v1)|^2 is a comfortably normal number -- every
// case but the tiny or huge vectors that need the reference's rescaling --
// one reciprocal square root gives both beta = +-norm and 1/beta, and
// 1/z (z = v0 + beta) comes from tau = z/beta, whose real part lies in
// [1, 2]: 1/z = conj(tau) (1/beta) / |tau|^2, one more reciprocal.  Two
// reciprocal sequences replace the reference's square root, reciprocal and
// Smith division (a division and a reciprocal); the reflector is the same up
// to rounding.
template <class R> __device__ __forceinline__ R frsqrt(R x);
template <> __device__ __forceinline__ double frsqrt<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float frsqrt<float>(float x) { return rsqrtf(x); }
template <class R> struct rfl_range;  // |(v0, v1)|^2 range of the fast path
template <> struct rfl_range<double> { static __device__ __forceinline__ double lo() { return 1e-290; } };
template <> struct rfl_range<float> { static __device__ __forceinline__ float lo() { return 1e-36f; } };

template <class R>
__device__ __forceinline__ void zlarfg2(cx<R> &v0, cx<R> &v1, cx<R> &t1)
{
    if (v1.r == R(0) && v1.i == R(0) && v0.i == R(0)) {
        t1 = mk(R(0), R(0));
        return;
    }
    const R nrm2 = fma(v1.i, v1.i, fma(v1.r, v1.r, fma(v0.i, v0.i, v0.r * v0.r)));
    if (nrm2 >= rfl_range<R>::lo() && nrm2 <= lim<R>::huge()) {
        const R rn = frsqrt<R>(nrm2);  // 1 / norm
        const R beta = copysign(nrm2 * rn, v0.r), rb = copysign(rn, v0.r);
        t1 = cscal(mk(v0.r + beta, v0.i), rb);  // tau = z / beta
        const R q = rb * frcp<R>(fma(t1.r, t1.r, t1.i * t1.i));
        v1 = cmul(v1, mk(t1.r * q, -t1.i * q));  // v1 / z
        v0 = mk(-beta, R(0));
        return;
    }
    const R safmin = lim<R>::tiny() / (lim<R>::eps() * R(0.5));
    R norm = fsqrt<R>(nrm2);
    int knt = 0;
    if (norm < safmin) {
        const R rs = R(1) / safmin;
        do {
            ++knt;
            v1 = cscal(v1, rs);
            v0 = cscal(v0, rs);
            norm *= rs;
        } while (norm < safmin && knt < 40);
        norm = fsqrt<R>(fma(v1.i, v1.i, fma(v1.r, v1.r, fma(v0.i, v0.i, v0.r * v0.r))));
    }
    R beta = copysign(norm, v0.r);
    const cx<R> z = mk(v0.r + beta, v0.i);
    t1 = cscal(z, frcp<R>(beta));
    v1 = cmul(v1, cinv(z));
    for (int q = 0; q < knt; ++q) beta *= safmin;
    v0 = mk(-beta, R(0));
}

// ---------------------------------------------------------------------------
// Warp-cooperative FP32 helpers: one matrix per warp in shared memory
// (column-major, leading dimension lda = n + 1 so that a row sweep and a
// column sweep are both free of bank conflicts).  Lane l owns row l + 1 in
// column operations and column l + 1 in row operations; scalar steps run
// redundantly on all lanes from shared values (uniform control flow).
// ---------------------------------------------------------------------------
struct SmemMat {
    float2 *p;
    int lda;
    __device__ __forceinline__ cx<float> ld(int i, int j) const
    {
        VES_CHECK_IJ(i, j, lda - 1);
        const float2 v = p[(i - 1) + (j - 1) * lda];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, int j, cx<float> v) const
    {
        VES_CHECK_IJ(i, j, lda - 1);
        p[(i - 1) + (j - 1) * lda] = make_float2(v.r, v.i);
    }
};
struct SmemCol {  // column of a SmemMat as a vector
    float2 *p;
    __device__ __forceinline__ cx<float> ld(int i) const
    {
        VES_CHECK_I(i);
        const float2 v = p[i - 1];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ void st(int i, cx<float> v) const
    {
        VES_CHECK_I(i);
        p[i - 1] = make_float2(v.r, v.i);
    }
};

// Sum over a group of G lanes (G = 32: the warp; G = 16: one half of it);
// mask holds the group's lanes.
template <int G>
__device__ __forceinline__ float group_sum(float v, unsigned mask)
{
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) { return group_sum<32>(v, FULL); }

// The lanes of the G-lane group that lane `lane` of the warp belongs to.
template <int G>
__device__ __forceinline__ unsigned group_mask(int lane)
{
    return G == 32 ? FULL : (((1u << G) - 1u) << (lane & ~(G - 1)));
}

// zgehd2 on a G-lane group's matrix (n <= G): H = Q^H A Q, the same
// reflector conventions and per-element operation order as zgehrd_lane;
// reflector vectors below the subdiagonal, tau(i) in sTau[i - 1].  gl is the
// lane's index in its group, mask the group's lanes.
template <int G>
__device__ __forceinline__ void hess_group(const int n, const SmemMat &H, float2 *sTau, const int gl, const unsigned mask)
{
    const int j = gl + 1;
    for (int i = 1; i <= n - 1; ++i) {
        const int mm = n - i;
        const cx<float> xk = (j >= i + 2 && j <= n) ? H.ld(j, i) : mk(0.f, 0.f);
        const float xnorm2 = group_sum<G>(fmaf(xk.i, xk.i, xk.r * xk.r), mask);
        const cx<float> alpha = H.ld(i + 1, i);
        const bool trivial = (xnorm2 == 0.f) && (alpha.i == 0.f);
        const float beta = trivial ? alpha.r : -copysignf(fsqrt<float>(fmaf(alpha.r, alpha.r, fmaf(alpha.i, alpha.i, xnorm2))), alpha.r);
        cx<float> t = mk(0.f, 0.f), scale = mk(0.f, 0.f);
        if (!trivial) {
            const float rb = frcp<float>(beta);
            t = mk((beta - alpha.r) * rb, -alpha.i * rb);
            scale = cinv(mk(alpha.r - beta, alpha.i));
        }
        __syncwarp(mask);  // every lane has read alpha and its x element
        if (j >= i + 2 && j <= n) H.st(j, i, cmul(xk, scale));
        if (gl == 0) sTau[i - 1] = make_float2(t.r, t.i);
        __syncwarp(mask);
        // right: row j of A(1:n, i+1:n) -= tau (A v)_j v^H
        if (j <= n) {
            cx<float> sacc = H.ld(j, i + 1);
            for (int q = 2; q <= mm; ++q) sacc = cmac(sacc, H.ld(j, i + q), H.ld(i + q, i));
            const cx<float> ts = cmul(t, sacc);
            H.st(j, i + 1, csub(H.ld(j, i + 1), ts));
            for (int q = 2; q <= mm; ++q) H.st(j, i + q, cnmacc(H.ld(j, i + q), ts, H.ld(i + q, i)));
        }
        __syncwarp(mask);
        // left: column j of A(i+1:n, i+1:n) -= conj(tau) v (v^H A)_j
        if (j >= i + 1 && j <= n) {
            const cx<float> tcj = conj(t);
            cx<float> sacc = H.ld(i + 1, j);
            for (int q = 2; q <= mm; ++q) sacc = cjmac(sacc, H.ld(i + q, i), H.ld(i + q, j));
            const cx<float> ts = cmul(tcj, sacc);
            H.st(i + 1, j, csub(H.ld(i + 1, j), ts));
            for (int q = 2; q <= mm; ++q) H.st(i + q, j, cnmac(H.ld(i + q, j), H.ld(i + q, i), ts));
        }
        __syncwarp(mask);
        if (gl == 0) H.st(i + 1, i, mk(beta, 0.f));
        __syncwarp(mask);
    }
}

__device__ __forceinline__ void hess32_warp(const int n, const SmemMat &H, float2 *sTau, const int lane)
{
    hess_group<32>(n, H, sTau, lane, FULL);
}

//
// kSchur = false is the eigenvalues-only form (LAPACK wantT = wantZ = false,
// the reference's dead zlahqr_ at Toolbox.hpp:1663-1890): only the active block
// L..I is transformed (I1 = L, I2 = I) and Z is never touched.  The arithmetic
// on the active block is the same as with kSchur = true, so the eigenvalues
// are the same bit for bit.
// Shift providers for zlahqr_warp.  NoShiftPredictions: the reference's
// Wilkinson / exceptional shifts only.  ShiftPredictions: n predicted
// eigenvalues per matrix (the learned-shift network's output); for the first
// `sweeps` sweeps of each eigenvalue the unused prediction nearest to the
// Wilkinson estimate replaces it, after which (and for the exceptional shifts)
// the reference's shifts take over.  An eigenvalue that still needs more than
// sweeps + 2 sweeps counts as a fallback to Wilkinson.
struct NoShiftPredictions {
    template <class R> __device__ __forceinline__ void pick(int, int, cx<R> &, R) {}
    __device__ __forceinline__ void deflated(int) {}
};
// Learned shifts: for the first `sweeps` sweeps of an eigenvalue, the QR shift
// is the unused prediction nearest to the Wilkinson estimate -- provided the
// subdiagonal |H(I,I-1)| still exceeds `gate` (absolute) when the eigenvalue
// starts: once it is that small the Wilkinson shift is already more accurate
// than the predictions, and they are left alone.
struct ShiftPredictions {
    VecIlv<double> S;  // this matrix's n predictions in the workspace (NaN: none)
    int n, sweeps;
    double gate;
    unsigned long long used;
    int current;
    int fallbacks;
    template <class R> __device__ __forceinline__ void pick(int its, int, cx<R> &t, R hsub)
    {
        if (its == 0) {
            current = -1;
            if (sweeps > 0 && hsub > (R)gate) {
                R best = R(0);
                int bi = -1;
                for (int k = 0; k < n; ++k) {
                    if ((used >> k) & 1ULL) continue;
                    const cx<double> p = S.ld(k + 1);
                    if (p.r != p.r) continue;  // dropped prediction
                    const R dr = (R)p.r - t.r, di = (R)p.i - t.i;
                    const R d = dr * dr + di * di;
                    if (bi < 0 || d < best) { best = d; bi = k; }
                }
                current = bi;
                if (bi >= 0) used |= 1ULL << bi;
            }
        }
        if (its >= sweeps || its == 10 || its == 20) return;
        if (current >= 0) {
            const cx<double> p = S.ld(current + 1);
            t = mk((R)p.r, (R)p.i);
        }
    }
    // a predicted eigenvalue that still needed more than sweeps + 2 sweeps
    __device__ __forceinline__ void deflated(int its) { if (current >= 0 && its > sweeps + 2) ++fallbacks; }
};

// Polish of the predicted shifts: simultaneous (Aberth-Ehrlich) iteration on
// det(H - s I) for the upper Hessenberg H, in FP32 on Hf (an FP32 copy of H).
// Hyman's recurrence gives the Newton correction N = p(s) / p'(s): with x_n = 1,
//     x_{i-1} = -[(h_ii - s) x_i + sum_{j>i} h_ij x_j] / h_{i,i-1},   i = n..2,
//     r(s)    = (h_11 - s) x_1 + sum_{j>1} h_1j x_j,
// det(H - s I) = c r(s) with c independent of s, so N = r / r', r' from the
// differentiated recurrence (x, x' are rescaled together when they grow: the
// ratio does not depend on their common scale).  Aberth's step is Newton's on
// p(s) / prod_{q != k} (s - s_q): s_k -= N / (1 - N sum_{q != k} 1/(s_k - s_q)),
// which pushes two predictions near one eigenvalue apart instead of letting
// both converge to it (Aberth 1973, Ehrlich 1967).  Here the sweep over the
// predictions uses the newest values (Gauss-Seidel order).  Each prediction
// in S takes up to `steps` steps, stopping once a step is below `tol`; it is
// kept only if its last step was below `keep` (the iteration has reached its
// fast phase): one that has not converged, or whose iteration broke down (a
// zero subdiagonal, non-finite values), or that lands within `dup` of an
// earlier one is dropped (NaN), and its eigenvalue is found with the
// Wilkinson shift -- a far prediction costs sweeps, a dropped one costs
// nothing.  The FP32 pipe does this work at a small fraction of one FP64 QR
// sweep.
template <int MAXN>
__device__ void polish_shifts_lane(const int n, const MatIlv<float> &Hf, const VecIlv<double> &S, const int steps,
                                   const float tol, const float keep, const float dup)
{
    static_assert(MAXN <= 64, "one bit per prediction");
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    cx<float> x[MAXN], dx[MAXN];
    unsigned long long live = 0, done = 0, good = 0;
    for (int k = 1; k <= n; ++k) {
        const cx<double> s0 = S.ld(k);
        if (!nonfinite(s0.r) && !nonfinite(s0.i) && n >= 2) live |= 1ULL << (k - 1);
    }
    for (int it = 0; it < steps && (live & ~done); ++it) {
        for (int k = 1; k <= n; ++k) {
            const unsigned long long bit = 1ULL << (k - 1);
            if (!(live & bit) || (done & bit)) continue;
            const cx<double> s0 = S.ld(k);
            const cx<float> s = mk((float)s0.r, (float)s0.i);
            bool ok = true;
            x[n - 1] = mk(1.f, 0.f);
            dx[n - 1] = mk(0.f, 0.f);
            for (int i = n; i >= 2; --i) {
                const cx<float> d = csub(Hf.ld(i, i), s);
                cx<float> acc = cmul(d, x[i - 1]);
                cx<float> dacc = csub(cmul(d, dx[i - 1]), x[i - 1]);
                for (int j = i + 1; j <= n; ++j) {
                    const cx<float> h = Hf.ld(i, j);
                    acc = cmac(acc, h, x[j - 1]);
                    dacc = cmac(dacc, h, dx[j - 1]);
                }
                const cx<float> sub = Hf.ld(i, i - 1);
                if (sub.r == 0.f && sub.i == 0.f) { ok = false; break; }
                x[i - 2] = cdiv(mk(-acc.r, -acc.i), sub);
                dx[i - 2] = cdiv(mk(-dacc.r, -dacc.i), sub);
                if (cabs1(x[i - 2]) > 1e18f) {
                    for (int j = i - 1; j <= n; ++j) { x[j - 1] = cscal(x[j - 1], 1e-18f); dx[j - 1] = cscal(dx[j - 1], 1e-18f); }
                }
            }
            cx<float> delta = mk(0.f, 0.f);
            if (ok) {
                const cx<float> d1 = csub(Hf.ld(1, 1), s);
                cx<float> r = cmul(d1, x[0]);
                cx<float> rp = csub(cmul(d1, dx[0]), x[0]);
                for (int j = 2; j <= n; ++j) {
                    const cx<float> h = Hf.ld(1, j);
                    r = cmac(r, h, x[j - 1]);
                    rp = cmac(rp, h, dx[j - 1]);
                }
                delta = cdiv(r, rp);
                ok = !nonfinite(delta.r) && !nonfinite(delta.i);
            }
            if (!ok) { live &= ~bit; continue; }
            cx<float> w = mk(0.f, 0.f);
            for (int q = 1; q <= n; ++q) {
                if (q == k || !(live & (1ULL << (q - 1)))) continue;
                const cx<double> sq = S.ld(q);
                const cx<float> d = mk(s.r - (float)sq.r, s.i - (float)sq.i);
                if (d.r != 0.f || d.i != 0.f) w = cadd(w, cinv(d));
            }
            const cx<float> ab = cdiv(delta, csub(mk(1.f, 0.f), cmul(delta, w)));
            if (!nonfinite(ab.r) && !nonfinite(ab.i)) delta = ab;
            const cx<float> sn = csub(s, delta);
            S.st(k, mk((double)sn.r, (double)sn.i));
            const float last = cabs1(delta);
            good = last <= keep ? (good | bit) : (good & ~bit);
            if (last <= tol) done |= bit;
        }
    }
    for (int k = 1; k <= n; ++k)
        if (!(live & good & (1ULL << (k - 1)))) S.st(k, mk(nan, nan));
    for (int k = 2; k <= n; ++k) {
        const cx<double> sk = S.ld(k);
        for (int j = 1; j < k; ++j) {
            const cx<double> sj = S.ld(j);
            if (sj.r == sj.r && fabs(sj.r - sk.r) + fabs(sj.i - sk.i) <= (double)dup) {
                S.st(k, mk(nan, nan));
                break;
            }
        }
    }
}

// One Newton step in FP64 on det(H - s I) for every finite prediction in S,
// H the solve's own FP64 Hessenberg matrix (real subdiagonal, as zgehrd
// leaves it).  The FP32 polish works on an FP32 Hessenberg form of A, whose
// eigenvalues are those of A to about 1e-6 of their scale; from there one
// step takes a prediction to about 1e-12, and a QR sweep with that shift all
// but deflates its eigenvalue.  Hyman's recurrence gives r(s) in FP64 (x in
// X); the derivative r'(s) only has to be right to a few digits (Newton with
// a derivative of relative error e gains a factor e on top of the quadratic
// step), so its recurrence runs in FP32 on Hf, an FP32 copy of H (x' in DX):
// half the step's FP64 work moves to the FP32 pipe.  x and x' are rescaled
// together when x grows (the Newton ratio does not depend on their common
// scale).  A step that is non-finite or longer than `maxstep` (the FP32 polish
// had not converged there) leaves the prediction as it was; a zero
// subdiagonal (H already splits) leaves all of them.
template <class MH>
__device__ void newton64_shifts_lane(const int n, const MH &H, const MatIlv<float> &Hf, const VecIlv<double> &S,
                                     const VecIlv<double> &X, const VecIlv<float> &DX, const double maxstep)
{
    for (int i = 2; i <= n; ++i)
        if (H.ld(i, i - 1).r == 0.0) return;
    for (int k = 1; k <= n; ++k) {
        const cx<double> s = S.ld(k);
        if (nonfinite(s.r) || nonfinite(s.i)) continue;
        const cx<float> sf = mk((float)s.r, (float)s.i);
        X.st(n, mk(1.0, 0.0));
        DX.st(n, mk(0.f, 0.f));
        for (int i = n; i >= 2; --i) {
            const cx<double> xi = X.ld(i);
            const cx<float> xif = mk((float)xi.r, (float)xi.i);
            cx<double> acc = cmul(csub(H.ld(i, i), s), xi);
            cx<float> dacc = csub(cmul(csub(Hf.ld(i, i), sf), DX.ld(i)), xif);
            for (int j = i + 1; j <= n; ++j) {
                acc = cmac(acc, H.ld(i, j), X.ld(j));
                dacc = cmac(dacc, Hf.ld(i, j), DX.ld(j));
            }
            const double rs = -1.0 / H.ld(i, i - 1).r;
            cx<double> xn = cscal(acc, rs);
            cx<float> dxn = cscal(dacc, (float)rs);
            if (cabs1(xn) > 1e18) {
                for (int j = i; j <= n; ++j) {
                    X.st(j, cscal(X.ld(j), 1e-18));
                    DX.st(j, cscal(DX.ld(j), 1e-18f));
                }
                xn = cscal(xn, 1e-18);
                dxn = cscal(dxn, 1e-18f);
            }
            X.st(i - 1, xn);
            DX.st(i - 1, dxn);
        }
        const cx<double> x1 = X.ld(1);
        cx<double> r = cmul(csub(H.ld(1, 1), s), x1);
        cx<float> rp = csub(cmul(csub(Hf.ld(1, 1), sf), DX.ld(1)), mk((float)x1.r, (float)x1.i));
        for (int j = 2; j <= n; ++j) {
            r = cmac(r, H.ld(1, j), X.ld(j));
            rp = cmac(rp, Hf.ld(1, j), DX.ld(j));
        }
        const cx<double> delta = cdiv(r, mk((double)rp.r, (double)rp.i));
        if (!nonfinite(delta.r) && !nonfinite(delta.i) && cabs1(delta) <= maxstep) S.st(k, csub(s, delta));
    }
}

// kDefl64 (FP32 data only): the deflation test in FP64 (deflation_scan64).
template <class R, bool kSchur = true, bool kDefl64 = false, class MH, class MZ, class SP = NoShiftPredictions>
__device__ void zlahqr_warp(const int n, const MH &H, const MZ &Z, const bool valid, const int max_its,
                            int &nsweeps, int &status, SP *sp = nullptr)
{
    const R ulp = lim<R>::eps();
    const R smlnum = lim<R>::tiny() * (R(n) / ulp);
    if (valid) make_subdiag_real_lane<R, kSchur>(n, H, Z);

    // Lane state: active block L..I and the sweep count at this I.  As in the
    // reference, L only moves up while I stays, and resets to 1 when I moves.
    int I = n, L = 1, its = 0;
    bool done = !valid || n <= 1;
    for (;;) {
        bool sweep = false;
        cx<R> v0 = mk(R(0), R(0)), v1 = mk(R(0), R(0));
        if (!done) {
            for (;;) {
                if (I <= 1) { done = true; break; }
                if (its > max_its) { status |= ST_ITCAP; --I; L = 1; its = 0; continue; }
                L = deflation_scan_sel<R, kDefl64>(I, L, H, n, ulp, smlnum);
                if (L > 1) H.st(L, L - 1, mk(R(0), R(0)));
                if (L >= I) {
                    if (sp) sp->deflated(its);
                    --I; L = 1; its = 0;
                    continue;
                }
                cx<R> t = qr_shift<R>(I, L, its, H);
                if (sp) sp->template pick<R>(its, I, t, fabs(H.ld(I, I - 1).r));
                const cx<R> h11s = csub(H.ld(L, L), t);
                const R h21 = H.ld(L + 1, L).r;
                const R rs = frcp<R>(cabs1(h11s) + fabs(h21));
                v0 = cscal(h11s, rs);
                v1 = mk(h21 * rs, R(0));
                sweep = true;
                ++its;
                ++nsweeps;
                break;
            }
        }
        if (!__any_sync(FULL, sweep)) break;  // every lane is done
        const int Kmin = __reduce_min_sync(FULL, sweep ? L : INT_MAX);
        const int Kmax = __reduce_max_sync(FULL, sweep ? I - 1 : 0);
        for (int K = Kmin; K <= Kmax; ++K) {
            const bool act = sweep && K >= L && K <= I - 1;
            cx<R> t1 = mk(R(0), R(0)), w1 = mk(R(0), R(0));
            if (act) {
                cx<R> a0 = v0, a1 = v1;
                if (K > L) { a0 = H.ld(K, K - 1); a1 = H.ld(K + 1, K - 1); }
                zlarfg2<R>(a0, a1, t1);
                if (K > L) { H.st(K, K - 1, a0); H.st(K + 1, K - 1, mk(R(0), R(0))); }
                w1 = a1;
            }
            const R t2 = fma(t1.r, w1.r, -(t1.i * w1.i));
            if (kSchur) {
                if (act) {
                    // rows K, K+1 of H (columns K..n; wantT: I2 = n) and columns
                    // K, K+1 of Z (rows 1..n) in one loop: the two updates touch
                    // disjoint data, and interleaving them gives every iteration two
                    // independent rotation chains (the FP64 pipe's latency is hidden
                    // by 2 warps per scheduler otherwise).  Same arithmetic per element.
                    const cx<R> c1 = conj(t1), cw = conj(w1);
                    for (int j = 1; j <= n; ++j) {
                        cx<R> z1 = Z.ld(j, K), z2 = Z.ld(j, K + 1);
                        if (j >= K) {
                            cx<R> h1 = H.ld(K, j), h2 = H.ld(K + 1, j);
                            rot_pair(z1, z2, t1, t2, cw);
                            rot_pair(h1, h2, c1, t2, w1);
                            H.st(K, j, h1);
                            H.st(K + 1, j, h2);
                        } else {
                            rot_pair(z1, z2, t1, t2, cw);
                        }
                        Z.st(j, K, z1);
                        Z.st(j, K + 1, z2);
                    }
                }
            } else {
                // rows K, K+1, columns K..I (I2 = I, per lane)
                const cx<R> c1 = conj(t1);
                for (int j = K; j <= Kmax + 1; ++j) {
                    if (act && j <= I) {
                        cx<R> h1 = H.ld(K, j), h2 = H.ld(K + 1, j);
                        rot_pair(h1, h2, c1, t2, w1);
                        H.st(K, j, h1);
                        H.st(K + 1, j, h2);
                    }
                }
            }
            // columns K, K+1, rows I1..min(K+2, I) (I1 = 1, or L without the Schur
            // form), after the row update (they share the 2x2 block at K, K+1);
            // two rows per iteration for two independent chains
            const int je = (K + 2) < n ? (K + 2) : n;
            const cx<R> cw1 = conj(w1);
            int j = kSchur ? 1 : Kmin;
            for (; j + 1 <= je; j += 2) {
                const bool pa = act && j <= I && (kSchur || j >= L);
                const bool pb = act && j + 1 <= I && (kSchur || j + 1 >= L);
                cx<R> a1 = mk(R(0), R(0)), a2 = a1, b1 = a1, b2 = a1;
                if (pa) { a1 = H.ld(j, K); a2 = H.ld(j, K + 1); }
                if (pb) { b1 = H.ld(j + 1, K); b2 = H.ld(j + 1, K + 1); }
                rot_pair(a1, a2, t1, t2, cw1);
                rot_pair(b1, b2, t1, t2, cw1);
                if (pa) { H.st(j, K, a1); H.st(j, K + 1, a2); }
                if (pb) { H.st(j + 1, K, b1); H.st(j + 1, K + 1, b2); }
            }
            if (j <= je && act && j <= I && (kSchur || j >= L)) {
                cx<R> h1 = H.ld(j, K), h2 = H.ld(j, K + 1);
                rot_pair(h1, h2, t1, t2, cw1);
                H.st(j, K, h1);
                H.st(j, K + 1, h2);
            }
        }
        if (sweep) {
            // make H(I, I-1) real (reference :337-367)
            const cx<R> h = H.ld(I, I - 1);
            if (h.i != R(0)) {
                const R d = cabs(h);
                const cx<R> z = conj(cscal(h, frcp<R>(d)));
                H.st(I, I - 1, mk(d, R(0)));
                if (kSchur)
                    for (int j = I + 1; j <= n; ++j) H.st(I, j, cmul(H.ld(I, j), z));
                for (int j = kSchur ? 1 : L; j <= I - 1; ++j) H.st(j, I, cmulc(H.ld(j, I), z));
                if (kSchur)
                    for (int j = 1; j <= n; ++j) Z.st(j, I, cmulc(Z.ld(j, I), z));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// ztrevc: right eigenvectors of the upper-triangular T, back-transformed by
// the Schur vectors R in place (reference Toolbox.hpp:1133-1313 with the
// back substitution of :31-136; LAPACK ztrevc SIDE='R', HOWMNY='B').  The
// shifted diagonal T(k,k) - T(ki,ki), clamped to smin as in the reference, is
// formed on the fly, so T is read only.  x is held in the work vector `x`.
// Eigenvector ki comes out as R * [x; 1; 0], the reference's scaling.
//
// Overflow guard: the reference's back substitution has none (it omits the
// scaled solver zlatrs that LAPACK's ztrevc uses), so a defective T -- a
// Jordan block, whose shifted diagonal is clamped to smin ~ 1e-291 -- gives
// Inf/NaN vectors.  Here, whenever an entry of x would exceed `big`, the
// whole vector, including its unit entry, is scaled down; the result is then
// R * [s x; s; 0] for some 0 < s < 1, still an eigenvector.  When no entry
// gets that large (every well-posed case), s = 1 and the arithmetic is the
// reference's.
// ---------------------------------------------------------------------------
template <class R> struct trevc_lim;
template <> struct trevc_lim<double> { static __device__ __forceinline__ double big() { return 1e150; } };
template <> struct trevc_lim<float> { static __device__ __forceinline__ float big() { return 1e15f; } };

// Back substitution for column ki of the T-eigenvector matrix, in x(1:ki-1);
// returns the scale s of the unit entry.
template <class R, class MT, class V>
__device__ __forceinline__ R trevc_solve(const int ki, const MT &T, const V &x, const R smin, const cx<R> tkk)
{
    const R big = trevc_lim<R>::big();
    R s = R(1);
    for (int k = 1; k <= ki - 1; ++k) { const cx<R> v = T.ld(k, ki); x.st(k, mk(-v.r, -v.i)); }
    for (int j = ki - 1; j >= 1; --j) {
        cx<R> d = csub(T.ld(j, j), tkk);
        if (cabs1(d) < smin) d = mk(smin, R(0));
        cx<R> xj = x.ld(j);
        const R num = cabs1(xj), den = cabs1(d);
        if (num > big * den) {
            // x(j)/d would exceed big: scale x(1:ki-1) and the unit entry so that it is big
            const R f = (big * den) / num;
            for (int i = 1; i <= ki - 1; ++i) x.st(i, cscal(x.ld(i), f));
            xj = cscal(xj, f);
            s *= f;
        }
        xj = cdiv(xj, d);
        x.st(j, xj);
        for (int i = j - 1; i >= 1; --i) x.st(i, cnmac(x.ld(i), T.ld(i, j), xj));
    }
    return s;
}

template <class R, class MT, class MR, class V>
__device__ void ztrevc_lane(const int n, const MT &T, const MR &Rm, const V &x)
{
    const R ulp = lim<R>::eps();
    const R smlnum = lim<R>::tiny() * (R(n) / ulp);
    for (int ki = n; ki >= 2; --ki) {
        const cx<R> tkk = T.ld(ki, ki);
        const R smin = fmax(ulp * cabs1(tkk), smlnum);
        // back substitution with (T(1:ki-1,1:ki-1) - T(ki,ki) I)
        const R s = trevc_solve<R>(ki, T, x, smin, tkk);
        // R(:, ki) := R(:, 1:ki-1) x + s R(:, ki)
        for (int i = 1; i <= n; ++i) {
            cx<R> acc = Rm.ld(i, ki);
            if (s != R(1)) acc = cscal(acc, s);
            for (int j = 1; j <= ki - 1; ++j) acc = cmac(acc, Rm.ld(i, j), x.ld(j));
            Rm.st(i, ki, acc);
        }
    }
}

// ---------------------------------------------------------------------------
// Small BLAS-2 helpers of the reference's test surface.
// ---------------------------------------------------------------------------

// y := A x + beta y, or A^H x + beta y (reference zgemv_simple Toolbox.hpp:1033-1131
// on the full matrix; its Hermitian branch reads Re(y) for Im(y) (:1125) -- here
// the imaginary part is read).
template <class R, class M, class V>
__device__ void zgemv_lane(const bool herm, const int n, const M &A, const V &x, const cx<R> beta, const V &y)
{
    for (int i = 1; i <= n; ++i) y.st(i, cmul(y.ld(i), beta));
    if (!herm) {
        for (int j = 1; j <= n; ++j) {
            const cx<R> xj = x.ld(j);
            for (int i = 1; i <= n; ++i) y.st(i, cadd(y.ld(i), cmul(A.ld(i, j), xj)));
        }
    } else {
        for (int j = 1; j <= n; ++j) {
            cx<R> acc = mk(R(0), R(0));
            for (int i = 1; i <= n; ++i) acc = cadd(acc, cmulc(x.ld(i), A.ld(i, j)));
            y.st(j, cadd(y.ld(j), acc));
        }
    }
}

// Solve T x = b for upper-triangular T, b in x (reference Toolbox.hpp:31-136).
template <class R, class M, class V>
__device__ void backsubs_lane(const int n, const M &T, const V &x)
{
    for (int j = n; j >= 1; --j) {
        const cx<R> xj = cdiv(x.ld(j), T.ld(j, j));
        x.st(j, xj);
        for (int i = j - 1; i >= 1; --i) x.st(i, csub(x.ld(i), cmul(T.ld(i, j), xj)));
    }
}

}  // namespace ves
