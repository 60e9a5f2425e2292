// ves_mixed.cu -- mixed-precision form of the eigensolver: the whole
// reference path (zgehrd -> zunghr -> zlahqr -> ztrevc) in complex FP32, then
// every eigenpair refined by Newton's method with the residual in FP64.
//
// Why: on GB300 the FP32 pipe retires ~58x the FP64 pipe's FMAs, so the
// O(90 n^3) flops of the reduction and the QR sweeps are cheap in FP32; the
// FP64 work shrinks to the residuals r = A v - lambda v (4 n^2 FMAs per pair
// and step).
//
// Refinement of pair k (Newton on (A - lambda I) v = 0 with the component of v
// along the k-th Schur vector held fixed; Dongarra, Moler & Wilkinson,
// "Improving the accuracy of computed eigenvalues and eigenvectors", SIAM J.
// Numer. Anal. 20 (1983)).  With the FP32 Schur form A ~ Z T Z^H and the
// T-eigenvector x (x_k = 1, x_i = 0 for i > k):
//     r    = A v - lambda v                    FP64
//     r'   = Z^H r                             FP32
//     (T - lambda I) dx - dlambda x = -r', dx_k = 0:
//        rows i > k : back substitution for dx_i
//        row  k     : dlambda = r'_k + sum_{j>k} T_kj dx_j
//        rows i < k : back substitution including + dlambda x_i
//     v += Z dx, lambda += dlambda             FP64 update
// until ||r|| <= tol ||A||_F ||v|| (checked in FP64 on the final residual).
// A pair that does not converge in `max_steps` corrections, a matrix whose
// FP32 QR hit its sweep cap, or non-finite data sends the matrix to the FP64
// solver (a second launch over the list of such matrices), flagged in status.
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>
#include <cstdlib>

namespace ves {

namespace {

constexpr int kMixedThreads = 128;

__device__ __forceinline__ long long soa_mat_off_m(long long m, int n, int tc)
{
    return (m / tc) * (long long)tc * n * n + (m % tc);
}
__device__ __forceinline__ long long soa_vec_off_m(long long m, int n, int tc)
{
    return (m / tc) * (long long)tc * n + (m % tc);
}

// Per-slot (warp) workspace, every region [elements][32 lanes]:
//   V64 n*n double2 | T n*n float2 | Z n*n float2 | X n*n float2 | 4 vectors of n float2
__host__ __device__ __forceinline__ long long mixed_slot_bytes(int n)
{
    return 32LL * (16LL * n * n + 8LL * (3LL * n * n + 4LL * n));
}

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

__global__ void __launch_bounds__(kMixedThreads) fused_mixed_kernel(const MixedArgs a)
{
    const int n = a.g.n, tc = a.g.tc;
    const long long N = a.g.N;
    const int lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * (kMixedThreads / 32) + (threadIdx.x >> 5);
    const long long nslots = (long long)gridDim.x * (kMixedThreads / 32);
    const long long ngroups = (N + 31) / 32;

    char *sb = reinterpret_cast<char *>(a.ws) + slot * mixed_slot_bytes(n);
    const long long nn = (long long)n * n;
    double2 *pV = reinterpret_cast<double2 *>(sb) + lane;
    float2 *pT = reinterpret_cast<float2 *>(sb + 32LL * 16 * nn) + lane;
    float2 *pZ = pT + 32 * nn;
    float2 *pX = pZ + 32 * nn;
    float2 *pW = pX + 32 * nn;
    const MatIlv<double> V{pV, n};
    const MatIlv<float> T{pT, n}, Z{pZ, n}, X{pX, n};
    const VecIlv<float> tau{pW}, r32{pW + 32 * n}, rp{pW + 64 * n}, dx{pW + 96 * n};
    const double tol2 = a.tol * a.tol;

    for (long long g = slot; g < ngroups; g += nslots) {
        const long long m = g * 32 + lane;
        const bool valid = m < N;
        const long long mo = valid ? soa_mat_off_m(m, n, tc) : 0;
        const long long vo = valid ? soa_vec_off_m(m, n, tc) : 0;
        const MatSoA<double> A{const_cast<double *>(a.rA) + mo, const_cast<double *>(a.iA) + mo, tc, n};
        int status = 0, sweeps = 0;
        bool fb = false;  // hand this matrix to the FP64 solver
        float nA2 = 0.f;

        if (valid) {
            bool bad = false;
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) {
                    const cx<double> v = A.ld(i, j);
                    bad |= nonfinite(v.r) | nonfinite(v.i);
                    const cx<float> f = down(v);
                    nA2 += f.r * f.r + f.i * f.i;
                    T.st(i, j, f);
                }
            // FP32 range: entries beyond ~1e18 or a norm that overflows go to FP64
            fb = bad || !(nA2 < 1e36f);
            zgehrd_lane<float>(n, T, tau);
            zunghr_lane<float>(n, T, Z, tau);
            clear_below_subdiag_lane<float>(n, T);
        }
        zlahqr_warp<float>(n, T, Z, valid && !fb, a.max_its, sweeps, status);
        if (status & ST_ITCAP) fb = true;
        const bool work = valid && !fb;
        if (work) {
            trevc_x_lane<float>(n, T, pX);
            // initial eigenvectors V = Z X (X upper triangular), stored in FP64
            for (int k = 1; k <= n; ++k)
                for (int i = 1; i <= n; ++i) {
                    cx<float> acc = mk(0.f, 0.f);
                    for (int j = 1; j <= k; ++j) acc = cmac(acc, Z.ld(i, j), X.ld(j, k));
                    V.st(i, k, up(acc));
                }
        }

        // Newton refinement, pair by pair (k warp-uniform)
        for (int k = 1; k <= n; ++k) {
            cx<double> lam = work ? up(T.ld(k, k)) : mk(0.0, 0.0);
            bool act = work && !fb;
            for (int step = 0; step <= a.max_steps; ++step) {
                if (!__any_sync(FULL, act)) break;
                if (!act) continue;
                // FP64 residual
                double rn2 = 0.0, vn2 = 0.0;
                for (int i = 1; i <= n; ++i) {
                    const cx<double> vi = V.ld(i, k);
                    cx<double> acc = mk(-(lam.r * vi.r - lam.i * vi.i), -(lam.r * vi.i + lam.i * vi.r));
                    for (int j = 1; j <= n; ++j) acc = cmac(acc, A.ld(i, j), V.ld(j, k));
                    rn2 = fma(acc.i, acc.i, fma(acc.r, acc.r, rn2));
                    vn2 = fma(vi.i, vi.i, fma(vi.r, vi.r, vn2));
                    r32.st(i, down(acc));
                }
                if (rn2 <= tol2 * (double)nA2 * vn2) { act = false; continue; }
                if (step == a.max_steps) { fb = true; act = false; continue; }
                // FP32 correction through the Schur form
                for (int i = 1; i <= n; ++i) {
                    cx<float> s = mk(0.f, 0.f);
                    for (int j = 1; j <= n; ++j) s = cjmac(s, Z.ld(j, i), r32.ld(j));
                    rp.st(i, s);
                }
                const cx<float> l32 = down(lam);
                const float smin = fmax(lim<float>::eps() * cabs1(l32), lim<float>::tiny() * (float(n) / lim<float>::eps()));
                cx<float> dl = mk(0.f, 0.f);
                for (int i = n; i >= 1; --i) {
                    cx<float> s = rp.ld(i);
                    s = mk(-s.r, -s.i);
                    for (int j = i + 1; j <= n; ++j) s = cnmac(s, T.ld(i, j), dx.ld(j));
                    if (i == k) {  // dlambda x_k = r'_k + sum_{j>k} T_kj dx_j = -s
                        dl = cscal(mk(-s.r, -s.i), 1.f / X.ld(k, k).r);
                        dx.st(i, mk(0.f, 0.f));
                        continue;
                    }
                    if (i < k) s = cadd(s, cmul(dl, X.ld(i, k)));
                    cx<float> d = csub(T.ld(i, i), l32);
                    if (cabs1(d) < smin) d = mk(smin, 0.f);
                    dx.st(i, cdiv(s, d));
                }
                for (int i = 1; i <= n; ++i) {
                    cx<float> s = mk(0.f, 0.f);
                    for (int j = 1; j <= n; ++j) s = cmac(s, Z.ld(i, j), dx.ld(j));
                    V.st(i, k, cadd(V.ld(i, k), up(s)));
                }
                lam = cadd(lam, up(dl));
            }
            if (work && !fb) {
                const VecSoA<double> E{a.rE + vo, a.iE + vo, tc};
                E.st(k, lam);
            }
        }

        if (valid) {
            if (fb) {
                status |= ST_REFINE_FALLBACK;
                const int slotk = atomicAdd(a.fb_count, 1);
                a.fb_list[slotk] = (int)m;
            } else {
                const MatSoA<double> Vo{a.rV + mo, a.iV + mo, tc, n};
                for (int j = 1; j <= n; ++j) {
                    double scale = 1.0;
                    if (a.vnorm == 1) {
                        double mx = 0.0;
                        for (int i = 1; i <= n; ++i) mx = fmax(mx, cabs1(V.ld(i, j)));
                        scale = mx > 0.0 ? 1.0 / mx : 1.0;
                    } else if (a.vnorm == 2) {
                        double s2 = 0.0;
                        for (int i = 1; i <= n; ++i) { const cx<double> z = V.ld(i, j); s2 += z.r * z.r + z.i * z.i; }
                        scale = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
                    }
                    for (int i = 1; i <= n; ++i) Vo.st(i, j, cscal(V.ld(i, j), scale));
                }
            }
            if (a.status) a.status[m] = status;
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
    }
}

int g_mixed_blocks_per_sm = 2;

}  // namespace

size_t mixed_workspace_bytes(int n, long long N, int *out_blocks, int *out_threads)
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
            if (v >= 1 && v <= 16) g_mixed_blocks_per_sm = v;
        }
    }
    const long long groups = (N + 31) / 32;
    const int wpb = kMixedThreads / 32;
    long long blocks = std::min<long long>((groups + wpb - 1) / wpb, (long long)sms * g_mixed_blocks_per_sm);
    if (blocks < 1) blocks = 1;
    if (out_blocks) *out_blocks = (int)blocks;
    if (out_threads) *out_threads = kMixedThreads;
    return (size_t)mixed_slot_bytes(n) * (size_t)blocks * wpb;
}

cudaError_t launch_mixed(const MixedArgs &a, cudaStream_t st)
{
    if (a.g.N <= 0) return cudaSuccess;
    int blocks = 0, threads = 0;
    mixed_workspace_bytes(a.g.n, a.g.N, &blocks, &threads);
    fused_mixed_kernel<<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace ves
