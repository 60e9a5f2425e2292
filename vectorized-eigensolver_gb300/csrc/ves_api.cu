// ves_api.cu -- the C ABI of libves.so (declared in include/ves.h).
//
// Drop-in layer: the reference's host entry points (utils.cpp) with host
// pointers and synchronous semantics.  Each call copies its inputs to device
// buffers that the library caches between calls (the reference allocates and
// frees them in every call, utils.cpp:178-214), runs the sm_103a kernels and
// copies the results back.
//
// Native layer: ves_* on device pointers, stream-ordered.
#include "ves.h"
#include "ves_internal.h"

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <array>
#include <mutex>
#include <string>
#include <vector>

namespace ves {

void load_kernels()
{
    static std::mutex mu;
    static std::vector<char> done;  // [device]
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    std::lock_guard<std::mutex> lk(mu);
    if ((int)done.size() <= d) done.resize(d + 1, 0);
    if (done[d]) return;
    done[d] = 1;
    load_mixed_kernels();
    load_fused_kernels();
    load_varsize_kernels();
    load_extras_kernels();
    load_shiftnet_kernels();
    cudaGetLastError();  // a failed load shows again, with its cause, at the launch
}

}  // namespace ves

namespace {

constexpr int kMaxDim = 512;

thread_local std::string t_last_error;

void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_last_error = buf;
}

// Start of every entry point that launches work: clear the calling thread's
// message and load the library's kernels on the current device (once).
void begin_call()
{
    t_last_error.clear();
    ves::load_kernels();
}

// Drop-in layer failures go to stderr as well: the reference API returns void.
void report(const char *where)
{
    fprintf(stderr, "libves: %s: %s\n", where, t_last_error.c_str());
}

bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
}

bool geom_ok(int dim, int block_cnt, int thread_cnt, ves::Geom *g)
{
    if (dim < 1 || dim > kMaxDim) { set_error("dim=%d outside [1, %d]", dim, kMaxDim); return false; }
    if (block_cnt < 0 || thread_cnt < 1) {
        set_error("block_cnt=%d thread_cnt=%d: need block_cnt >= 0, thread_cnt >= 1", block_cnt, thread_cnt);
        return false;
    }
    g->n = dim;
    g->N = (long long)block_cnt * thread_cnt;
    g->tc = thread_cnt;
    return true;
}

// Grow-only device buffers, one set per device, shared by the drop-in calls
// (serialised by a mutex).
struct Pool {
    std::mutex mu;
    struct Slot { void *p = nullptr; size_t n = 0; };
    std::vector<std::vector<Slot>> dev;  // [device][slot]

    void *get(int slot, size_t bytes)
    {
        int d = 0;
        if (cudaGetDevice(&d) != cudaSuccess) return nullptr;
        if ((int)dev.size() <= d) dev.resize(d + 1);
        if ((int)dev[d].size() <= slot) dev[d].resize(slot + 1);
        Slot &s = dev[d][slot];
        if (bytes == 0) bytes = 1;
        if (s.n >= bytes) return s.p;
        if (s.p) cudaFree(s.p);
        s.p = nullptr;
        s.n = 0;
        if (cudaMalloc(&s.p, bytes) != cudaSuccess) {
            cudaGetLastError();
            s.p = nullptr;
            return nullptr;
        }
        s.n = bytes;
        return s.p;
    }
    void release()
    {
        int cur = 0;
        cudaGetDevice(&cur);
        for (size_t d = 0; d < dev.size(); ++d) {
            if (cudaSetDevice((int)d) != cudaSuccess) continue;
            for (Slot &s : dev[d])
                if (s.p) cudaFree(s.p);
            dev[d].clear();
        }
        cudaSetDevice(cur);
    }
};
Pool &pool()
{
    static Pool *p = new Pool();  // never destroyed: freeing at exit races the CUDA runtime's teardown
    return *p;
}

// Scoped acquisition of the pool for one drop-in call.
struct Bufs {
    std::lock_guard<std::mutex> lk;
    Bufs() : lk(pool().mu) {}
    double *d(int slot, size_t count) { return static_cast<double *>(pool().get(slot, count * sizeof(double))); }
    void *raw(int slot, size_t bytes) { return pool().get(slot, bytes); }
};

bool h2d(void *dst, const void *src, size_t bytes) { return cuda_ok(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy H2D"); }
bool d2h(void *dst, const void *src, size_t bytes) { return cuda_ok(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "cudaMemcpy D2H"); }
bool sync_ok(const char *what) { return cuda_ok(cudaDeviceSynchronize(), what); }

#define NEED(ptr)                                                    \
    do {                                                             \
        if (!(ptr)) { set_error("device allocation failed"); return false; } \
    } while (0)

// Workspace of ves_eigensolve: the FP64 solver's slots, and for the mixed
// form also its FP32 slots, the fallback list and its counter (256-byte aligned).
struct WsPlan {
    size_t fp64, mixed, list, count, total;
};
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
WsPlan workspace_plan(int precision, int n, long long N, bool vectors, int bps)
{
    WsPlan p{};
    if (!vectors) {
        p.fp64 = align256(ves::eigvals_workspace_bytes(n, N, bps));
        p.total = p.fp64;
        return p;
    }
    // FP64: blocks_per_sm shapes the fused kernel; FP32 + refinement: it shapes
    // the FP32 Schur kernel and the FP64 fallback pass keeps the default grid
    const bool mixed = precision == VES_PREC_FP32_REFINE;
    p.fp64 = align256(ves::fused_workspace_bytes(n, N, mixed ? 0 : bps, nullptr, nullptr));
    if (mixed) {
        p.mixed = align256(ves::mixed_workspace_bytes(n, N, bps, nullptr, nullptr));
        p.list = align256((size_t)N * sizeof(int));
        p.count = 256;
    }
    p.total = p.fp64 + p.mixed + p.list + p.count;
    return p;
}

// ---------------------------------------------------------------------------
// Drop-in bodies (bool: success).
// ---------------------------------------------------------------------------
// Streams the asynchronous entry points fork work onto (the FP32+refine form's
// Schur / refinement overlap), two per device, created on first use; work on
// them is always ordered after and joined back into the caller's stream.
cudaStream_t library_stream(int k)
{
    static std::mutex mu;
    static std::vector<std::array<cudaStream_t, 2>> streams;  // [device][k]
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if ((int)streams.size() <= d) streams.resize(d + 1, std::array<cudaStream_t, 2>{nullptr, nullptr});
    cudaStream_t &st = streams[d][k];
    if (!st && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        st = nullptr;
    }
    return st;
}

// Streams of the drop-in eigensolver's copy/solve pipeline, created once per
// device (called with the pool mutex held).
cudaStream_t pipeline_stream(int k)
{
    static std::vector<std::array<cudaStream_t, 2>> streams;  // [device][k]
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return nullptr;
    if ((int)streams.size() <= d) streams.resize(d + 1, std::array<cudaStream_t, 2>{nullptr, nullptr});
    cudaStream_t &st = streams[d][k];
    if (!st && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        st = nullptr;
    }
    return st;
}

// The reference's eigensolver() on host buffers.  Whole SoA blocks of
// thread_cnt matrices are contiguous in every plane, so the batch is cut into
// chunks of blocks and two streams alternate chunks: while one chunk is being
// solved, the next one's input is copied in and the previous one's results are
// copied out.  Each stream has its own workspace, since two solves can be
// resident at once (which also fills the tail of each launch).  The issue
// order (next chunk's copy-in and solve before this chunk's copy-out) keeps the
// GPU busy even when the host buffers are pageable and copy-outs block the
// calling thread.  Results are the same as one launch over the whole batch:
// every matrix is solved by the same lane code whatever the grid.
bool do_eigensolver(int dim, int bc, int tc, double *rA, double *iA, double *rE, double *iE, double *rV, double *iV)
{
    ves::NvtxRange range("ves eigensolver (drop-in)");
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rA || !iA || !rE || !iE || !rV || !iV) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dAr = b.d(0, nm), *dAi = b.d(1, nm), *dVr = b.d(2, nm), *dVi = b.d(3, nm);
    double *dEr = b.d(4, nv), *dEi = b.d(5, nv);
    NEED(dAr); NEED(dAi); NEED(dVr); NEED(dVi); NEED(dEr); NEED(dEi);

    // Up to 16 chunks of at least 65,536 matrices (each launch's persistent grid
    // stays busy).  1,048,576 x 16x16 from pinned host buffers on GB300, chunks
    // -> ms per call: 8 -> 638, 12 -> 632, 16 -> 625, 24 -> 671, 32 -> 715 (the
    // device-resident solve: 621): the first copy-in and the last copy-out are
    // what is not hidden, and more, smaller launches leave more tails.
    constexpr long long kMinChunk = 65536;
    long long nchunks = std::min<long long>(16, std::max<long long>(1, g.N / kMinChunk));
    if (const char *e = getenv("VES_DROPIN_CHUNKS")) {  // tuning: the chunk count itself
        const int v = atoi(e);
        if (v >= 1 && v <= 64) nchunks = v;
    }
    nchunks = std::min<long long>(nchunks, bc);
    const long long cb = (bc + nchunks - 1) / nchunks;  // blocks per chunk
    nchunks = (bc + cb - 1) / cb;
    const size_t wsb = ves::fused_workspace_bytes(dim, cb * (long long)tc, 0, nullptr, nullptr);
    void *ws[2] = {b.raw(6, wsb), nchunks > 1 ? b.raw(9, wsb) : nullptr};
    NEED(ws[0]);
    if (nchunks > 1) NEED(ws[1]);
    cudaStream_t st[2] = {pipeline_stream(0), pipeline_stream(1)};
    if (!st[0] || !st[1]) { set_error("stream creation failed"); return false; }

    const size_t mstride = (size_t)tc * dim * dim, vstride = (size_t)tc * dim;  // elements per block
    auto chunk = [&](long long c, long long &b0, long long &nb) {
        b0 = c * cb;
        nb = std::min<long long>(cb, bc - b0);
    };
    auto copy_in_and_solve = [&](long long c) -> bool {
        ves::NvtxRange r("ves chunk: copy in + solve");
        long long b0, nb;
        chunk(c, b0, nb);
        cudaStream_t s = st[c & 1];
        const size_t mo = b0 * mstride, vo = b0 * vstride, mb = nb * mstride * 8;
        if (!cuda_ok(cudaMemcpyAsync(dAr + mo, rA + mo, mb, cudaMemcpyHostToDevice, s), "H2D") ||
            !cuda_ok(cudaMemcpyAsync(dAi + mo, iA + mo, mb, cudaMemcpyHostToDevice, s), "H2D"))
            return false;
        ves::FusedArgs a{};
        a.g = ves::Geom{dim, nb * (long long)tc, tc};
        a.rA = dAr + mo; a.iA = dAi + mo;
        a.rE = dEr + vo; a.iE = dEi + vo;
        a.rV = dVr + mo; a.iV = dVi + mo;
        a.rT = dAr + mo; a.iT = dAi + mo;  // A is overwritten with T, as in the reference
        a.ws = ws[c & 1];
        a.max_its = 30;
        a.vnorm = VES_VNORM_REFERENCE;
        return cuda_ok(ves::launch_fused_fp64(a, s), "eigensolver kernel launch");
    };
    auto copy_out = [&](long long c) -> bool {
        ves::NvtxRange r("ves chunk: copy out");
        long long b0, nb;
        chunk(c, b0, nb);
        cudaStream_t s = st[c & 1];
        const size_t mo = b0 * mstride, vo = b0 * vstride, mb = nb * mstride * 8, vb = nb * vstride * 8;
        return cuda_ok(cudaMemcpyAsync(rE + vo, dEr + vo, vb, cudaMemcpyDeviceToHost, s), "D2H") &&
               cuda_ok(cudaMemcpyAsync(iE + vo, dEi + vo, vb, cudaMemcpyDeviceToHost, s), "D2H") &&
               cuda_ok(cudaMemcpyAsync(rV + mo, dVr + mo, mb, cudaMemcpyDeviceToHost, s), "D2H") &&
               cuda_ok(cudaMemcpyAsync(iV + mo, dVi + mo, mb, cudaMemcpyDeviceToHost, s), "D2H") &&
               cuda_ok(cudaMemcpyAsync(rA + mo, dAr + mo, mb, cudaMemcpyDeviceToHost, s), "D2H") &&
               cuda_ok(cudaMemcpyAsync(iA + mo, dAi + mo, mb, cudaMemcpyDeviceToHost, s), "D2H");
    };
    bool ok = copy_in_and_solve(0);
    for (long long c = 0; ok && c < nchunks; ++c) {
        if (c + 1 < nchunks) ok = copy_in_and_solve(c + 1);
        ok = ok && copy_out(c);
    }
    ves::NvtxRange wait("ves eigensolver: wait");
    const bool s0 = cuda_ok(cudaStreamSynchronize(st[0]), "eigensolver stream 0");
    const bool s1 = cuda_ok(cudaStreamSynchronize(st[1]), "eigensolver stream 1");
    return ok && s0 && s1;
}

bool do_hessenberg(int dim, int bc, int tc, double *rA, double *iA, double *rQ, double *iQ)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rA || !iA || !rQ || !iQ) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dAr = b.d(0, nm), *dAi = b.d(1, nm), *dQr = b.d(2, nm), *dQi = b.d(3, nm);
    double *dtr = b.d(4, nv), *dti = b.d(5, nv);
    NEED(dAr); NEED(dAi); NEED(dQr); NEED(dQi); NEED(dtr); NEED(dti);
    if (!h2d(dAr, rA, nm * 8) || !h2d(dAi, iA, nm * 8)) return false;
    if (!cuda_ok(ves::launch_hessenberg(g, dAr, dAi, dQr, dQi, dtr, dti, 0), "hessenberg kernel launch")) return false;
    if (!sync_ok("hessenberg kernel")) return false;
    return d2h(rA, dAr, nm * 8) && d2h(iA, dAi, nm * 8) && d2h(rQ, dQr, nm * 8) && d2h(iQ, dQi, nm * 8);
}

bool do_zgehrd(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rA || !iA || !rtau || !itau) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dAr = b.d(0, nm), *dAi = b.d(1, nm), *dtr = b.d(4, nv), *dti = b.d(5, nv);
    NEED(dAr); NEED(dAi); NEED(dtr); NEED(dti);
    if (!h2d(dAr, rA, nm * 8) || !h2d(dAi, iA, nm * 8)) return false;
    // tau's last entry per matrix is not written by the reduction: keep the caller's values there
    if (!h2d(dtr, rtau, nv * 8) || !h2d(dti, itau, nv * 8)) return false;
    if (!cuda_ok(ves::launch_zgehrd(g, dAr, dAi, dtr, dti, 0), "zgehrd kernel launch")) return false;
    if (!sync_ok("zgehrd kernel")) return false;
    return d2h(rA, dAr, nm * 8) && d2h(iA, dAi, nm * 8) && d2h(rtau, dtr, nv * 8) && d2h(itau, dti, nv * 8);
}

bool do_zunghr(int dim, int bc, int tc, double *rA, double *iA, double *rtau, double *itau)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rA || !iA || !rtau || !itau) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dAr = b.d(0, nm), *dAi = b.d(1, nm), *dtr = b.d(4, nv), *dti = b.d(5, nv);
    NEED(dAr); NEED(dAi); NEED(dtr); NEED(dti);
    if (!h2d(dAr, rA, nm * 8) || !h2d(dAi, iA, nm * 8) || !h2d(dtr, rtau, nv * 8) || !h2d(dti, itau, nv * 8))
        return false;
    if (!cuda_ok(ves::launch_zunghr(g, dAr, dAi, dtr, dti, 0), "zunghr kernel launch")) return false;
    if (!sync_ok("zunghr kernel")) return false;
    return d2h(rA, dAr, nm * 8) && d2h(iA, dAi, nm * 8);
}

bool do_zlahqr(int dim, int bc, int tc, double *rE, double *iE, double *rM, double *iM, double *rS, double *iS)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rE || !iE || !rM || !iM || !rS || !iS) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dMr = b.d(0, nm), *dMi = b.d(1, nm), *dSr = b.d(2, nm), *dSi = b.d(3, nm);
    double *dEr = b.d(4, nv), *dEi = b.d(5, nv);
    NEED(dMr); NEED(dMi); NEED(dSr); NEED(dSi); NEED(dEr); NEED(dEi);
    if (!h2d(dMr, rM, nm * 8) || !h2d(dMi, iM, nm * 8)) return false;
    if (!cuda_ok(ves::launch_zlahqr(g, dEr, dEi, dMr, dMi, dSr, dSi, nullptr, 30, 0), "zlahqr kernel launch"))
        return false;
    if (!sync_ok("zlahqr kernel")) return false;
    return d2h(rE, dEr, nv * 8) && d2h(iE, dEi, nv * 8) && d2h(rM, dMr, nm * 8) && d2h(iM, dMi, nm * 8) &&
           d2h(rS, dSr, nm * 8) && d2h(iS, dSi, nm * 8);
}

bool do_ztrevc(int dim, int bc, int tc, double *rT, double *iT, double *rR, double *iR)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rT || !iT || !rR || !iR) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dTr = b.d(0, nm), *dTi = b.d(1, nm), *dRr = b.d(2, nm), *dRi = b.d(3, nm);
    double *dwr = b.d(4, nv), *dwi = b.d(5, nv);
    NEED(dTr); NEED(dTi); NEED(dRr); NEED(dRi); NEED(dwr); NEED(dwi);
    if (!h2d(dTr, rT, nm * 8) || !h2d(dTi, iT, nm * 8) || !h2d(dRr, rR, nm * 8) || !h2d(dRi, iR, nm * 8))
        return false;
    if (!cuda_ok(ves::launch_ztrevc(g, dTr, dTi, dRr, dRi, dwr, dwi, 0), "ztrevc kernel launch")) return false;
    if (!sync_ok("ztrevc kernel")) return false;
    return d2h(rR, dRr, nm * 8) && d2h(iR, dRi, nm * 8);
}

bool do_zgemv(bool herm, int dim, int bc, int tc, double *rM, double *iM, double *rx, double *ix, double *ry,
              double *iy, double rbeta, double ibeta)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rM || !iM || !rx || !ix || !ry || !iy) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dMr = b.d(0, nm), *dMi = b.d(1, nm), *dxr = b.d(4, nv), *dxi = b.d(5, nv);
    double *dyr = b.d(7, nv), *dyi = b.d(8, nv);
    NEED(dMr); NEED(dMi); NEED(dxr); NEED(dxi); NEED(dyr); NEED(dyi);
    if (!h2d(dMr, rM, nm * 8) || !h2d(dMi, iM, nm * 8) || !h2d(dxr, rx, nv * 8) || !h2d(dxi, ix, nv * 8) ||
        !h2d(dyr, ry, nv * 8) || !h2d(dyi, iy, nv * 8))
        return false;
    if (!cuda_ok(ves::launch_zgemv(g, herm, dMr, dMi, dxr, dxi, rbeta, ibeta, dyr, dyi, 0), "zgemv kernel launch"))
        return false;
    if (!sync_ok("zgemv kernel")) return false;
    return d2h(ry, dyr, nv * 8) && d2h(iy, dyi, nv * 8);
}

bool do_backsubs(int dim, int bc, int tc, double *rT, double *iT, double *rb, double *ib)
{
    ves::Geom g;
    if (!geom_ok(dim, bc, tc, &g)) return false;
    if (g.N == 0) return true;
    if (!rT || !iT || !rb || !ib) { set_error("null pointer"); return false; }
    const size_t nm = (size_t)g.N * dim * dim, nv = (size_t)g.N * dim;
    Bufs b;
    double *dTr = b.d(0, nm), *dTi = b.d(1, nm), *dbr = b.d(4, nv), *dbi = b.d(5, nv);
    NEED(dTr); NEED(dTi); NEED(dbr); NEED(dbi);
    if (!h2d(dTr, rT, nm * 8) || !h2d(dTi, iT, nm * 8) || !h2d(dbr, rb, nv * 8) || !h2d(dbi, ib, nv * 8))
        return false;
    if (!cuda_ok(ves::launch_backsubs(g, dTr, dTi, dbr, dbi, 0), "backsubstitution kernel launch")) return false;
    if (!sync_ok("backsubstitution kernel")) return false;
    return d2h(rb, dbr, nv * 8) && d2h(ib, dbi, nv * 8);
}

template <class F>
void dropin(const char *name, F f)
{
    begin_call();
    if (!f()) report(name);
}

int native(bool ok) { return ok ? VES_OK : (t_last_error.find("alloc") != std::string::npos ? VES_ERR_NOMEM : VES_ERR_CUDA); }

}  // namespace

namespace ves {
void set_error_message(const char *msg) { t_last_error = msg ? msg : ""; }
}  // namespace ves

#ifdef VES_BOUNDS_CHECK
namespace {
// the device counters of the bounds-checked build, one per translation unit
struct BoundsRegistry {
    std::mutex mu;
    std::vector<std::pair<unsigned long long (*)(), void (*)()>> counters;
};
BoundsRegistry &bounds_registry()
{
    static BoundsRegistry r;  // constructed on first use: the units register during static initialisation
    return r;
}
}  // namespace
namespace ves {
void register_bounds_counter(unsigned long long (*read)(), void (*reset)())
{
    std::lock_guard<std::mutex> lk(bounds_registry().mu);
    bounds_registry().counters.emplace_back(read, reset);
}
}  // namespace ves
#endif

namespace ves {

// The drop-in bodies behind the C names below and the C++ names of
// ves_dropin_cxx.cpp (the reference declares its host API with C++
// linkage, utils.h:37-65; the Cython module binds utils.cpp the same way).
void dropin_eigensolver(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rE, double *iE, double *rV,
                 double *iV)
{
    dropin("eigensolver", [&] { return do_eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV); });
}

void dropin_hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ)
{
    dropin("hessenberg", [&] { return do_hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ); });
}

void dropin_call_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    dropin("call_zgehrd", [&] { return do_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau); });
}

void dropin_call_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    dropin("call_zunghr", [&] { return do_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau); });
}

void dropin_call_zlahqr_new(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM, double *rS,
                     double *iS)
{
    dropin("call_zlahqr_new", [&] { return do_zlahqr(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS); });
}

void dropin_call_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR)
{
    dropin("call_ztrevc", [&] { return do_ztrevc(dim, block_cnt, thread_cnt, rT, iT, rR, iR); });
}

void dropin_call_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, double *rM, double *iM, double *rx, double *ix,
                double *ry, double *iy, double rbeta, double ibeta)
{
    dropin("call_zgemv", [&] {
        return do_zgemv(hermitian, dim, block_cnt, thread_cnt, rM, iM, rx, ix, ry, iy, rbeta, ibeta);
    });
}

void dropin_call_backsubstitution(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rb, double *ib)
{
    dropin("call_backsubstitution", [&] { return do_backsubs(dim, block_cnt, thread_cnt, rT, iT, rb, ib); });
}

void dropin_repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out)
{
    const long long n2 = (long long)dim * dim;
    for (long long e = 0; e < n2; ++e)
        for (long long b = 0; b < block_cnt; ++b)
            for (long long t = 0; t < thread_cnt; ++t) out[b * thread_cnt * n2 + e * thread_cnt + t] = matrix[e];
}

void dropin_repVectorSoA(int dim, int block_cnt, int thread_cnt, double *vec, double *out)
{
    for (long long e = 0; e < dim; ++e)
        for (long long b = 0; b < block_cnt; ++b)
            for (long long t = 0; t < thread_cnt; ++t) out[b * thread_cnt * dim + e * thread_cnt + t] = vec[e];
}

void dropin_rearrangeMatrices(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    const long long n2 = (long long)dim * dim;
    for (long long b = 0; b < block_cnt; ++b)
        for (long long t = 0; t < thread_cnt; ++t)
            for (long long e = 0; e < n2; ++e)
                out[b * thread_cnt * n2 + e * thread_cnt + t] = in[(b * thread_cnt + t) * n2 + e];
}

void dropin_arrangeMatricesAoS(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    const long long n2 = (long long)dim * dim;
    for (long long b = 0; b < block_cnt; ++b)
        for (long long t = 0; t < thread_cnt; ++t)
            for (long long e = 0; e < n2; ++e)
                out[(b * thread_cnt + t) * n2 + e] = in[b * thread_cnt * n2 + e * thread_cnt + t];
}

}  // namespace ves

extern "C" {

// ------------------------------- drop-in ----------------------------------
void eigensolver(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rE, double *iE,
                 double *rV, double *iV)
{
    ves::dropin_eigensolver(dim, block_cnt, thread_cnt, rA, iA, rE, iE, rV, iV);
}

void hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ)
{
    ves::dropin_hessenberg(dim, block_cnt, thread_cnt, rA, iA, rQ, iQ);
}

void call_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    ves::dropin_call_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau);
}

void call_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    ves::dropin_call_zunghr(dim, block_cnt, thread_cnt, rA, iA, rtau, itau);
}

void call_zlahqr_new(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM,
                     double *rS, double *iS)
{
    ves::dropin_call_zlahqr_new(dim, block_cnt, thread_cnt, rE, iE, rM, iM, rS, iS);
}

void call_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR)
{
    ves::dropin_call_ztrevc(dim, block_cnt, thread_cnt, rT, iT, rR, iR);
}

void call_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, double *rM, double *iM, double *rx,
                double *ix, double *ry, double *iy, double rbeta, double ibeta)
{
    ves::dropin_call_zgemv(hermitian, dim, block_cnt, thread_cnt, rM, iM, rx, ix, ry, iy, rbeta, ibeta);
}

void call_backsubstitution(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rb, double *ib)
{
    ves::dropin_call_backsubstitution(dim, block_cnt, thread_cnt, rT, iT, rb, ib);
}

void repMatrixSoA(int dim, int block_cnt, int thread_cnt, double *matrix, double *out)
{
    ves::dropin_repMatrixSoA(dim, block_cnt, thread_cnt, matrix, out);
}

void repVectorSoA(int dim, int block_cnt, int thread_cnt, double *vec, double *out)
{
    ves::dropin_repVectorSoA(dim, block_cnt, thread_cnt, vec, out);
}

void rearrangeMatrices(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    ves::dropin_rearrangeMatrices(dim, block_cnt, thread_cnt, in, out);
}

void arrangeMatricesAoS(int dim, int block_cnt, int thread_cnt, double *in, double *out)
{
    ves::dropin_arrangeMatricesAoS(dim, block_cnt, thread_cnt, in, out);
}

// -------------------------------- native ----------------------------------
void ves_default_options(ves_options *opt)
{
    if (!opt) return;
    memset(opt, 0, sizeof *opt);
    opt->precision = VES_PREC_FP64;
    opt->max_its = 30;
    opt->vnorm = VES_VNORM_REFERENCE;
    opt->refine_steps = 8;
    opt->refine_tol = 5e-14;
    opt->want_vectors = 1;
    opt->blocks_per_sm = 0;
    opt->varsize_order = 0;
    opt->shift_sweeps = 1;
    opt->shift_gate = 0.f;
    opt->shift_polish = 0;
    opt->work_counts = nullptr;
}

size_t ves_eigensolve_workspace_size(int dim, int block_cnt, int thread_cnt, const ves_options *opt)
{
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return 0;
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    return workspace_plan(o.precision, dim, g.N, o.want_vectors != 0, o.blocks_per_sm).total;
}

int ves_eigensolve(int dim, int block_cnt, int thread_cnt, const double *rA, const double *iA, double *rE, double *iE,
                   double *rV, double *iV, double *rT, double *iT, int *status, int *sweeps, const ves_options *opt,
                   void *workspace, size_t workspace_bytes, void *stream)
{
    begin_call();
    ves::NvtxRange range("ves_eigensolve");
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    if (g.N == 0) return VES_OK;
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    const bool vectors = o.want_vectors != 0;
    if (!rA || !iA || !rE || !iE || (vectors && (!rV || !iV)) || (!rT) != (!iT)) {
        set_error("null pointer");
        return VES_ERR_ARG;
    }
    if (!vectors && (rT || o.precision != VES_PREC_FP64)) {
        set_error("eigenvalues only (want_vectors = 0) runs in FP64 and returns no Schur form");
        return VES_ERR_UNSUPPORTED;
    }
    if (o.precision != VES_PREC_FP64 && o.precision != VES_PREC_FP32_REFINE) {
        set_error("precision mode %d unknown", o.precision);
        return VES_ERR_ARG;
    }
    if (o.precision == VES_PREC_FP32_REFINE && rT) {
        set_error("the Schur form output needs precision VES_PREC_FP64");
        return VES_ERR_UNSUPPORTED;
    }
    if (o.precision == VES_PREC_FP32_REFINE && dim > 64) {
        set_error("precision VES_PREC_FP32_REFINE supports dim <= 64 (dim=%d)", dim);
        return VES_ERR_UNSUPPORTED;
    }
    if (o.max_its < 0 || o.max_its > 10000) { set_error("max_its=%d outside [0, 10000]", o.max_its); return VES_ERR_ARG; }
    if (o.vnorm < 0 || o.vnorm > 2) { set_error("vnorm=%d unknown", o.vnorm); return VES_ERR_ARG; }
    if (o.blocks_per_sm < 0 || o.blocks_per_sm > 16) {
        set_error("blocks_per_sm=%d outside [0, 16]", o.blocks_per_sm);
        return VES_ERR_ARG;
    }
    if (o.refine_steps < 0 || o.refine_steps > 100 || !(o.refine_tol > 0.0)) {
        set_error("refine_steps=%d / refine_tol=%g out of range", o.refine_steps, o.refine_tol);
        return VES_ERR_ARG;
    }
    const WsPlan plan = workspace_plan(o.precision, dim, g.N, vectors, o.blocks_per_sm);
    const size_t need = plan.total;
    void *ws = workspace;
    std::unique_lock<std::mutex> lk;
    if (!ws) {
        lk = std::unique_lock<std::mutex>(pool().mu);
        ws = pool().get(15, need);
        if (!ws) { set_error("device allocation of %zu workspace bytes failed", need); return VES_ERR_NOMEM; }
    } else if (workspace_bytes < need || ((uintptr_t)ws & 255)) {
        set_error("workspace: %zu bytes given, %zu needed (256-byte aligned)", workspace_bytes, need);
        return VES_ERR_ARG;
    }
    ves::FusedArgs a{};
    a.g = g;
    a.rA = rA; a.iA = iA;
    a.rE = rE; a.iE = iE;
    a.rV = rV; a.iV = iV;
    a.rT = rT; a.iT = iT;
    a.status = status; a.sweeps = sweeps;
    a.ws = ws;
    a.max_its = o.max_its;
    a.vnorm = o.vnorm;
    a.blocks_per_sm = o.precision == VES_PREC_FP64 ? o.blocks_per_sm : 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (!vectors)
        return native(cuda_ok(
            ves::launch_eigvals(g, rA, iA, rE, iE, status, sweeps, ws, o.max_its, o.blocks_per_sm, st),
            "eigenvalues kernel launch"));
    if (o.precision == VES_PREC_FP64)
        return native(cuda_ok(ves::launch_fused_fp64(a, st), "eigensolve kernel launch"));

    char *base = static_cast<char *>(ws);
    int *list = reinterpret_cast<int *>(base + plan.fp64 + plan.mixed);
    int *count = reinterpret_cast<int *>(base + plan.fp64 + plan.mixed + plan.list);
    if (!cuda_ok(cudaMemsetAsync(count, 0, sizeof(int), st), "fallback counter reset")) return VES_ERR_CUDA;
    ves::MixedArgs m{};
    m.g = g;
    m.rA = rA; m.iA = iA;
    m.rE = rE; m.iE = iE;
    m.rV = rV; m.iV = iV;
    m.status = status; m.sweeps = sweeps;
    m.ws = base + plan.fp64;
    m.max_its = o.max_its;
    m.vnorm = o.vnorm;
    m.max_steps = o.refine_steps;
    m.tol = o.refine_tol;
    m.fb_list = list;
    m.fb_count = count;
    m.blocks_per_sm = o.blocks_per_sm;
    m.work = o.work_counts;
    // refinement steps with a float-float residual: 2 (default) or 1; VES_MIXED_FF_STEPS overrides (tuning)
    m.ff_steps = 2;
    if (const char *ff = getenv("VES_MIXED_FF_STEPS"))
        if (ff[0] == '1' || ff[0] == '2') m.ff_steps = ff[0] - '0';
    // The Schur stage of one chunk overlaps the refinement of the previous one on
    // two library streams (forked from and joined back into the caller's);
    // VES_MIXED_OVERLAP=0 runs the two stages one after the other on the caller's
    // stream.  So does a call whose stream is being captured: the library streams
    // are shared by every caller on the device, and forking them into one
    // caller's capture would pull other callers' work into that graph.
    // Overlap pays for n >= 32; below, the stages measured faster one after the
    // other on GB300 (FP32+refine eigensolves/s, serial against overlapped: n=8
    // 47.9 / 44.8 M/s, n=16 (group Schur kernel) 7.04 / 5.17, n=20 (warp Schur
    // kernel) 3.78 / 3.05, n=24 2.42 / 2.23, n=28 1.60 / 1.48; n=32 1.095 / 1.106).
    // VES_MIXED_OVERLAP=1 / 0 forces it on / off.
    const char *ov = getenv("VES_MIXED_OVERLAP");
    const bool overlap = ov && (ov[0] == '0' || ov[0] == '1') ? ov[0] == '1' : dim >= 32;
    cudaStream_t s_schur = nullptr, s_refine = nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!cuda_ok(cudaStreamIsCapturing(st, &cap), "cudaStreamIsCapturing")) return VES_ERR_CUDA;
    if (overlap && cap == cudaStreamCaptureStatusNone) {
        s_schur = library_stream(0);
        s_refine = library_stream(1);
    }
    const cudaError_t me = (s_schur && s_refine) ? ves::launch_mixed_overlap(m, st, s_schur, s_refine)
                                                 : ves::launch_mixed(m, st);
    if (!cuda_ok(me, "mixed-precision kernel launch")) return VES_ERR_CUDA;
    a.list = list;
    a.list_count = count;
    return native(cuda_ok(ves::launch_fp64_list(a, st), "fallback kernel launch"));
}

size_t ves_polyroots_workspace_size(int degree, int block_cnt, int thread_cnt)
{
    ves::Geom g;
    if (!geom_ok(degree, block_cnt, thread_cnt, &g)) return 0;
    return align256(ves::eigvals_workspace_bytes(degree, g.N, 0));
}

int ves_polyroots(int degree, int block_cnt, int thread_cnt, const double *rC, const double *iC, double *rR,
                  double *iR, int *status, void *workspace, size_t workspace_bytes, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(degree, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    if (g.N == 0) return VES_OK;
    if (!rC || !iC || !rR || !iR) { set_error("null pointer"); return VES_ERR_ARG; }
    const size_t need = align256(ves::eigvals_workspace_bytes(degree, g.N, 0));
    void *ws = workspace;
    std::unique_lock<std::mutex> lk;
    if (!ws) {
        lk = std::unique_lock<std::mutex>(pool().mu);
        ws = pool().get(14, need);
        if (!ws) { set_error("device allocation of %zu workspace bytes failed", need); return VES_ERR_NOMEM; }
    } else if (workspace_bytes < need || ((uintptr_t)ws & 255)) {
        set_error("workspace: %zu bytes given, %zu needed (256-byte aligned)", workspace_bytes, need);
        return VES_ERR_ARG;
    }
    return native(cuda_ok(ves::launch_polyroots(g, rC, iC, rR, iR, status, ws, 30, (cudaStream_t)stream),
                          "polyroots kernel launch"));
}

static int transpose_call(bool to_soa, bool vec, int dim, int block_cnt, int thread_cnt, const double *re_in,
                          const double *im_in, double *re_out, double *im_out, const void *z_in, void *z_out,
                          int row_major, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    if (g.N == 0) return VES_OK;
    const void *zp = to_soa ? z_in : z_out;
    if (!zp || (to_soa ? (!re_out || !im_out) : (!re_in || !im_in))) { set_error("null pointer"); return VES_ERR_ARG; }
    if ((uintptr_t)zp & 15) { set_error("the interleaved complex array must be 16-byte aligned"); return VES_ERR_ARG; }
    const long long len = vec ? dim : (long long)dim * dim;
    return native(cuda_ok(ves::launch_transpose(to_soa, re_in, im_in, re_out, im_out, static_cast<const double *>(z_in),
                                                static_cast<double *>(z_out), g.N, dim, len, thread_cnt,
                                                !vec && row_major != 0, (cudaStream_t)stream),
                          "transpose launch"));
}

int ves_soa_from_complex(int dim, int block_cnt, int thread_cnt, const void *z, int row_major, double *re, double *im,
                         void *stream)
{
    return transpose_call(true, false, dim, block_cnt, thread_cnt, nullptr, nullptr, re, im, z, nullptr, row_major,
                          stream);
}

int ves_complex_from_soa(int dim, int block_cnt, int thread_cnt, const double *re, const double *im, int row_major,
                         void *z, void *stream)
{
    return transpose_call(false, false, dim, block_cnt, thread_cnt, re, im, nullptr, nullptr, nullptr, z, row_major,
                          stream);
}

int ves_soa_vec_from_complex(int dim, int block_cnt, int thread_cnt, const void *z, double *re, double *im,
                             void *stream)
{
    return transpose_call(true, true, dim, block_cnt, thread_cnt, nullptr, nullptr, re, im, z, nullptr, 0, stream);
}

int ves_complex_from_soa_vec(int dim, int block_cnt, int thread_cnt, const double *re, const double *im, void *z,
                             void *stream)
{
    return transpose_call(false, true, dim, block_cnt, thread_cnt, re, im, nullptr, nullptr, nullptr, z, 0, stream);
}

// Workspace of ves_eigensolve_shifts: the shift-seeded kernel's slots, and
// for the polish pre-pass (shift_polish > 0, dim <= 32) the polished
// predictions (two SoA vector planes).
struct ShiftsPlan {
    size_t fused, polish, total;
};
ShiftsPlan shifts_plan(int dim, long long N, const ves_options &o)
{
    ShiftsPlan p{};
    p.fused = align256(ves::fused_workspace_bytes(dim, N, o.blocks_per_sm, nullptr, nullptr, true));
    p.polish = (o.shift_polish > 0 && dim <= 32) ? align256((size_t)N * dim * 2 * sizeof(double)) : 0;
    p.total = p.fused + p.polish;
    return p;
}

size_t ves_eigensolve_shifts_workspace_size(int dim, int block_cnt, int thread_cnt, const ves_options *opt)
{
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g) || dim > 64) return 0;
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    return shifts_plan(dim, g.N, o).total;
}

int ves_eigensolve_shifts(int dim, int block_cnt, int thread_cnt, const double *rA, const double *iA, double *rE,
                          double *iE, double *rV, double *iV, const double *rS, const double *iS, int *status,
                          int *sweeps, int *fallbacks, const ves_options *opt, void *workspace,
                          size_t workspace_bytes, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    if (dim > 64) { set_error("learned shifts support dim <= 64"); return VES_ERR_UNSUPPORTED; }
    if (g.N == 0) return VES_OK;
    if (!rA || !iA || !rE || !iE || !rV || !iV || !rS || !iS) { set_error("null pointer"); return VES_ERR_ARG; }
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    if (o.max_its < 0 || o.max_its > 10000 || o.vnorm < 0 || o.vnorm > 2 || o.shift_sweeps < 0 ||
        o.shift_sweeps > 9 || o.blocks_per_sm < 0 || o.blocks_per_sm > 16 || !(o.shift_gate >= 0.f) ||
        o.shift_gate > 1e6f || o.shift_polish < 0 || o.shift_polish > 64) {
        set_error("option out of range");
        return VES_ERR_ARG;
    }
    const ShiftsPlan plan = shifts_plan(dim, g.N, o);
    const size_t need = plan.total;
    void *ws = workspace;
    std::unique_lock<std::mutex> lk;
    if (!ws) {
        lk = std::unique_lock<std::mutex>(pool().mu);
        ws = pool().get(12, need);
        if (!ws) { set_error("device allocation of %zu workspace bytes failed", need); return VES_ERR_NOMEM; }
    } else if (workspace_bytes < need || ((uintptr_t)ws & 255)) {
        set_error("workspace: %zu bytes given, %zu needed (256-byte aligned)", workspace_bytes, need);
        return VES_ERR_ARG;
    }
    ves::FusedArgs a{};
    a.g = g;
    a.rA = rA; a.iA = iA; a.rE = rE; a.iE = iE; a.rV = rV; a.iV = iV;
    a.status = status; a.sweeps = sweeps;
    a.ws = ws;
    a.max_its = o.max_its;
    a.vnorm = o.vnorm;
    a.rS = rS; a.iS = iS;
    a.shift_sweeps = o.shift_sweeps;
    a.shift_gate = o.shift_gate;
    a.shift_polish = o.shift_polish;
    // with the polish, one FP64 Newton step per prediction on the solve's own
    // Hessenberg matrix; VES_POLISH_FP64_STEP=0 / 2 takes none / two (tuning)
    const char *f64s = getenv("VES_POLISH_FP64_STEP");
    a.shift_newton64 = o.shift_polish > 0 ? ((f64s && (f64s[0] == '0' || f64s[0] == '2')) ? f64s[0] - '0' : 1) : 0;
    a.fallbacks = fallbacks;
    a.blocks_per_sm = o.blocks_per_sm;
    cudaStream_t st = (cudaStream_t)stream;
    if (plan.polish) {
        // n <= 32: polish in a warp-per-matrix FP32 pre-pass, the solve reads the result
        double *rP = reinterpret_cast<double *>(static_cast<char *>(ws) + plan.fused);
        double *iP = rP + (size_t)g.N * dim;
        if (!cuda_ok(ves::launch_polish32(g, rA, iA, rS, iS, rP, iP, o.shift_polish, o.work_counts, st), "shift polish launch"))
            return VES_ERR_CUDA;
        a.rS = rP;
        a.iS = iP;
        a.shift_polish = 0;
    }
    return native(cuda_ok(ves::launch_fused_fp64(a, st), "learned-shift solve launch"));
}

int ves_gemm_bf16(int M, int N, int K, const void *A, int lda, const void *Bt, int ldb, const float *bias, int act,
                  void *C, float *Cf, int ldc, int *err, void *stream)
{
    begin_call();
    if (M < 0 || N < 0 || K < 0 || (K & 7) || (lda & 7) || (ldb & 7) || lda < K || ldb < K || ldc < N ||
        act < 0 || act > 1) {
        set_error("gemm: bad sizes (K, lda, ldb must be multiples of 8, lda, ldb >= K, ldc >= N)");
        return VES_ERR_ARG;
    }
    if ((M && K && !A) || (N && K && !Bt) || (!C && !Cf) || ((uintptr_t)A & 15) || ((uintptr_t)Bt & 15)) {
        set_error("gemm: null or misaligned pointer");
        return VES_ERR_ARG;
    }
    return native(cuda_ok(ves::launch_gemm_bf16(M, N, K, A, lda, Bt, ldb, bias, act, C, Cf, ldc, err,
                                                (cudaStream_t)stream),
                          "gemm launch"));
}

static int varsize_bps(const ves_options &o) { return o.blocks_per_sm > 0 ? o.blocks_per_sm : 4; }

size_t ves_eigensolve_varsize_workspace_size(long long count, int max_dim, const ves_options *opt)
{
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    if (count < 0 || max_dim < 1 || max_dim > VES_VARSIZE_MAX_DIM) return 0;
    return align256(ves::varsize_workspace_bytes(count, max_dim, varsize_bps(o)));
}

static int varsize_check(long long count, int max_dim, const int *dims, const double *rA, const double *iA,
                         const double *rE, const double *iE, const double *rV, const double *iV,
                         const ves_options &o)
{
    if (count < 0 || count > (1LL << 31) - 1) { set_error("count=%lld out of range", count); return VES_ERR_ARG; }
    if (max_dim < 1 || max_dim > VES_VARSIZE_MAX_DIM) {
        set_error("max_dim=%d outside [1, VES_VARSIZE_MAX_DIM=%d]", max_dim, VES_VARSIZE_MAX_DIM);
        return VES_ERR_ARG;
    }
    if (count > 0 && (!dims || !rA || !iA || !rE || !iE || !rV || !iV)) { set_error("null pointer"); return VES_ERR_ARG; }
    if (o.precision != VES_PREC_FP64 || !o.want_vectors) {
        set_error("mixed-size batches run the FP64 eigenvalue-and-vector path");
        return VES_ERR_UNSUPPORTED;
    }
    if (o.max_its < 0 || o.max_its > 10000 || o.vnorm < 0 || o.vnorm > 2 || o.blocks_per_sm < 0 ||
        o.blocks_per_sm > 16 || o.varsize_order < 0 || o.varsize_order > 1) {
        set_error("option out of range");
        return VES_ERR_ARG;
    }
    return VES_OK;
}

int ves_eigensolve_varsize(long long count, int max_dim, const int *dims, const double *rA, const double *iA,
                           double *rE, double *iE, double *rV, double *iV, int *status, int *sweeps,
                           const ves_options *opt, void *workspace, size_t workspace_bytes, void *stream)
{
    begin_call();
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    int rc = varsize_check(count, max_dim, dims, rA, iA, rE, iE, rV, iV, o);
    if (rc != VES_OK || count == 0) return rc;
    const size_t need = align256(ves::varsize_workspace_bytes(count, max_dim, varsize_bps(o)));
    void *ws = workspace;
    std::unique_lock<std::mutex> lk;
    if (!ws) {
        lk = std::unique_lock<std::mutex>(pool().mu);
        ws = pool().get(13, need);
        if (!ws) { set_error("device allocation of %zu workspace bytes failed", need); return VES_ERR_NOMEM; }
    } else if (workspace_bytes < need || ((uintptr_t)ws & 255)) {
        set_error("workspace: %zu bytes given, %zu needed (256-byte aligned)", workspace_bytes, need);
        return VES_ERR_ARG;
    }
    return native(cuda_ok(ves::launch_varsize(count, max_dim, dims, rA, iA, rE, iE, rV, iV, status, sweeps, ws,
                                              o.max_its, o.vnorm, varsize_bps(o), o.varsize_order,
                                              (cudaStream_t)stream),
                          "mixed-size solve launch"));
}

}  // extern "C"

struct ves_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

int ves_graph_capture_varsize(ves_graph **out, long long count, int max_dim, const int *dims, const double *rA,
                              const double *iA, double *rE, double *iE, double *rV, double *iV, int *status,
                              int *sweeps, const ves_options *opt, void *workspace, size_t workspace_bytes)
{
    begin_call();
    if (!out) { set_error("null pointer"); return VES_ERR_ARG; }
    *out = nullptr;
    ves_options o;
    ves_default_options(&o);
    if (opt) o = *opt;
    int rc = varsize_check(count, max_dim, dims, rA, iA, rE, iE, rV, iV, o);
    if (rc != VES_OK) return rc;
    const size_t need = align256(ves::varsize_workspace_bytes(count, max_dim, varsize_bps(o)));
    if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) {
        set_error("graph capture needs a caller workspace of %zu bytes (256-byte aligned)", need);
        return VES_ERR_ARG;
    }
    cudaStream_t cs = nullptr;
    if (!cuda_ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream")) return VES_ERR_CUDA;
    ves_graph *g = new ves_graph();
    bool ok = cuda_ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (ok) {
        const cudaError_t le = ves::launch_varsize(count, max_dim, dims, rA, iA, rE, iE, rV, iV, status, sweeps,
                                                   workspace, o.max_its, o.vnorm, varsize_bps(o), o.varsize_order, cs);
        const cudaError_t ee = cudaStreamEndCapture(cs, &g->graph);
        ok = cuda_ok(le, "captured launch") && cuda_ok(ee, "end capture");
    }
    if (ok) ok = cuda_ok(cudaGraphInstantiate(&g->exec, g->graph, 0), "graph instantiate");
    cudaStreamDestroy(cs);
    if (!ok) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        delete g;
        return VES_ERR_CUDA;
    }
    *out = g;
    return VES_OK;
}

int ves_graph_launch(ves_graph *graph, void *stream)
{
    begin_call();
    if (!graph || !graph->exec) { set_error("null graph"); return VES_ERR_ARG; }
    return native(cuda_ok(cudaGraphLaunch(graph->exec, (cudaStream_t)stream), "graph launch"));
}

void ves_graph_destroy(ves_graph *graph)
{
    if (!graph) return;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
}

int ves_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_zgehrd(g, rA, iA, rtau, itau, (cudaStream_t)stream), "zgehrd launch"));
}

int ves_zunghr(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, const double *rtau, const double *itau,
               void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_zunghr(g, rA, iA, rtau, itau, (cudaStream_t)stream), "zunghr launch"));
}

int ves_hessenberg(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rQ, double *iQ,
                   double *rtau, double *itau, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_hessenberg(g, rA, iA, rQ, iQ, rtau, itau, (cudaStream_t)stream), "hessenberg launch"));
}

int ves_zlahqr(int dim, int block_cnt, int thread_cnt, double *rE, double *iE, double *rM, double *iM, double *rS,
               double *iS, int *status, int max_its, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    if (max_its < 0 || max_its > 10000) { set_error("max_its=%d outside [0, 10000]", max_its); return VES_ERR_ARG; }
    return native(cuda_ok(ves::launch_zlahqr(g, rE, iE, rM, iM, rS, iS, status, max_its, (cudaStream_t)stream),
                          "zlahqr launch"));
}

int ves_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rR, double *iR, double *rwork,
               double *iwork, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_ztrevc(g, rT, iT, rR, iR, rwork, iwork, (cudaStream_t)stream), "ztrevc launch"));
}

int ves_zgemv(bool hermitian, int dim, int block_cnt, int thread_cnt, const double *rM, const double *iM,
              const double *rx, const double *ix, double *ry, double *iy, double rbeta, double ibeta, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_zgemv(g, hermitian, rM, iM, rx, ix, rbeta, ibeta, ry, iy, (cudaStream_t)stream),
                          "zgemv launch"));
}

int ves_backsubstitution(int dim, int block_cnt, int thread_cnt, const double *rT, const double *iT, double *rb,
                         double *ib, void *stream)
{
    begin_call();
    ves::Geom g;
    if (!geom_ok(dim, block_cnt, thread_cnt, &g)) return VES_ERR_ARG;
    return native(cuda_ok(ves::launch_backsubs(g, rT, iT, rb, ib, (cudaStream_t)stream), "backsubstitution launch"));
}

int ves_fp64_fma_rate(double *flops_per_s, void *stream)
{
    begin_call();
    if (!flops_per_s) { set_error("null pointer"); return VES_ERR_ARG; }
    return native(cuda_ok(ves::fp64_fma_rate(flops_per_s, (cudaStream_t)stream), "fp64 probe"));
}

int ves_fp32_fma_rate(double *flops_per_s, void *stream)
{
    begin_call();
    if (!flops_per_s) { set_error("null pointer"); return VES_ERR_ARG; }
    return native(cuda_ok(ves::fp32_fma_rate(flops_per_s, (cudaStream_t)stream), "fp32 probe"));
}

int ves_bounds_violations(unsigned long long *count, int reset)
{
    if (!count) { set_error("ves_bounds_violations: null pointer"); return VES_ERR_ARG; }
    *count = 0;
#ifdef VES_BOUNDS_CHECK
    std::lock_guard<std::mutex> lk(bounds_registry().mu);
    for (auto &c : bounds_registry().counters) {
        *count += c.first();
        if (reset) c.second();
    }
    return VES_OK;
#else
    (void)reset;
    set_error("ves_bounds_violations: this library was built without VES_BOUNDS_CHECK");
    return VES_ERR_UNSUPPORTED;
#endif
}

int ves_partition_blocks(int block_cnt, int parts, int part, int *first_block, int *n_blocks)
{
    if (block_cnt < 0 || parts < 1 || part < 0 || part >= parts || !first_block || !n_blocks) {
        set_error("ves_partition_blocks: need block_cnt >= 0, parts >= 1, 0 <= part < parts");
        return VES_ERR_ARG;
    }
    // the first (block_cnt % parts) parts get one block more
    const int base = block_cnt / parts, extra = block_cnt % parts;
    *n_blocks = base + (part < extra ? 1 : 0);
    *first_block = part * base + (part < extra ? part : extra);
    return VES_OK;
}

const char *ves_last_error(void) { return t_last_error.c_str(); }

void ves_release(void)
{
    std::lock_guard<std::mutex> lk(pool().mu);
    pool().release();
}

int ves_version(void) { return 100; }

}  // extern "C"
