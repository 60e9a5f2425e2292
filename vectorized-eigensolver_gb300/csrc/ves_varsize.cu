// ves_varsize.cu -- uneven-size batching: one solve over matrices of mixed
// order n (1..VES_VARSIZE_MAX_DIM), binned on the device by n and run by one
// persistent kernel, the whole sequence capturable in a CUDA graph.
//
// Packed layout (device pointers): matrix m has order dims[m]; its dims[m]^2
// elements are stored column-major and contiguous at element offset
// sum_{j<m} dims[j]^2 of the real and imaginary planes; its eigenvalues at
// sum_{j<m} dims[j]; its eigenvectors in the same layout as A.
//
// Sequence (no host synchronisation, so it can be captured):
//   1. offsets      two-level exclusive scans of dims^2 and dims
//   2. bin          histogram of n, exclusive scan over bins, scatter of
//                   matrix indices into n-sorted order
//   3. work items   groups of up to 32 equal-n matrices, largest n first
//                   (longest-processing-time order) or natural order
//   4. solve        persistent warps take items from an atomic counter; the
//                   32 lanes of an item run the lockstep FP64 path of the
//                   fixed-size solver (same routines), one matrix per lane
// The lockstep routines need all lanes of a warp at the same n; binning is
// what lets a mixed batch keep them full.
#include "ves_device.cuh"
#include "ves_internal.h"

#include <algorithm>

namespace ves {

namespace {

constexpr int kMaxVarDim = 64;
constexpr int kScanBlock = 1024;
constexpr int kSolveThreads = 128;

struct Item {
    int n;
    int count;     // matrices in this group (1..32)
    long long at;  // first position in the n-sorted index array
};

// ---- 1. exclusive scans of dims^2 and dims (two levels) -------------------
__global__ void scan_blocks_kernel(const int *dims, long long count, long long *aoff, long long *eoff,
                                   long long *bsum_a, long long *bsum_e)
{
    __shared__ long long sa[kScanBlock], se[kScanBlock];
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    // the layout counts every matrix at its stated size, solvable or not
    const int d = i < count ? max(dims[i], 0) : 0;
    sa[threadIdx.x] = (long long)d * d;
    se[threadIdx.x] = d;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {  // Hillis-Steele inclusive scan
        long long va = threadIdx.x >= off ? sa[threadIdx.x - off] : 0;
        long long ve = threadIdx.x >= off ? se[threadIdx.x - off] : 0;
        __syncthreads();
        sa[threadIdx.x] += va;
        se[threadIdx.x] += ve;
        __syncthreads();
    }
    if (i < count) {
        aoff[i] = sa[threadIdx.x] - (long long)d * d;
        eoff[i] = se[threadIdx.x] - d;
    }
    if (threadIdx.x == kScanBlock - 1) {
        bsum_a[blockIdx.x] = sa[threadIdx.x];
        bsum_e[blockIdx.x] = se[threadIdx.x];
    }
}

__global__ void scan_sums_kernel(long long *bsum_a, long long *bsum_e, long long nblocks)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long ra = 0, re = 0;  // serial: nblocks = count / 1024
    for (long long b = 0; b < nblocks; ++b) {
        const long long a = bsum_a[b], e = bsum_e[b];
        bsum_a[b] = ra;
        bsum_e[b] = re;
        ra += a;
        re += e;
    }
}

__global__ void scan_apply_kernel(long long *aoff, long long *eoff, const long long *bsum_a, const long long *bsum_e,
                                  long long count)
{
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < count) {
        aoff[i] += bsum_a[blockIdx.x];
        eoff[i] += bsum_e[blockIdx.x];
    }
}

// ---- 2. binning by n ------------------------------------------------------
__global__ void histogram_kernel(const int *dims, long long count, int maxd, int *hist)
{
    __shared__ int h[kMaxVarDim + 1];
    for (int b = threadIdx.x; b <= kMaxVarDim; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int d = dims[i];
        if (d >= 1 && d <= maxd) atomicAdd(&h[d], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= kMaxVarDim; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], h[b]);
}

// bin starts, cursors, and the work-item list (one thread; 64 bins)
__global__ void plan_kernel(const int *hist, long long *bin_start, long long *cursor, Item *items, int *nitems,
                            int order)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long s = 0;
    for (int b = 0; b <= kMaxVarDim; ++b) {
        bin_start[b] = s;
        cursor[b] = s;
        s += hist[b];
    }
    int it = 0;
    for (int k = 0; k < kMaxVarDim; ++k) {
        const int b = order == 0 ? kMaxVarDim - k : k + 1;  // 0: largest n first
        for (long long at = bin_start[b]; at < bin_start[b] + hist[b]; at += 32) {
            Item x;
            x.n = b;
            x.count = (int)min(32LL, bin_start[b] + hist[b] - at);
            x.at = at;
            items[it++] = x;
        }
    }
    *nitems = it;
}

// Matrices of order outside [1, maxd] are left out of the bins and flagged.
__global__ void scatter_kernel(const int *dims, long long count, int maxd, long long *cursor, int *sorted, int *status)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int d = dims[i];
        if (d >= 1 && d <= maxd) {
            const long long pos = atomicAdd(reinterpret_cast<unsigned long long *>(&cursor[d]), 1ULL);
            sorted[pos] = (int)i;
        } else if (status) {
            status[i] = ST_BAD_DIM;
        }
    }
}

// ---- 4. persistent solve ---------------------------------------------------
struct VarArgs {
    const double *rA, *iA;
    double *rE, *iE, *rV, *iV;
    int *status, *sweeps;
    const long long *aoff, *eoff;
    const int *sorted;
    const Item *items;
    const int *nitems;
    int *next_item;
    void *ws;
    int max_dim;  // sizes the per-warp workspace
    int max_its;
    int vnorm;
};

__global__ void __launch_bounds__(kSolveThreads) varsize_solve_kernel(const VarArgs a)
{
    const int lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * (kSolveThreads / 32) + (threadIdx.x >> 5);
    const int MD = a.max_dim;
    double2 *base = reinterpret_cast<double2 *>(a.ws) + slot * (2LL * MD * MD + MD) * 32 + lane;
    const int total = *a.nitems;
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.next_item, 1);
        it = __shfl_sync(FULL, it, 0);
        if (it >= total) break;
        const Item item = a.items[it];
        const int n = item.n;
        const MatIlv<double> H{base, n};
        const MatIlv<double> Z{base + (long long)n * n * 32, n};
        const VecIlv<double> W{base + 2LL * n * n * 32};
        const bool valid = lane < item.count;
        const long long m = valid ? a.sorted[item.at + lane] : 0;
        const long long ao = valid ? a.aoff[m] : 0, eo = valid ? a.eoff[m] : 0;
        int status = 0, sweeps = 0;
        if (valid) {
            const MatSoA<double> A{const_cast<double *>(a.rA) + ao, const_cast<double *>(a.iA) + ao, 1, n};
            bool bad = false;
            for (int j = 1; j <= n; ++j)
                for (int i = 1; i <= n; ++i) {
                    const cx<double> v = A.ld(i, j);
                    bad |= nonfinite(v.r) | nonfinite(v.i);
                    H.st(i, j, v);
                }
            if (bad) status |= ST_NONFINITE;
            zgehrd_lane<double>(n, H, W);
            zunghr_lane<double>(n, H, Z, W);
            clear_below_subdiag_lane<double>(n, H);
        }
        zlahqr_warp<double>(n, H, Z, valid && !(status & ST_NONFINITE), a.max_its, sweeps, status);
        if (valid) {
            const VecSoA<double> E{a.rE + eo, a.iE + eo, 1};
            for (int k = 1; k <= n; ++k) E.st(k, H.ld(k, k));
            ztrevc_lane<double>(n, H, Z, W);
            const MatSoA<double> V{a.rV + ao, a.iV + ao, 1, n};
            for (int j = 1; j <= n; ++j) {
                double scale = 1.0;
                if (a.vnorm == 1) {
                    double mx = 0.0;
                    for (int i = 1; i <= n; ++i) mx = fmax(mx, cabs1(Z.ld(i, j)));
                    scale = mx > 0.0 ? 1.0 / mx : 1.0;
                } else if (a.vnorm == 2) {
                    double s2 = 0.0;
                    for (int i = 1; i <= n; ++i) { const cx<double> z = Z.ld(i, j); s2 = fma(z.i, z.i, fma(z.r, z.r, s2)); }
                    scale = s2 > 0.0 ? 1.0 / sqrt(s2) : 1.0;
                }
                for (int i = 1; i <= n; ++i) V.st(i, j, cscal(Z.ld(i, j), scale));
            }
            if (a.status) a.status[m] = status;
            if (a.sweeps) a.sweeps[m] = sweeps;
        }
    }
}

inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

struct VarPlan {
    size_t aoff, eoff, bsa, bse, hist, bstart, cursor, items, nitems, next, sorted, slots, total;
    long long nblocks, nslots;
};

VarPlan var_plan(long long count, int max_dim, int blocks_per_sm)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    VarPlan p{};
    p.nblocks = (count + kScanBlock - 1) / kScanBlock;
    const long long max_items = count / 32 + kMaxVarDim + 1;
    const long long solve_blocks = std::max<long long>(1, std::min<long long>((max_items + 3) / 4,
                                                                               (long long)sms * blocks_per_sm));
    p.nslots = solve_blocks * (kSolveThreads / 32);
    size_t o = 0;
    p.aoff = o; o += al(count * 8);
    p.eoff = o; o += al(count * 8);
    p.bsa = o; o += al(p.nblocks * 8);
    p.bse = o; o += al(p.nblocks * 8);
    p.hist = o; o += al((kMaxVarDim + 1) * 4);
    p.bstart = o; o += al((kMaxVarDim + 1) * 8);
    p.cursor = o; o += al((kMaxVarDim + 1) * 8);
    p.items = o; o += al(max_items * sizeof(Item));
    p.nitems = o; o += 256;
    p.next = o; o += 256;
    p.sorted = o; o += al(count * 4);
    p.slots = o; o += al((size_t)p.nslots * (2ULL * max_dim * max_dim + max_dim) * 32 * sizeof(double2));
    p.total = o;
    return p;
}

}  // namespace

size_t varsize_workspace_bytes(long long count, int max_dim, int blocks_per_sm)
{
    return var_plan(count, max_dim, blocks_per_sm).total;
}

cudaError_t launch_varsize(long long count, int max_dim, const int *dims, const double *rA, const double *iA,
                           double *rE, double *iE, double *rV, double *iV, int *status, int *sweeps, void *ws,
                           int max_its, int vnorm, int blocks_per_sm, int order, cudaStream_t st)
{
    if (count <= 0) return cudaSuccess;
    const VarPlan p = var_plan(count, max_dim, blocks_per_sm);
    char *w = static_cast<char *>(ws);
    long long *aoff = reinterpret_cast<long long *>(w + p.aoff);
    long long *eoff = reinterpret_cast<long long *>(w + p.eoff);
    long long *bsa = reinterpret_cast<long long *>(w + p.bsa);
    long long *bse = reinterpret_cast<long long *>(w + p.bse);
    int *hist = reinterpret_cast<int *>(w + p.hist);
    long long *bstart = reinterpret_cast<long long *>(w + p.bstart);
    long long *cursor = reinterpret_cast<long long *>(w + p.cursor);
    Item *items = reinterpret_cast<Item *>(w + p.items);
    int *nitems = reinterpret_cast<int *>(w + p.nitems);
    int *next = reinterpret_cast<int *>(w + p.next);
    int *sorted = reinterpret_cast<int *>(w + p.sorted);
    cudaError_t e;
    if ((e = cudaMemsetAsync(hist, 0, (kMaxVarDim + 1) * 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(next, 0, 4, st)) != cudaSuccess) return e;
    scan_blocks_kernel<<<(unsigned)p.nblocks, kScanBlock, 0, st>>>(dims, count, aoff, eoff, bsa, bse);
    scan_sums_kernel<<<1, 32, 0, st>>>(bsa, bse, p.nblocks);
    scan_apply_kernel<<<(unsigned)p.nblocks, kScanBlock, 0, st>>>(aoff, eoff, bsa, bse, count);
    const unsigned hb = (unsigned)std::min<long long>((count + 255) / 256, 4096);
    histogram_kernel<<<hb, 256, 0, st>>>(dims, count, max_dim, hist);
    plan_kernel<<<1, 32, 0, st>>>(hist, bstart, cursor, items, nitems, order);
    scatter_kernel<<<hb, 256, 0, st>>>(dims, count, max_dim, cursor, sorted, status);
    VarArgs a{};
    a.rA = rA; a.iA = iA; a.rE = rE; a.iE = iE; a.rV = rV; a.iV = iV;
    a.status = status; a.sweeps = sweeps;
    a.aoff = aoff; a.eoff = eoff; a.sorted = sorted; a.items = items; a.nitems = nitems; a.next_item = next;
    a.ws = w + p.slots; a.max_dim = max_dim; a.max_its = max_its; a.vnorm = vnorm;
    varsize_solve_kernel<<<(unsigned)(p.nslots / (kSolveThreads / 32)), kSolveThreads, 0, st>>>(a);
    return cudaGetLastError();
}

void load_varsize_kernels()
{
    load_kernel(varsize_solve_kernel);
    load_kernel(scan_blocks_kernel);
    load_kernel(scan_sums_kernel);
    load_kernel(scan_apply_kernel);
    load_kernel(histogram_kernel);
    load_kernel(plan_kernel);
    load_kernel(scatter_kernel);
}

}  // namespace ves
