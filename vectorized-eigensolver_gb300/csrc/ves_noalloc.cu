// ves_noalloc.cu -- ves_eigensolve_noalloc: the FP64 eigensolver for callers
// that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running where the allocator is
// owned by someone else (a framework's caching allocator, a memory-capped
// plugin host), code that must not allocate after start-up (real-time or
// certified pipelines that allocate once at initialisation), or code that
// must not synchronise the device, which cudaMalloc/cudaFree may do.  For
// them the solver's scratch space lives in a file-scope __device__ array
// that is part of the library image: every GPU that loads libves.so holds
// these kScratchBytes until the process exits.  The caller still passes the
// inputs and outputs.
//
// The array is shared by every call on a device and keeps whatever the last
// call left in it.  The solver writes every scratch element it reads (the
// working Hessenberg matrix, the Schur vectors and the work vector are
// produced from the input before use), so nothing has to start at zero.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads) race on the array and give wrong results: serialise them.
#include "ves.h"
#include "ves_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

namespace {

constexpr size_t kScratchBytes = VES_NOALLOC_SCRATCH_BYTES;  // 64 MiB per device
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The host-side name g_noalloc_scratch is a stand-in, not a device address;
// the address is looked up once per device, with that device current, and
// kept for the life of the process (a cudaDeviceReset() of the device would
// make it stale: the header tells callers not to use the entry point after
// one).
void *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mu;

// errors are reported through ves_last_error(), like every other entry point
int fail(int code, const char *msg)
{
    ves::set_error_message(msg);
    return code;
}

}  // namespace

extern "C" {

int ves_eigensolve_noalloc(int dim, int block_cnt, int thread_cnt, const double *rA, const double *iA, double *rE,
                           double *iE, double *rV, double *iV, int *status, void *stream)
{
    ves::set_error_message("");
    if (dim < 1 || dim > VES_NOALLOC_MAX_DIM)
        return fail(VES_ERR_ARG, "ves_eigensolve_noalloc: dim outside [1, VES_NOALLOC_MAX_DIM = 64]");
    if (block_cnt < 0 || thread_cnt < 1)
        return fail(VES_ERR_ARG, "ves_eigensolve_noalloc: need block_cnt >= 0 and thread_cnt >= 1");
    const long long N = (long long)block_cnt * thread_cnt;
    if (N == 0) return VES_OK;
    if (!rA || !iA || !rE || !iE || !rV || !iV) return fail(VES_ERR_ARG, "ves_eigensolve_noalloc: null pointer");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(VES_ERR_CUDA, "ves_eigensolve_noalloc: no usable CUDA device");
    ves::load_kernels();
    void *scratch = nullptr;
    {
        // Set-up, once per device, on this call's (current) device.
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return fail(VES_ERR_CUDA, "ves_eigensolve_noalloc: cudaGetSymbolAddress of the scratch array failed");
            }
            g_scratch_ptr[dev] = p;
        }
        scratch = g_scratch_ptr[dev];
    }

    // As many persistent warps as the array holds (4 warps per block), never
    // more than there are 32-matrix groups; each warp loops over groups.
    const long long per_warp = (2LL * dim * dim + dim) * 32 * (long long)sizeof(double2);
    const long long warps_fit = (long long)kScratchBytes / per_warp;  // >= 15 for dim <= 64
    if (warps_fit < 4) return fail(VES_ERR_ARG, "ves_eigensolve_noalloc: dim too large for the scratch array");
    const long long groups = (N + 31) / 32;
    const long long blocks = std::min<long long>((groups + 3) / 4, warps_fit / 4);

    ves::FusedArgs a{};
    a.g.n = dim;
    a.g.N = N;
    a.g.tc = thread_cnt;
    a.rA = rA; a.iA = iA;
    a.rE = rE; a.iE = iE;
    a.rV = rV; a.iV = iV;
    a.status = status;
    a.ws = scratch;
    a.max_its = 30;
    a.vnorm = VES_VNORM_REFERENCE;
    const cudaError_t e = ves::launch_fused_fp64_blocks(a, (int)blocks, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(VES_ERR_CUDA, "ves_eigensolve_noalloc: kernel launch failed");
    return VES_OK;
}

}  // extern "C"
