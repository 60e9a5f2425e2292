// ves_tc.cuh -- a BF16 GEMM on the 5th-generation tensor cores (tcgen05) for
// the learned-shift network:  C[M x N] = A[M x K] * B[K x N] (+ bias, GELU).
//
//   A   row-major M x K (K-major), BF16, leading dimension lda (multiple of 8)
//   Bt  B transposed: row-major N x K (K-major), BF16, leading dimension ldb
//   C   row-major M x N: BF16 act(A*B + bias) and/or FP32 A*B + bias (the
//       pre-activation, kept for the GELU backward pass in training)
//
// One CTA of 128 threads computes a 128-row x NT-column tile.  K is consumed in
// chunks of 32: the 4 warps stage the A and B chunks into shared memory in the
// canonical no-swizzle K-major layout (8-row x 16-byte core matrices, core
// matrices adjacent in K 128 bytes apart, adjacent in M/N 512 bytes apart), one
// elected thread issues two tcgen05.mma (M=128, N=NT, K=16) accumulating in
// tensor memory (TMEM), tcgen05.commit signals an mbarrier when they are done.
// The epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM lanes /
// rows 32w..32w+31), adds the bias, applies GELU and stores.
//
// Every wait on the mbarrier is bounded: on timeout the kernel records an
// error, stops issuing work, and still releases its TMEM columns.
#pragma once

#include <cuda.h>  // CUtensorMap (the TMA tensor-map type)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace ves {
namespace tc {

constexpr int kKC = 32;            // K per shared-memory chunk (4 core-matrix columns)
constexpr int kM = 128;            // rows per CTA (UMMA M)
constexpr unsigned kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (no swizzle, K-major).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);       // start address
    d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;   // leading-dimension byte offset (K direction)
    d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;   // stride-dimension byte offset (M/N direction)
    d |= (uint64_t)1 << 46;                        // descriptor version for this architecture
    return d;                                      // base offset 0, layout SWIZZLE_NONE
}

// Instruction descriptor: kind::f16, BF16 x BF16 -> FP32, both K-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N)
{
    return (1u << 4)                   // D format: F32
           | (1u << 7)                 // A format: BF16
           | (1u << 10)                // B format: BF16
           | ((uint32_t)(N >> 3) << 17)
           | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// Bounded wait for phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    const uint32_t a = smem_addr(bar);
    for (unsigned it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem_d), "l"(da), "l"(db), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float x)
{
    // tanh form of GELU (Hendrycks & Gimpel 2016)
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    return 0.5f * x * (1.f + tanhf(k0 * (x + k1 * x * x * x)));
}

// NT: columns per CTA (16..256, multiple of 16).  grid = (ceil(M/128), ceil(N/NT)).
//
// Split K (gridDim.z > 1, the weight gradients of training, where K is the
// batch): CTA z takes the K range [z * kz, (z + 1) * kz), kz a multiple of 32,
// and writes its FP32 partial product to Cf + z * zstride (no bias, no C);
// the caller sums the partials.
template <int NT>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *Bt,
                                                        int ldb, int M, int N, int K, const float *bias, int act,
                                                        __nv_bfloat16 *C, float *Cf, int ldc, int *err,
                                                        long long zstride = 0)
{
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
    constexpr int kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));  // TMEM columns
    __shared__ __align__(1024) unsigned char sA[kM * kKC * 2];
    __shared__ __align__(1024) unsigned char sB[NT * kKC * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kM, n0 = blockIdx.y * NT;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    constexpr uint32_t idesc = make_idesc(kM, NT);

    unsigned phase = 0;
    // this CTA's K range (the whole of K unless split)
    const int kz = gridDim.z > 1 ? (K + (int)gridDim.z * kKC - 1) / ((int)gridDim.z * kKC) * kKC : K;
    const int kb = (int)blockIdx.z * kz, ke = min(K, kb + kz);
    if (gridDim.z > 1) {
        Cf += (long long)blockIdx.z * zstride;
        bias = nullptr;
        C = nullptr;
    }
    const int nchunks = ke > kb ? (ke - kb + kKC - 1) / kKC : 0;
    for (int c = 0; c < nchunks && !failed; ++c) {
        const int k0 = kb + c * kKC;
        // stage A: 128 rows x 8 core columns of 16 bytes
        constexpr int kcs = kKC / 8;  // core-matrix columns per chunk
        for (int p = tid; p < kM * kcs; p += 128) {
            const int r = p / kcs, kc = p % kcs, k = k0 + kc * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (m0 + r < M && k < ke) v = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * lda + k);
            *reinterpret_cast<uint4 *>(sA + ((r >> 3) * kcs + kc) * 128 + (r & 7) * 16) = v;
        }
        for (int p = tid; p < NT * kcs; p += 128) {
            const int r = p / kcs, kc = p % kcs, k = k0 + kc * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n0 + r < N && k < ke) v = *reinterpret_cast<const uint4 *>(Bt + (size_t)(n0 + r) * ldb + k);
            *reinterpret_cast<uint4 *>(sB + ((r >> 3) * kcs + kc) * 128 + (r & 7) * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // smem writes -> tensor core (async proxy)
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int s = 0; s < kKC / 16; ++s) {
                const uint64_t da = make_desc(smem_addr(sA) + s * 256, 128, (kKC / 8) * 128);
                const uint64_t db = make_desc(smem_addr(sB) + s * 256, 128, (kKC / 8) * 128);
                mma_bf16(tmem, da, db, idesc, (c > 0 || s > 0) ? 1u : 0u);
            }
            mma_commit(&bar);
        }
        const bool ok = mbar_wait(&bar, phase);
        phase ^= 1;
        if (!ok) failed = 1;
        __syncthreads();  // the chunk's MMAs are done: shared memory may be overwritten
    }
    asm volatile("tcgen05.fence::after_thread_sync;");

    if (!failed) {
        const int row = m0 + warp * 32 + lane;
        for (int cb = 0; cb < NT; cb += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            if (nchunks == 0)  // an empty K range (split K): nothing was accumulated
                for (int i = 0; i < 16; ++i) v[i] = 0.f;
            if (row < M) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int col = n0 + cb + i;
                    if (col < N) {
                        const float z = v[i] + (bias ? bias[col] : 0.f);  // pre-activation
                        if (Cf) Cf[(size_t)row * ldc + col] = z;
                        if (C) C[(size_t)row * ldc + col] = __float2bfloat16(act == 1 ? gelu(z) : z);
                    }
                }
            }
        }
    } else if (tid == 0 && err) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// ---------------------------------------------------------------------------
// Persistent variant for K <= 256 (the network's layers): the CTA keeps the
// whole N-tile of B (the weights, NT x K) in shared memory for all its M-tiles
// and stages each 128 x K A-tile whole, so one tcgen05.commit covers the K/16
// MMAs of a tile.  The A-tile of the CTA's next M-tile is fetched with cp.async
// while the epilogue of the current one drains TMEM; the epilogue stores 16
// consecutive columns per thread as 16-byte vectors.  Dynamic shared memory:
// (128 + NT) * K * 2 bytes (192 KB at K = 256, NT = 256).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(uint32_t saddr, const void *g, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(saddr), "l"(g), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// rows x K (K-major) from global into the no-swizzle core-matrix layout;
// rows past `valid` are zero-filled
__device__ __forceinline__ void stage_rows(unsigned char *dst, const __nv_bfloat16 *src, int ld, int rows, int valid,
                                           int K)
{
    const int kcs = K / 8;  // 16-byte core-matrix columns
    const uint32_t base = smem_addr(dst);
    for (int p = threadIdx.x; p < rows * kcs; p += blockDim.x) {
        const int r = p / kcs, kc = p % kcs;
        const bool ok = r < valid;
        const __nv_bfloat16 *g = ok ? src + (size_t)r * ld + kc * 8 : src;
        cp_async16(base + (uint32_t)(((r >> 3) * kcs + kc) * 128 + (r & 7) * 16), g, ok ? 16u : 0u);
    }
}

template <int NT>
__global__ void __launch_bounds__(128) gemm_bf16_persistent_kernel(const __nv_bfloat16 *A, int lda,
                                                                   const __nv_bfloat16 *Bt, int ldb, int M, int N,
                                                                   int K, const float *bias, int act,
                                                                   __nv_bfloat16 *C, float *Cf, int ldc, int *err)
{
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
    constexpr int kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) unsigned char dsm[];
    unsigned char *sA = dsm;
    unsigned char *sB = dsm + (size_t)kM * K * 2;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.y * NT;
    const int mtiles = (M + kM - 1) / kM;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    int tile = blockIdx.x;
    // B (this CTA's N-tile, all of K) and the first A-tile
    stage_rows(sB, Bt + (size_t)n0 * ldb, ldb, NT, N - n0, K);
    if (tile < mtiles) stage_rows(sA, A + (size_t)tile * kM * lda, lda, kM, M - tile * kM, K);
    cp_async_wait_all();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    constexpr uint32_t idesc = make_idesc(kM, NT);
    const uint32_t sbo = (uint32_t)(K / 8) * 128;

    unsigned phase = 0;
    for (; tile < mtiles && !failed; tile += gridDim.x) {
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            for (int s = 0; s < K / 16; ++s) {
                const uint64_t da = make_desc(smem_addr(sA) + s * 256, 128, sbo);
                const uint64_t db = make_desc(smem_addr(sB) + s * 256, 128, sbo);
                mma_bf16(tmem, da, db, idesc, s > 0 ? 1u : 0u);
            }
            mma_commit(&bar);
        }
        const bool ok = mbar_wait(&bar, phase);
        phase ^= 1;
        if (!ok) failed = 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        __syncthreads();  // every thread saw the MMAs complete (or the failure)
        if (failed) break;
        // the MMAs have read sA: fetch the next tile's A while draining TMEM
        const int next = tile + gridDim.x;
        if (next < mtiles) stage_rows(sA, A + (size_t)next * kM * lda, lda, kM, M - next * kM, K);
        const int row = tile * kM + warp * 32 + lane;
        for (int cb = 0; cb < NT; cb += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            const int col = n0 + cb;
            if (row < M && col < N) {  // N is a multiple of 16: a chunk is all in or all out
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] += bias ? bias[col + i] : 0.f;
                if (Cf) {
                    float4 *dst = reinterpret_cast<float4 *>(Cf + (size_t)row * ldc + col);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
                if (C) {
                    uint32_t pk[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float x0 = act == 1 ? gelu(v[2 * q]) : v[2 * q];
                        const float x1 = act == 1 ? gelu(v[2 * q + 1]) : v[2 * q + 1];
                        __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
                        pk[q] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(C + (size_t)row * ldc + col);
                    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            }
        }
        cp_async_wait_all();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // next A staged, TMEM drained
    }
    if (failed) {
        // a wait gave up: give in-flight MMAs one more bounded wait, report, free TMEM
        if (tid == 0) (void)mbar_wait(&bar, phase ^ 1);
        if (tid == 0 && err) atomicExch(err, 1);
        cp_async_wait_all();
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// ---------------------------------------------------------------------------
// The persistent GEMM with its operands loaded by the Tensor Memory Accelerator
// (cp.async.bulk.tensor): one thread issues, per 16-byte column of K, a 2-D box
// of 8 elements x 128 rows of A (x NT rows of B) from a tensor map.  A box
// lands row after row, 16 bytes a row, so each box is a column of core
// matrices: M-adjacent core matrices 128 bytes apart (stride-dimension offset)
// and K-adjacent ones a box apart (leading-dimension offset 128 x 16 bytes for
// A, NT x 16 for B).  Rows past M or N are filled with zeros by the TMA unit.
// The x coordinate of every box is a multiple of 8 elements (16 bytes).  The
// boxes of a tile arrive on one mbarrier with the tile's byte count; the next
// A-tile is fetched while the epilogue drains TMEM.  Every wait is bounded; on
// a timeout the kernel waits (bounded) for its own copies and MMAs still in
// flight, records the error and frees its TMEM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

template <int NT>
__global__ void __launch_bounds__(128) gemm_bf16_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                            const __grid_constant__ CUtensorMap tmB, int M, int N,
                                                            int K, const float *bias, int act, __nv_bfloat16 *C,
                                                            float *Cf, int ldc, int *err)
{
    static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
    constexpr int kCols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
    extern __shared__ __align__(1024) unsigned char dsm[];
    unsigned char *sA = dsm;
    unsigned char *sB = dsm + (size_t)kM * K * 2;
    __shared__ __align__(8) uint64_t bar;   // MMAs of a tile done
    __shared__ __align__(8) uint64_t tbar;  // a tile's TMA boxes landed
    __shared__ uint32_t tmem_base;
    __shared__ int failed;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.y * NT;
    const int mtiles = (M + kM - 1) / kM;
    const int kcs = K / 8;  // 16-byte columns of K: one box each

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init(&tbar, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    int tile = blockIdx.x;
    if (tid == 0 && tile < mtiles) {  // B (this CTA's N-tile, all of K) and the first A-tile
        mbar_expect_tx(&tbar, (uint32_t)((kM + NT) * K * 2));
        for (int kc = 0; kc < kcs; ++kc) tma_load_2d(smem_addr(sB) + kc * NT * 16, &tmB, kc * 8, n0, &tbar);
        for (int kc = 0; kc < kcs; ++kc) tma_load_2d(smem_addr(sA) + kc * kM * 16, &tmA, kc * 8, tile * kM, &tbar);
    }
    const uint32_t tmem = tmem_base;
    constexpr uint32_t idesc = make_idesc(kM, NT);

    unsigned phase = 0, tphase = 0;
    for (; tile < mtiles; tile += gridDim.x) {
        if (tid == 0) {
            if (!mbar_wait(&tbar, tphase)) {
                failed = 1;
                mbar_arrive(&bar);  // release the other threads' wait below
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;");
                for (int s = 0; s < K / 16; ++s) {
                    const uint64_t da = make_desc(smem_addr(sA) + s * 2 * kM * 16, kM * 16, 128);
                    const uint64_t db = make_desc(smem_addr(sB) + s * 2 * NT * 16, NT * 16, 128);
                    mma_bf16(tmem, da, db, idesc, s > 0 ? 1u : 0u);
                }
                mma_commit(&bar);
            }
            tphase ^= 1;
        }
        const bool ok = mbar_wait(&bar, phase);
        phase ^= 1;
        if (!ok) failed = 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        __syncthreads();  // every thread saw the MMAs complete (or the failure)
        if (failed) break;
        // the MMAs have read sA: fetch the next tile's A while draining TMEM
        const int next = tile + gridDim.x;
        if (tid == 0 && next < mtiles) {
            mbar_expect_tx(&tbar, (uint32_t)(kM * K * 2));
            for (int kc = 0; kc < kcs; ++kc)
                tma_load_2d(smem_addr(sA) + kc * kM * 16, &tmA, kc * 8, next * kM, &tbar);
        }
        const int row = tile * kM + warp * 32 + lane;
        for (int cb = 0; cb < NT; cb += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            const int col = n0 + cb;
            if (row < M && col < N) {  // N is a multiple of 16: a chunk is all in or all out
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] += bias ? bias[col + i] : 0.f;
                if (Cf) {
                    float4 *dst = reinterpret_cast<float4 *>(Cf + (size_t)row * ldc + col);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
                if (C) {
                    uint32_t pk[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float x0 = act == 1 ? gelu(v[2 * q]) : v[2 * q];
                        const float x1 = act == 1 ? gelu(v[2 * q + 1]) : v[2 * q + 1];
                        __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
                        pk[q] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(C + (size_t)row * ldc + col);
                    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();  // TMEM drained before the next tile's MMAs
    }
    if (failed && tid == 0) {
        // a wait gave up: one more bounded wait for the copies and MMAs still in
        // flight (the phases that did not complete), then report
        (void)mbar_wait(&tbar, tphase ^ 1);
        (void)mbar_wait(&bar, phase ^ 1);
        if (err) atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

}  // namespace tc
}  // namespace ves
