// Tensor-core GEMM for the learned tool predictor (a small MLP), on the
// 5th-generation tensor cores of sm_103a: D[M x N] = A[M x K] * B[N x K]^T
// (both operands bf16 and K-major, fp32 accumulation in tensor memory),
// with an optional bias + ReLU epilogue and a bf16 copy of the result.
//
// One CTA of 128 threads computes a 128-row tile with all N (<= 256)
// columns.  K is walked in chunks of 32: the threads stage the chunk of A
// (128 x 32) and B (N x 32) in shared memory in the canonical no-swizzle
// K-major layout (8 x 16-byte core matrices), make it visible to the tensor
// core (fence.proxy.async), and one thread issues two tcgen05.mma of K = 16
// and commits them to an mbarrier that every thread waits on before the
// chunk's shared memory is reused.  The waits are bounded: on a timeout the
// kernel records status 1, waits (bounded) for its MMAs, frees its tensor
// memory and returns.  The epilogue reads the accumulator with
// tcgen05.ld (warp w owns rows 32 w .. 32 w + 31).
#include <cuda_bf16.h>
#include <stdint.h>

#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {
namespace {

constexpr int kTileM = 128;
constexpr int kChunkK = 32;
constexpr int kCoreBytes = 128;                       // 8 rows x 16 bytes
constexpr int kChunkRowGroupBytes = (kChunkK / 8) * kCoreBytes;  // SBO: one 8-row group of a chunk
constexpr long long kWaitLimit = 1 << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (no swizzle, K-major): start address,
// leading byte offset (between the two core matrices along K of one MMA),
// stride byte offset (between 8-row groups), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: fp32 accumulator, bf16 A
// and B, both K-major, N >> 3 and M >> 4.
__device__ __forceinline__ uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) {
    for (long long i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Stage rows [row0, row0 + rows) x columns [k0, k0 + 32) of a K-major bf16
// matrix (row stride ld elements) into the core-matrix layout at dst;
// rows beyond `valid` are zero.
__device__ __forceinline__ void stage(uint8_t* dst, const uint16_t* __restrict__ src, int ld, int row0, int rows,
                                      int valid, int k0) {
    // one 16-byte piece (8 elements) per step: rows x 4 pieces
    for (int t = threadIdx.x; t < rows * (kChunkK / 8); t += blockDim.x) {
        const int r = t >> 2, piece = t & 3;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (row0 + r < valid) v = *reinterpret_cast<const uint4*>(src + (int64_t)(row0 + r) * ld + k0 + 8 * piece);
        *reinterpret_cast<uint4*>(dst + (r >> 3) * kChunkRowGroupBytes + piece * kCoreBytes + (r & 7) * 16) = v;
    }
}

__global__ void __launch_bounds__(128) k_gemm_tn(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                 float* __restrict__ D, int M, int N, int K, const float* bias,
                                                 int relu, uint16_t* Dh, int32_t* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    uint8_t* a_tile = smem;                                   // 128 x 32 bf16 = 8 KB
    uint8_t* b_tile = smem + kTileM * kChunkK * 2;            // N x 32 bf16 <= 16 KB
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kTileM;
    const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = instr_desc(kTileM, N);
    uint32_t phase = 0;
    bool ok = true;
    for (int k0 = 0; k0 < K && ok; k0 += kChunkK) {
        stage(a_tile, A, K, m0, kTileM, M, k0);
        stage(b_tile, B, K, 0, N, N, k0);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < kChunkK; kk += 16) {
                // two core matrices along K per MMA: the K-step is 2 x 128 bytes
                const uint64_t ad = smem_desc(smem_u32(a_tile) + (kk / 8) * kCoreBytes, kCoreBytes, kChunkRowGroupBytes);
                const uint64_t bd = smem_desc(smem_u32(b_tile) + (kk / 8) * kCoreBytes, kCoreBytes, kChunkRowGroupBytes);
                const uint32_t accumulate = (k0 + kk) > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bar))
                         : "memory");
        }
        const bool arrived = mbar_wait_bounded(smem_u32(&bar), phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        ok = __syncthreads_and(arrived) != 0;  // the same decision in every thread
    }
    if (!ok) {
        // record the timeout and give the MMAs in flight a last bounded wait before freeing their memory
        if (threadIdx.x == 0) atomicExch(status, 1);
        mbar_wait_bounded(smem_u32(&bar), phase ^ 1u);
    } else {
        // epilogue: warp w reads rows 32 w + lane, 32 columns at a time
        const int row = m0 + 32 * warp + lane;
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
                for (int j = 0; j < 32 && c0 + j < N; ++j) {
                    float v = __uint_as_float(r[j]);
                    if (bias) v = v + bias[c0 + j];
                    if (relu) v = fmaxf(v, 0.0f);
                    if (D) D[(int64_t)row * N + c0 + j] = v;
                    if (Dh) Dh[(int64_t)row * N + c0 + j] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_gemm_tn_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, const float* bias, int relu,
                    uint16_t* D_bf16, int32_t* status, void* stream) {
    if (!A || !B || !status || (!D && !D_bf16)) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    if (M < 1 || N < 16 || N > 256 || N % 16 != 0 || K < 32 || K % 32 != 0)
        return bm::fail(BM_ERR_ARGUMENT, "gemm: need M >= 1, N in 16..256 (multiple of 16), K a multiple of 32");
    const unsigned grid = (unsigned)((M + bm::kTileM - 1) / bm::kTileM);
    // 96 KB per CTA keeps at most two CTAs on an SM, so their tensor-memory
    // allocations (at most 256 columns each) always fit the SM's 512 columns.
    const size_t smem = 96 * 1024;
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(bm::k_gemm_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return bm::check_cuda("gemm_tn_bf16 shared memory");
        configured = true;
    }
    bm::k_gemm_tn<<<grid, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(A, B, D, M, N, K, bias, relu, D_bf16,
                                                                                 status);
    return bm::check_cuda("gemm_tn_bf16");
}

}  // extern "C"
