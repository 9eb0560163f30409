// Tensor-core GEMM for the learned tool predictor (a small MLP), on the
// 5th-generation tensor cores of sm_103a: D[M x N] = A[M x K] * B[N x K]^T
// (both operands bf16 and K-major, fp32 accumulation in tensor memory),
// with an optional bias + ReLU epilogue and a bf16 copy of the result.
//
// One CTA of 128 threads computes a 128-row tile with all N (<= 256)
// columns.  K is walked in chunks of 32 through a ring of four shared-memory
// stages: the threads copy the chunk of A (128 x 32) and B (N x 32) with
// cp.async (16 bytes each, no register round trip) into the canonical
// no-swizzle K-major layout (8 x 16-byte core matrices) two chunks ahead of
// the tensor core, make a landed chunk visible to it (fence.proxy.async),
// and one thread issues two tcgen05.mma of K = 16 and commits them to the
// stage's mbarrier.  A stage is refilled only after the commit of the chunk
// that last read it (two chunks earlier).  The waits are bounded: on a
// timeout the kernel records status 1 (2 if the final wait for the MMAs in
// flight also runs out), frees its tensor memory and returns.  The epilogue
// reads the accumulator with tcgen05.ld (warp w owns rows 32 w .. 32 w + 31)
// and transposes each 32 x 32 block through shared memory, so that every
// store of D writes four rows' 32 consecutive columns, 16 bytes per lane.
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
constexpr int kStageBytes = kTileM * kChunkK * 2 + 256 * kChunkK * 2;  // A tile + the widest B tile: 24 KB
constexpr int kStages = 4;  // 96 KB of dynamic shared memory
constexpr int kAhead = 2;   // chunks copied ahead of the one the tensor core takes next

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

// Poll limit of the waits inside the K loop (kWaitLimit unless a test lowers
// it to drive the timeout path); the final drain always polls kWaitLimit.
__device__ long long g_loop_wait_limit = kWaitLimit;

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase, long long limit = kWaitLimit) {
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Copies of one K chunk into the core-matrix layout with cp.async, 16 bytes
// per instruction straight into shared memory.  With 128 threads, thread t
// copies piece t % 4 (8 elements along K) of rows t / 4 + 32 i: its source
// and destination advance by fixed steps, so they are set up once per tile.
// Rows of A beyond M are zero-filled (source size 0, from A itself, which is
// always a valid address); rows of B beyond N are not copied.
__device__ __forceinline__ void cp_async16(uint32_t to, const void* from, bool in) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(to), "l"(from), "r"(in ? 16 : 0) : "memory");
}
struct ChunkCopy {
    const uint16_t* a_src;  // row m0 + t / 4, piece t % 4, chunk 0
    const uint16_t* b_src;  // row t / 4, piece t % 4, chunk 0
    uint32_t dst;           // offset of (row t / 4, piece t % 4) in a tile
    int a_rows;             // rows of A this thread copies that lie inside M (0..4)
    int b_rows;             // rows of B this thread copies (0..8)
};
__device__ __forceinline__ ChunkCopy chunk_copy(const uint16_t* A, const uint16_t* B, int M, int N, int K, int m0) {
    const int r0 = threadIdx.x >> 2, piece = threadIdx.x & 3;
    ChunkCopy c;
    c.a_src = A + (int64_t)(m0 + r0) * K + 8 * piece;
    c.b_src = B + (int64_t)r0 * K + 8 * piece;
    c.dst = (uint32_t)((r0 >> 3) * kChunkRowGroupBytes + piece * kCoreBytes + (r0 & 7) * 16);
    c.a_rows = 0;
    for (int i = 0; i < 4; ++i) c.a_rows += (m0 + r0 + 32 * i < M) ? 1 : 0;
    c.b_rows = 0;
    for (int i = 0; i < 8; ++i) c.b_rows += (r0 + 32 * i < N) ? 1 : 0;
    return c;
}
// rows r0 + 32 i are 4 row groups apart in the tile
constexpr uint32_t kRowStep = 4 * kChunkRowGroupBytes;
__device__ __forceinline__ void copy_chunk(const ChunkCopy& c, const uint16_t* A, uint32_t a_tile, uint32_t b_tile, int K,
                                           int k0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool in = i < c.a_rows;
        cp_async16(a_tile + c.dst + i * kRowStep, in ? c.a_src + (int64_t)i * 32 * K + k0 : A, in);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (i < c.b_rows) cp_async16(b_tile + c.dst + i * kRowStep, c.b_src + (int64_t)i * 32 * K + k0, true);
}

__global__ void __launch_bounds__(128) k_gemm_tn(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                 float* __restrict__ D, int M, int N, int K, const float* bias,
                                                 int relu, uint16_t* Dh, int32_t* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar[kStages];
    __shared__ uint32_t tmem_slot;
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
        for (int st = 0; st < kStages; ++st)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[st])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = instr_desc(kTileM, N);
    const int chunks = K / kChunkK;
    uint32_t phase[kStages];
    int pending[kStages];  // a commit on this stage's barrier not yet waited for (same in every thread)
#pragma unroll
    for (int st = 0; st < kStages; ++st) {
        phase[st] = 0u;
        pending[st] = 0;
    }
    auto a_tile = [&](int st) { return smem + st * kStageBytes; };                        // 128 x 32 bf16 = 8 KB
    auto b_tile = [&](int st) { return smem + st * kStageBytes + kTileM * kChunkK * 2; };  // N x 32 bf16 <= 16 KB
    const ChunkCopy cc = chunk_copy(A, B, M, N, K, m0);
    // the first kAhead chunks, one cp.async group each
    for (int c = 0; c < kAhead; ++c) {
        if (c < chunks) copy_chunk(cc, A, smem_u32(a_tile(c)), smem_u32(b_tile(c)), K, c * kChunkK);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    bool ok = true;
    for (int c = 0; c < chunks; ++c) {
        // refill the stage of chunk c + kAhead, last read by the MMAs of chunk c + kAhead - kStages
        const int next = c + kAhead, sn = next % kStages;
        if (next < chunks) {
            if (pending[sn]) {
                // one thread polls; the barrier orders its observation before every thread's copies
                bool arrived = true;
                if (threadIdx.x == 0) arrived = mbar_wait_bounded(smem_u32(&bar[sn]), phase[sn], g_loop_wait_limit);
                ok = __syncthreads_and(arrived) != 0;  // the same decision in every thread
                if (!ok) break;
                phase[sn] ^= 1u;
                pending[sn] = 0;
            }
            copy_chunk(cc, A, smem_u32(a_tile(sn)), smem_u32(b_tile(sn)), K, next * kChunkK);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        // chunk c's group has landed once at most kAhead later groups are outstanding
        asm volatile("cp.async.wait_group %0;" ::"n"(kAhead) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const int st = c % kStages;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < kChunkK; kk += 16) {
                // two core matrices along K per MMA: the K-step is 2 x 128 bytes
                const uint64_t ad = smem_desc(smem_u32(a_tile(st)) + (kk / 8) * kCoreBytes, kCoreBytes, kChunkRowGroupBytes);
                const uint64_t bd = smem_desc(smem_u32(b_tile(st)) + (kk / 8) * kCoreBytes, kCoreBytes, kChunkRowGroupBytes);
                const uint32_t accumulate = (c * kChunkK + kk) > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bar[st]))
                         : "memory");
        }
        pending[st] = 1;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    // Drain the commits not yet waited for (also after a timeout: every MMA
    // in flight gets a bounded wait before its tensor memory is freed).
    bool drained = true;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int st = 0; st < kStages; ++st)
            if (pending[st]) drained = mbar_wait_bounded(smem_u32(&bar[st]), phase[st]) && drained;
    }
    drained = __syncthreads_and(drained) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok || !drained) {
        // status 1: a wait ran out; 2: the last wait ran out too, so the
        // tensor memory is freed with MMAs possibly still in flight
        if (threadIdx.x == 0) atomicMax(status, drained ? 1 : 2);
    } else {
        // epilogue: warp w reads rows 32 w + lane, 32 columns at a time, and
        // writes them back through a padded 32 x 33 block of the (now idle)
        // operand stages: lane (r0, q) = (lane / 8, lane % 8) then stores
        // columns 4 q .. 4 q + 3 of rows r0, r0 + 4, ..., r0 + 28 as one
        // 16-byte store each (N is a multiple of 16, so a lane's four columns
        // are all inside D or all outside it)
        float* block = reinterpret_cast<float*>(smem) + warp * (32 * 33);
        const int q = lane & 7, r0 = lane >> 3;
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
#pragma unroll
            for (int j = 0; j < 32; ++j) block[lane * 33 + j] = __uint_as_float(r[j]);
            __syncwarp();
            const int col = c0 + 4 * q;
            if (col < N) {
                float b[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (bias) {
#pragma unroll
                    for (int e = 0; e < 4; ++e) b[e] = bias[col + e];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int rl = r0 + 4 * i, row = m0 + 32 * warp + rl;
                    if (row >= M) break;
                    float v[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        v[e] = block[rl * 33 + 4 * q + e];
                        if (bias) v[e] = v[e] + b[e];
                        if (relu) v[e] = fmaxf(v[e], 0.0f);
                    }
                    const int64_t at = (int64_t)row * N + col;
                    if (D) *reinterpret_cast<float4*>(D + at) = make_float4(v[0], v[1], v[2], v[3]);
                    if (Dh) {
                        const uint32_t lo = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[0])) |
                                            ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[1])) << 16);
                        const uint32_t hi = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2])) |
                                            ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[3])) << 16);
                        *reinterpret_cast<uint2*>(Dh + at) = make_uint2(lo, hi);
                    }
                }
            }
            __syncwarp();
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// ---------------------------------------------------------------- training

__device__ __forceinline__ uint16_t to_bf16(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float from_bf16(uint16_t v) { return __bfloat162float(__ushort_as_bfloat16(v)); }

// out[c][r] = in[r][c] (bf16 bits), 32 x 32 tiles through shared memory.
__global__ void k_transpose16(const uint16_t* __restrict__ in, uint16_t* __restrict__ out, int rows, int cols) {
    __shared__ uint16_t tile[32][33];
    const int c = blockIdx.x * 32 + threadIdx.x, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
        if (r0 + i < rows && c < cols) tile[i][threadIdx.x] = in[(int64_t)(r0 + i) * cols + c];
    __syncthreads();
    const int r = r0 + threadIdx.x, c0 = blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
        if (c0 + i < cols && r < rows) out[(int64_t)(c0 + i) * rows + r] = tile[threadIdx.x][i];
}

// Gradient through a ReLU layer: g[i] *= (h[i] > 0) in place (h is the layer's bf16
// output), and the result as bf16 in out.
__global__ void k_relu_grad(float* __restrict__ g, const uint16_t* __restrict__ h, uint16_t* __restrict__ out,
                            int64_t count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = from_bf16(h[i]) > 0.0f ? g[i] : 0.0f;
        g[i] = v;
        out[i] = to_bf16(v);
    }
}

// Occupancy of 4 x 4 x 4 bins in the knife's frame around its edge: local =
// rot^-1 (x - edge); bin i spans [-4 h, 4 h) across the blade (x), the
// blade length [-half_y, half_y) (y) and [-4 h, 4 h) about the edge (z).
// Particle counts (exact integer sums) per bin.
__global__ void k_pool(const float* __restrict__ x, int n, const float* __restrict__ tool_f, float h, float half_y,
                       int32_t* __restrict__ counts) {
    const ToolF T = load_tool(tool_f);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const bm_v3 local = q_rotate_inv(T.rot, v3_sub(ld3(x, n, p), T.edge));
        const float fx = (local.x + 4.0f * h) / (2.0f * h), fy = (local.y + half_y) / (0.5f * half_y),
                    fz = (local.z + 4.0f * h) / (2.0f * h);
        if (!(fx >= 0.0f && fx < 4.0f && fy >= 0.0f && fy < 4.0f && fz >= 0.0f && fz < 4.0f)) continue;
        atomicAdd(&counts[((int)fx * 4 + (int)fy) * 4 + (int)fz], 1);
    }
}

// Loss gradient of the mean squared error over rows x outputs (outputs of `width` columns,
// `pad` columns stored): d = 2 (y - t) / (rows * outputs), as fp32 and bf16; padded columns 0.
// Also sums the loss (fp32 per row, then one atomic per block).
__global__ void k_mse_grad(const float* __restrict__ y, const float* __restrict__ t, int rows, int outputs, int width,
                           float* __restrict__ d, uint16_t* __restrict__ dh, float* loss) {
    __shared__ float part[256];
    float local = 0.0f;
    const float scale = 2.0f / ((float)rows * (float)outputs);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)rows * width;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / width), c = (int)(i % width);
        float g = 0.0f;
        if (c < outputs) {
            const float e = y[i] - t[(int64_t)r * outputs + c];
            local += e * e;
            g = scale * e;
        }
        d[i] = g;
        dh[i] = to_bf16(g);
    }
    part[threadIdx.x] = local;
    __syncthreads();
    for (int step = blockDim.x / 2; step > 0; step >>= 1) {
        if (threadIdx.x < step) part[threadIdx.x] += part[threadIdx.x + step];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) atomicAdd(loss, part[0] / ((float)rows * (float)outputs));
}

// Column sums of a [rows x cols] fp32 matrix (bias gradients), one thread per column, rows in order.
__global__ void k_colsum(const float* __restrict__ g, int rows, int cols, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += g[(int64_t)r * cols + c];
    out[c] = s;
}

// bf16 bits of x (fp32) with a row stride conversion: out[r][c] for c < cols, 0 for cols <= c < pitch.
__global__ void k_cast_bf16(const float* __restrict__ x, int rows, int cols, int pitch, uint16_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)rows * pitch;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / pitch), c = (int)(i % pitch);
        out[i] = c < cols ? to_bf16(x[(int64_t)r * cols + c]) : (uint16_t)0;
    }
}

// Adam (Kingma and Ba 2015) on fp32 master weights; writes the bf16 copy used by the GEMMs.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       uint16_t* __restrict__ wh, int64_t count, float lr, float beta1, float beta2, float eps,
                       float correction1, float correction2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
        const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / correction1) / (sqrtf(vi / correction2) + eps);
        w[i] = wi;
        if (wh) wh[i] = to_bf16(wi);
    }
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_mlp_transpose16(const uint16_t* in, uint16_t* out, int rows, int cols, void* stream) {
    if (!in || !out || rows < 0 || cols < 0) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (!rows || !cols) return BM_OK;
    const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32)), block(32, 8);
    bm::k_transpose16<<<grid, block, 0, reinterpret_cast<cudaStream_t>(stream)>>>(in, out, rows, cols);
    return bm::check_cuda("mlp_transpose16");
}

int bm_mlp_relu_grad(float* g, const uint16_t* h, uint16_t* out, int64_t count, void* stream) {
    if (!g || !h || !out || count < 0) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (!count) return BM_OK;
    bm::k_relu_grad<<<bm::grid_for(count) < 1216 ? bm::grid_for(count) : 1216, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(g, h, out, count);
    return bm::check_cuda("mlp_relu_grad");
}

int bm_mlp_pool(const float* x, int n, const float* tool_f, float h, float half_y, int32_t* counts, void* stream) {
    if (!x || !tool_f || !counts || n < 0 || !(h > 0.0f) || !(half_y > 0.0f)) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaMemsetAsync(counts, 0, 64 * sizeof(int32_t), st);
    if (n) bm::k_pool<<<bm::grid_for(n) < 608 ? bm::grid_for(n) : 608, 256, 0, st>>>(x, n, tool_f, h, half_y, counts);
    return bm::check_cuda("mlp_pool");
}

int bm_mlp_mse_grad(const float* y, const float* t, int rows, int outputs, int width, float* d, uint16_t* d_bf16,
                    float* loss, void* stream) {
    if (!y || !t || !d || !d_bf16 || rows < 1 || outputs < 1 || width < outputs) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    const int64_t count = (int64_t)rows * width;
    bm::k_mse_grad<<<bm::grid_for(count) < 608 ? bm::grid_for(count) : 608, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        y, t, rows, outputs, width, d, d_bf16, loss);
    return bm::check_cuda("mlp_mse_grad");
}

int bm_mlp_colsum(const float* g, int rows, int cols, float* out, void* stream) {
    if (!g || !out || rows < 0 || cols < 1) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    bm::k_colsum<<<(cols + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(g, rows, cols, out);
    return bm::check_cuda("mlp_colsum");
}

int bm_mlp_cast_bf16(const float* x, int rows, int cols, int pitch, uint16_t* out, void* stream) {
    if (!x || !out || rows < 0 || cols < 0 || pitch < cols) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    const int64_t count = (int64_t)rows * pitch;
    if (!count) return BM_OK;
    bm::k_cast_bf16<<<bm::grid_for(count) < 1216 ? bm::grid_for(count) : 1216, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        x, rows, cols, pitch, out);
    return bm::check_cuda("mlp_cast_bf16");
}

int bm_mlp_adam(float* w, const float* g, float* m, float* v, uint16_t* w_bf16, int64_t count, float lr, float beta1,
                float beta2, float eps, int step, void* stream) {
    if (!w || !g || !m || !v || count < 0 || step < 1) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (!count) return BM_OK;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    bm::k_adam<<<bm::grid_for(count) < 1216 ? bm::grid_for(count) : 1216, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        w, g, m, v, w_bf16, count, lr, beta1, beta2, eps, c1, c2);
    return bm::check_cuda("mlp_adam");
}

int bm_gemm_set_loop_wait_limit(long long limit) {
    const long long value = limit < 0 ? bm::kWaitLimit : limit;
    if (cudaMemcpyToSymbol(bm::g_loop_wait_limit, &value, sizeof(value)) != cudaSuccess)
        return bm::check_cuda("gemm wait limit");
    return BM_OK;
}

int bm_gemm_tn_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, const float* bias, int relu,
                    uint16_t* D_bf16, int32_t* status, void* stream) {
    if (!A || !B || !status || (!D && !D_bf16)) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    if (M < 1 || N < 16 || N > 256 || N % 16 != 0 || K < 32 || K % 32 != 0)
        return bm::fail(BM_ERR_ARGUMENT, "gemm: need M >= 1, N in 16..256 (multiple of 16), K a multiple of 32");
    // 16-byte operand copies and 16-byte (fp32) / 8-byte (bf16) result stores
    if (reinterpret_cast<uintptr_t>(A) % 16 || reinterpret_cast<uintptr_t>(B) % 16 ||
        reinterpret_cast<uintptr_t>(D) % 16 || reinterpret_cast<uintptr_t>(D_bf16) % 8)
        return bm::fail(BM_ERR_ARGUMENT, "gemm: A, B and D must be 16-byte aligned, D_bf16 8-byte aligned");
    const unsigned grid = (unsigned)((M + bm::kTileM - 1) / bm::kTileM);
    // 96 KB per CTA keeps at most two CTAs on an SM, so their tensor-memory
    // allocations (at most 256 columns each) always fit the SM's 512 columns.
    const size_t smem = 96 * 1024;
    // a per-function attribute of the current device: set on every call (a cheap host call), so a
    // first launch on any device finds it set
    if (cudaFuncSetAttribute(bm::k_gemm_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return bm::check_cuda("gemm_tn_bf16 shared memory");
    bm::k_gemm_tn<<<grid, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(A, B, D, M, N, K, bias, relu, D_bf16,
                                                                                 status);
    return bm::check_cuda("gemm_tn_bf16");
}

}  // extern "C"
