// Device-side helpers shared by the kernels: structure-of-arrays access,
// stencil lookup, field slots, the float32 tool mirror and the exact 128-bit
// accumulators.  Every kernel translation unit is compiled with --fmad=false
// so the arithmetic matches the oracle's operation sequence.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/blademaster_gb300.h"
#include "bm_scalar.h"

namespace bm {

constexpr int kBlock = 256;
constexpr int kSMs = 152;  // streaming multiprocessors of a GB300

// Structure-of-arrays access with 32-bit indices (every array here holds
// fewer than 2^31 elements: n < 2^28 particles, fmax * node_count < 2^29).
__device__ __forceinline__ bm_v3 ld3(const float* __restrict__ a, int n, int i) {
    return v3(a[i], a[n + i], a[2 * n + i]);
}
__device__ __forceinline__ void st3(float* __restrict__ a, int n, int i, bm_v3 v) {
    a[i] = v.x;
    a[n + i] = v.y;
    a[2 * n + i] = v.z;
}
__device__ __forceinline__ bm_m33 ld9(const float* __restrict__ a, int n, int i) {
    bm_m33 m;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) m.m[r][c] = a[(3 * r + c) * n + i];
    return m;
}
__device__ __forceinline__ void st9(float* __restrict__ a, int n, int i, const bm_m33& m) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) a[(3 * r + c) * n + i] = m.m[r][c];
}

// Node offset of stencil index a = 4 ox + 2 oy + oz (geometry OFFSETS order).
__device__ __forceinline__ int node_offset(const bm_params& P, int a) {
    return ((a >> 2) & 1) * P.node_dims[1] * P.node_dims[2] + ((a >> 1) & 1) * P.node_dims[2] + (a & 1);
}
__device__ __forceinline__ int field_of(uint64_t fidx, int a) { return (int)((fidx >> (8 * a)) & 0xffu); }
__device__ __forceinline__ int slot_of(const bm_params& P, int base, uint64_t fidx, int a) {
    return field_of(fidx, a) * P.node_count + base + node_offset(P, a);
}
__device__ __forceinline__ float stencil_w(const bm_buffers& B, int sid, int a) { return __ldg(&B.stencil_w[8 * sid + a]); }
__device__ __forceinline__ bm_v3 stencil_g(const bm_buffers& B, int sid, int a) {
    const float* g = B.stencil_g + 24 * sid + 3 * a;
    return v3(__ldg(g), __ldg(g + 1), __ldg(g + 2));
}

struct ToolF {
    bm_v3 pos, vel, omega;
    bm_q rot;
    float speed;        // |vel|
    float spin_reach;   // |omega| * blade radius
    bm_v3 edge;         // pos + rot (0, 0, -half_z)
    bm_v3 down;         // rot (0, 0, -1)
    bm_v3 edge_vel;     // vel + omega x (edge - pos)
    bm_v3 ax, ay, az;   // knife axes in the world (for conservative pre-tests only)
};
// The record is read as nine 16-byte loads (records are 144 bytes, 16-byte aligned).
__device__ __forceinline__ ToolF load_tool(const float* __restrict__ t) {
    const float4* q = reinterpret_cast<const float4*>(t);
    const float4 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4], f = q[5], g = q[6], h = q[7], i = q[8];
    ToolF r;
    r.pos = v3(a.x, a.y, a.z);
    r.vel = v3(a.w, b.x, b.y);
    r.rot.x = b.z;
    r.rot.y = b.w;
    r.rot.z = c.x;
    r.rot.w = c.y;
    r.omega = v3(c.z, c.w, d.x);
    r.speed = d.y;
    r.spin_reach = d.z;
    r.edge = v3(d.w, e.x, e.y);
    r.down = v3(e.z, e.w, f.x);
    r.edge_vel = v3(f.y, f.z, f.w);
    r.ax = v3(g.x, g.y, g.z);
    r.ay = v3(g.w, h.x, h.y);
    r.az = v3(h.z, h.w, i.x);
    return r;
}
__device__ __forceinline__ float blade_radius(const bm_params& P) {
    return sqrtf((P.half[0] * P.half[0] + P.half[1] * P.half[1]) + P.half[2] * P.half[2]);
}

// Signed-integer keys that order like the floats (and back).
__device__ __forceinline__ int order_key(float f) {
    const int b = __float_as_int(f);
    return b ^ ((b >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float order_value(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7FFFFFFF)); }

// Bounding box (centre, half extent) of the positions of this warp's active
// lanes and the largest of their `speed` values.  All 32 lanes must call;
// `*any` is false when no lane is active.  The box is widened by 1 um so that
// it still contains every position after the rounding of centre and extent.
// Minima and maxima are exact (float warp reductions); a NaN among the active
// values makes the result NaN, which every knife test keeps.
__device__ __forceinline__ float warp_min(float v) {
    float r;
    asm("redux.sync.min.NaN.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float warp_max(float v) {
    float r;
    asm("redux.sync.max.NaN.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ void warp_box(bm_v3 x, float speed, bool active, bm_v3* centre, bm_v3* extent,
                                         float* max_speed, bool* any) {
    *any = __any_sync(0xffffffffu, active);
    const float inf = __int_as_float(0x7f800000);
    const bm_v3 lo = v3(warp_min(active ? x.x : inf), warp_min(active ? x.y : inf), warp_min(active ? x.z : inf));
    const bm_v3 hi = v3(warp_max(active ? x.x : -inf), warp_max(active ? x.y : -inf), warp_max(active ? x.z : -inf));
    *centre = v3_mul(v3_add(lo, hi), 0.5f);
    *extent = v3_add(v3_mul(v3_sub(hi, lo), 0.5f), v3(1.0e-6f, 1.0e-6f, 1.0e-6f));
    *max_speed = warp_max(active ? speed : -inf);
}

// Projection radius of a box with half extent e on direction a.
__device__ __forceinline__ float box_reach(bm_v3 a, bm_v3 e) {
    return (fabsf(a.x) * e.x + fabsf(a.y) * e.y) + fabsf(a.z) * e.z;
}

// Exact accumulation: warp-sum of 128-bit fixed-point values, then one
// carry-propagating pair of 64-bit atomics per warp.
__device__ __forceinline__ bm_fx warp_sum_fx(bm_fx v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        bm_fx o;
        o.lo = __shfl_xor_sync(0xffffffffu, v.lo, d);
        o.hi = __shfl_xor_sync(0xffffffffu, v.hi, d);
        v = bm_fx_add(v, o);
    }
    return v;
}
__device__ __forceinline__ void atomic_add_fx(uint64_t* acc, bm_fx v) {
    unsigned long long* lo = reinterpret_cast<unsigned long long*>(acc);
    unsigned long long* hi = lo + 1;
    unsigned long long old = atomicAdd(lo, (unsigned long long)v.lo);
    unsigned long long carry = (old + (unsigned long long)v.lo) < old ? 1ull : 0ull;
    unsigned long long add_hi = (unsigned long long)v.hi + carry;
    if (add_hi != 0ull) atomicAdd(hi, add_hi);
}
// All 32 lanes must call (values may be zero); lane 0 performs the atomics.
__device__ __forceinline__ void warp_accumulate(uint64_t* acc, bm_fx v) {
    v = warp_sum_fx(v);
    if ((threadIdx.x & 31) == 0 && (v.lo != 0u || v.hi != 0u)) atomic_add_fx(acc, v);
}
__device__ __forceinline__ bm_fx fx_zero() {
    bm_fx z;
    z.lo = 0u;
    z.hi = 0u;
    return z;
}

// 128-bit accumulator triples and float64 vectors in plain arrays.
__device__ __forceinline__ bm_v3d acc_read3(const uint64_t* acc, int word) {
    bm_fx a, b, c;
    a.lo = acc[word];
    a.hi = acc[word + 1];
    b.lo = acc[word + 2];
    b.hi = acc[word + 3];
    c.lo = acc[word + 4];
    c.hi = acc[word + 5];
    return v3d(bm_fx_to_double(a), bm_fx_to_double(b), bm_fx_to_double(c));
}
__device__ __forceinline__ void acc_clear3(uint64_t* acc, int word) {
    for (int i = 0; i < 6; ++i) acc[word + i] = 0u;
}
__device__ __forceinline__ bm_v3d dget3(const double* t) { return v3d(t[0], t[1], t[2]); }
__device__ __forceinline__ void dput3(double* t, bm_v3d v) {
    t[0] = v.x;
    t[1] = v.y;
    t[2] = v.z;
}

__device__ __forceinline__ void atomic_max_nonneg(float* addr, float v) {
    // Non-negative floats order like their bit patterns.
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

__device__ __forceinline__ int compatible_masks(uint64_t ones_a, uint64_t twos_a, uint64_t ones_b, uint64_t twos_b) {
    return (ones_a & twos_b) == 0u && (twos_a & ones_b) == 0u;
}

// material.compatible (material.py:23-34) on int64 codes.
__device__ __forceinline__ int compatible_codes(int64_t a, int64_t b) {
    while (a != 0 || b != 0) {
        int64_t x = a % 3, y = b % 3;
        if (x != 0 && y != 0 && x != y) return 0;
        a /= 3;
        b /= 3;
    }
    return 1;
}

__device__ __forceinline__ void digit_masks(int64_t code, uint64_t* ones, uint64_t* twos) {
    uint64_t o = 0u, t = 0u;
    int bit = 0;
    while (code != 0) {
        int64_t d = code % 3;
        if (d == 1) o |= (uint64_t)1 << bit;
        if (d == 2) t |= (uint64_t)1 << bit;
        code /= 3;
        ++bit;
    }
    *ones = o;
    *twos = t;
}

// Visit the contributions to node n in ascending particle order: adjacent
// cells in ascending cell index (stencil index a = 7 .. 0), particles of each
// cell in order.  fn(p, a) is called for each.
template <typename Fn>
__device__ __forceinline__ void for_contributions(const bm_params& P, const bm_buffers& B, int n, Fn fn) {
    const int nyz = P.node_dims[1] * P.node_dims[2];
    const int i = n / nyz, j = (n / P.node_dims[2]) % P.node_dims[1], k = n % P.node_dims[2];
#pragma unroll 1
    for (int a = 7; a >= 0; --a) {
        const int ci = i - ((a >> 2) & 1), cj = j - ((a >> 1) & 1), ck = k - (a & 1);
        if (ci < 0 || cj < 0 || ck < 0 || ci >= P.cell_dims[0] || cj >= P.cell_dims[1] || ck >= P.cell_dims[2]) continue;
        const int c = (ci * P.cell_dims[1] + cj) * P.cell_dims[2] + ck;
        const int begin = B.cell_start[c], end = B.cell_start[c + 1];
#pragma unroll 1
        for (int p = begin; p < end; ++p) fn(p, a);
    }
}

// material.corotated_stress (material.py:78-91) from the SVD of F Fp^-1.
__device__ __forceinline__ bm_m33 corotated_svd(const bm_m33& U, bm_v3 s, const bm_m33& V, const bm_m33& plastic_inverse, float mu,
                                float lam) {
    const float J = (s.x * s.y) * s.z;
    bm_v3 d;
    for (int i = 0; i < 3; ++i) {
        const float si = v3_get(s, i);
        v3_set(&d, i, 2.0f * mu * (si - 1.0f) + lam * (J - 1.0f) * J / si);
    }
    return m33_mul(m33_mul(m33_mul(U, m33_diag(d)), m33_transpose(V)), m33_transpose(plastic_inverse));
}

// The registration this substep runs (flags[BM_FLAG_REG_MODE]): none while the
// topology is clean; full when forced, after a host write (BM_FLAG_HOST_DIRTY,
// also set at creation) or a registration requested through the C-ABI;
// otherwise incremental over the nodes the side labelling listed.
__device__ __forceinline__ void begin_registration(const bm_buffers& B, int force) {
    const bool dirty = force || B.flags[BM_FLAG_TOPOLOGY_DIRTY] != 0;
    const int mode = !dirty ? 0 : ((force || B.flags[BM_FLAG_HOST_DIRTY] != 0) ? 1 : 2);
    B.flags[BM_FLAG_REG_MODE] = mode;
    if (mode != 0) {
        B.flags[BM_FLAG_MULTI] = 0;
        B.flags[BM_FLAG_REGISTRATIONS] += 1;
    }
    if (mode == 1) {
        B.flags[BM_FLAG_MIXED_CELLS] = 0;
        B.flags[BM_FLAG_HOST_DIRTY] = 0;
    }
}

inline unsigned grid_for(int64_t count, int block = kBlock) {
    int64_t g = (count + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

// Threads per block of a one-thread-per-item launch: kBlock, or fewer (a
// power of two, at least one warp) when kBlock-sized blocks would not give
// every SM a block.  A small scene's warps then spread over the SMs instead
// of queueing several to an SM (the triple cut's 4480 particles: 2.5 % less
// time per interval).  Kernels launched this way use no block-wide shared
// memory or barrier, only warp-level collectives.
inline int spread_block(int64_t count) {
    int threads = 32;
    while (threads < kBlock && (count + threads - 1) / threads > kSMs) threads *= 2;
    return threads;
}

}  // namespace bm
