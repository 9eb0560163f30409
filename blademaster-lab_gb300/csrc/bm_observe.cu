// Observations of the material state that callers take between intervals:
//
//  * bm_metrics: diagnostics.Metrics.read (diagnostics.py:7-48), the kinetic,
//    gravitational and elastic energy with the largest speed and height and
//    the smallest det F.  The three sums are exact (128-bit fixed point, so
//    the result does not depend on the order of the particles' additions);
//    the extrema are exact integer reductions of order keys.
//  * bm_components: topology.components (topology.py:17-57), the piece label
//    of every particle and the piece sizes, by union-find on the device.  The
//    graph's vertices are the particles and the (node, code) pairs of the
//    stencil nodes each particle weighs (weight > 0); two pairs at a node are
//    linked when their codes are compatible.  A (node, code) pair is stood
//    for by the first particle found with that code at that node, so linking
//    a particle to its pair is a union with that particle.  Every union links
//    the larger root under the smaller, so the root of a piece is its lowest
//    particle index and ranking the roots ranks the pieces as the reference
//    does (by the lowest particle index in each).
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {
namespace {

// Scratch words of a metrics call: three 128-bit sums at [8, 20), three order keys at [20, 23).
constexpr int kMetricSums = 8, kMetricKeys = 20;
// Scratch word counting unions that gave up (see cc_union).
constexpr int kPieceErrors = 24;

__global__ void k_metrics_begin(bm_buffers B) {
    const int t = threadIdx.x;
    if (t < 12) B.scratch[kMetricSums + t] = 0;
    if (t == 0) {
        B.scratch[kMetricKeys + 0] = order_key(0.0f);      // max |v|
        B.scratch[kMetricKeys + 1] = order_key(-1.0e20f);  // max z
        B.scratch[kMetricKeys + 2] = order_key(1.0e20f);   // min det F
    }
}

// diagnostics.metrics (diagnostics.py:7-32), one thread per particle.
__global__ void __launch_bounds__(256) k_metrics(bm_params P, bm_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < P.n;
    const int N = P.n;
    bm_fx kinetic = fx_zero(), gravity = fx_zero(), elastic = fx_zero();
    int speed_key = order_key(0.0f), z_key = order_key(-1.0e20f), det_key = order_key(1.0e20f);
    if (active) {
        const bm_v3 x = ld3(B.x, N, p), v = ld3(B.v, N, p);
        const bm_m33 F = ld9(B.F, N, p);
        const bm_m33 fe = m33_mul(F, m33_inverse(ld9(B.Fp, N, p)));
        bm_m33 U, V;
        bm_v3 s;
        bm_svd3(fe, &U, &s, &V);
        const bm_m33 strain = m33_sub(fe, m33_mul(U, m33_transpose(V)));
        float energy = 0.0f;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) energy = energy + P.mu * strain.m[a][b] * strain.m[a][b];
        const float J = m33_det(fe);
        energy = energy + 0.5f * P.lam * (J - 1.0f) * (J - 1.0f);
        kinetic = bm_fx_from_float(0.5f * P.mass * v3_dot(v, v));
        gravity = bm_fx_from_float(P.mass * 9.81f * x.z);
        elastic = bm_fx_from_float(P.volume * energy);
        // a NaN takes no part in an extremum (it compares false, as in the oracle)
        const float len = v3_len(v), det = m33_det(F);
        if (len == len) speed_key = order_key(len);
        if (x.z == x.z) z_key = order_key(x.z);
        if (det == det) det_key = order_key(det);
    }
    uint64_t* sums = reinterpret_cast<uint64_t*>(B.scratch + kMetricSums);
    warp_accumulate(sums + 0, kinetic);
    warp_accumulate(sums + 2, gravity);
    warp_accumulate(sums + 4, elastic);
    speed_key = __reduce_max_sync(0xffffffffu, speed_key);
    z_key = __reduce_max_sync(0xffffffffu, z_key);
    det_key = __reduce_min_sync(0xffffffffu, det_key);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(B.scratch + kMetricKeys + 0, speed_key);
        atomicMax(B.scratch + kMetricKeys + 1, z_key);
        atomicMin(B.scratch + kMetricKeys + 2, det_key);
    }
}

__global__ void k_metrics_finish(bm_buffers B, double* out) {
    const uint64_t* sums = reinterpret_cast<const uint64_t*>(B.scratch + kMetricSums);
    for (int i = 0; i < 3; ++i) {
        bm_fx a;
        a.lo = sums[2 * i];
        a.hi = sums[2 * i + 1];
        out[i] = bm_fx_to_double(a);
        out[3 + i] = (double)order_value(B.scratch[kMetricKeys + i]);
    }
}

// ------------------------------------------------------------- pieces

// Root of x.  Parent pointers only ever point to a smaller index, so each
// step (path halving) lowers x and the loop ends within x steps.
__device__ __forceinline__ int cc_find(int32_t* parent, int x) {
    for (;;) {
        const int up = __ldcg(parent + x);
        if (up == x) return x;
        const int grand = __ldcg(parent + up);
        if (grand != up) parent[x] = grand;
        x = grand;
    }
}

// Joins the sets of a and b, linking the larger root under the smaller.  A
// failed exchange means another union linked that root meanwhile, so the
// retries are bounded by the unions that succeed; the limit only guards the
// count and is reported as an error.
__device__ void cc_union(int32_t* parent, int a, int b, int32_t* errors) {
    for (int attempt = 0; attempt < (1 << 20); ++attempt) {
        a = cc_find(parent, a);
        b = cc_find(parent, b);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(parent + b, b, a) == b) return;
    }
    atomicAdd(errors, 1);
}

__global__ void k_cc_init(int32_t* parent, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = i;
}

constexpr int kCodesPerNode = 16;

// One thread per active node: each particle that weighs the node (weight > 0)
// joins the first particle with its code there; the first particles of two
// compatible codes are joined.  Particle ids are reference indices order[p].
__global__ void k_cc_nodes(bm_params P, bm_buffers B, const int64_t* __restrict__ codes,
                           const int64_t* __restrict__ order, int32_t* parent) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int node = B.active[t];
    int32_t* errors = B.scratch + kPieceErrors;
    int64_t seen[kCodesPerNode];
    int first[kCodesPerNode];
    int k = 0;
    bool overflow = false;
    for_contributions(P, B, node, [&](int p, int a) {
        if (!(stencil_w(B, B.stencil_id[p], a) > 0.0f)) return;
        const int64_t c = codes[p];
        const int u = (int)order[p];
        int i = 0;
        while (i < k && seen[i] != c) ++i;
        if (i < k) {
            cc_union(parent, u, first[i], errors);
        } else if (k < kCodesPerNode) {
            seen[k] = c;
            first[k] = u;
            ++k;
        } else {
            overflow = true;
        }
    });
    for (int i = 0; i < k; ++i)
        for (int j = i + 1; j < k; ++j)
            if (compatible_codes(seen[i], seen[j])) cc_union(parent, first[i], first[j], errors);
    if (!overflow) return;
    // More distinct codes than the table holds: join every two weighing
    // particles with compatible codes directly (the same connectivity).
    for_contributions(P, B, node, [&](int p, int a) {
        if (!(stencil_w(B, B.stencil_id[p], a) > 0.0f)) return;
        for_contributions(P, B, node, [&](int q, int b) {
            if (q <= p || !(stencil_w(B, B.stencil_id[q], b) > 0.0f)) return;
            if (compatible_codes(codes[p], codes[q])) cc_union(parent, (int)order[p], (int)order[q], errors);
        });
    });
}

// parent -> root of each particle; roots flagged in is_root.
__global__ void k_cc_flatten(int32_t* parent, int32_t* is_root, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int root = cc_find(parent, i);
    is_root[i] = root == i ? 1 : 0;
    parent[i] = root;
}

// label = rank of the particle's root among the roots (exclusive scan).
__global__ void k_cc_rank(int32_t* labels, const int32_t* rank, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) labels[i] = rank[labels[i]];
}

__global__ void k_cc_zero(int32_t* a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = 0;
}

__global__ void k_cc_sizes(const int32_t* labels, int32_t* sizes, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(sizes + labels[i], 1);
}

__global__ void k_cc_finish(bm_buffers B, int32_t* count) {
    if (B.scratch[kPieceErrors] != 0) *count = -1;
    B.scratch[kPieceErrors] = 0;
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_metrics(bm_solver* s, double* out, void* stream) {
    if (!s || !out) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    bm::k_metrics_begin<<<1, 32, 0, st>>>(s->B);
    bm::k_metrics<<<bm::grid_for(s->P.n), bm::kBlock, 0, st>>>(s->P, s->B);
    bm::k_metrics_finish<<<1, 1, 0, st>>>(s->B, out);
    return bm::check_cuda("metrics");
}

int bm_components(bm_solver* s, const int64_t* codes, const int64_t* order, int32_t* labels, int32_t* sizes,
                  int32_t* count, void* stream) {
    if (!s || !order || !labels || !sizes || !count) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    const int n = s->P.n;
    if ((int64_t)(n + 1023) / 1024 > s->buckets / 1024)
        return bm::fail(BM_ERR_ARGUMENT, "components: more particle tiles than scan partials (bucket table too small)");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t* c = codes ? codes : s->B.codes;
    const unsigned g = bm::grid_for(n);
    bm::k_cc_init<<<g, bm::kBlock, 0, st>>>(labels, n);
    bm::k_cc_nodes<<<bm::grid_for(s->P.active_nodes), bm::kBlock, 0, st>>>(s->P, s->B, c, order, labels);
    bm::k_cc_flatten<<<g, bm::kBlock, 0, st>>>(labels, sizes, n);
    bm::launch_exclusive_scan(sizes, sizes, n, s->scan_partials, count, bm::scan_ticket(s->B), nullptr, st);
    bm::k_cc_rank<<<g, bm::kBlock, 0, st>>>(labels, sizes, n);
    bm::k_cc_zero<<<g, bm::kBlock, 0, st>>>(sizes, n);
    bm::k_cc_sizes<<<g, bm::kBlock, 0, st>>>(labels, sizes, n);
    bm::k_cc_finish<<<1, 1, 0, st>>>(s->B, count);
    return bm::check_cuda("components");
}

}  // extern "C"
