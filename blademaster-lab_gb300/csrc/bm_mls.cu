// MLS-MPM cutting baseline (blademaster_warp/mlsmpm.py): updated-Lagrangian
// MLS-MPM (quadratic B-splines, APIC, one velocity field) on a dense grid
// around the material, with TopoCut damage (Eqs. 6, 7) and the TLMPM rigid
// contact for a held knife.  Particles keep the reference order; the P2G
// scatter adds each contribution as a 64-bit fixed-point integer (exact and
// independent of the order of the atomics), and every other step is a
// per-particle or per-node map, so the results are bit-identical to the CPU
// oracle's.
#include <new>

#include "bm_device.cuh"
#include "bm_internal.h"

struct bm_mls {
    bm_mls_params P;
    bm_mls_buffers B;
    bm_solver contact;  // rigid contact and knife state (one knife, no pair search)
    int64_t nodes;
};

namespace bm {
namespace {

constexpr float kMinSingularValue = 0.05f;  // mlsmpm.py:38 (PlasticineLab's clamp)

// spline_weights (mlsmpm.py:41-51): row a holds the weights of node offset a per axis.
__device__ __forceinline__ void spline_weights(bm_v3 fx, float w[3][3]) {
#pragma unroll
    for (int axis = 0; axis < 3; ++axis) {
        const float f = v3_get(fx, axis);
        w[0][axis] = 0.5f * (1.5f - f) * (1.5f - f);
        w[1][axis] = 0.75f - (f - 1.0f) * (f - 1.0f);
        w[2][axis] = 0.5f * (f - 0.5f) * (f - 0.5f);
    }
}

// cell_base + inside_domain (mlsmpm.py:54-72); false for non-finite or
// out-of-grid positions.  fx is the position relative to the base node.
__device__ __forceinline__ bool locate(const bm_mls_params& P, bm_v3 x, int base[3], bm_v3* fx) {
    if (!bm_isfinitef(x.x) || !bm_isfinitef(x.y) || !bm_isfinitef(x.z)) return false;
    const bm_v3 local = v3_div(v3_sub(x, v3(P.origin[0], P.origin[1], P.origin[2])), P.dx);
    float f[3];
    for (int i = 0; i < 3; ++i) {
        const float b = floorf(v3_get(local, i) - 0.5f);
        // base < dims - 2 (a diverged coordinate fails here before any conversion)
        if (!(b >= 0.0f && b < (float)(P.dims[i] - 2))) return false;
        base[i] = (int)b;
        f[i] = v3_get(local, i) - b;
    }
    *fx = v3(f[0], f[1], f[2]);
    return true;
}

__device__ __forceinline__ int64_t node_index(const bm_mls_params& P, int i, int j, int k) {
    return ((int64_t)i * P.dims[1] + j) * P.dims[2] + k;
}

// mlsmpm.accumulate_reaction (mlsmpm.py:140-154): interval sums, then clear.
__global__ void k_mls_accumulate(bm_buffers B) {
    const bm_v3d j = acc_read3(B.acc, BM_ACC_REACTION(0)), tau = acc_read3(B.acc, BM_ACC_TORQUE(0));
    dput3(B.interval, v3d_add(dget3(B.interval), j));
    dput3(B.interval + 3, v3d_add(dget3(B.interval + 3), tau));
    acc_clear3(B.acc, BM_ACC_REACTION(0));
    acc_clear3(B.acc, BM_ACC_TORQUE(0));
    acc_clear3(B.acc, BM_ACC_BOARD);
    B.speed[0] = 0.0f;
}

// p2g (mlsmpm.py:75-119).
__global__ void k_mls_p2g(bm_mls_params P, bm_mls_buffers B, const float* __restrict__ impulses) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const int n = P.n;
    int base[3];
    bm_v3 fx;
    if (!locate(P, ld3(B.x, n, p), base, &fx)) return;
    float w[3][3];
    spline_weights(fx, w);
    const float shear = B.damage[p] > 0.0f ? P.mu * P.damaged_shear : P.mu;
    const bm_m33 F = ld9(B.F, n, p);
    bm_m33 U, V;
    bm_v3 sigma;
    bm_svd3(F, &U, &sigma, &V);
    const bm_m33 Ps = corotated_svd(U, sigma, V, m33_identity(), shear, P.lam);
    const bm_m33 stress = m33_mul(m33_scale(Ps, (-P.dt * P.volume * 4.0f) / (P.dx * P.dx)), m33_transpose(F));
    const bm_m33 affine = m33_add(stress, m33_scale(ld9(B.C, n, p), P.mass));
    const bm_v3 momentum = v3_add(v3_mul(ld3(B.v, n, p), P.mass), ld3(impulses, n, p));
    const int64_t G = (int64_t)P.dims[0] * P.dims[1] * P.dims[2];
    unsigned long long* gm = reinterpret_cast<unsigned long long*>(B.grid_mass);
    unsigned long long* gp = reinterpret_cast<unsigned long long*>(B.grid_momentum);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float weight = (w[i][0] * w[j][1]) * w[k][2];
                const bm_v3 dpos = v3_mul(v3_sub(v3((float)i, (float)j, (float)k), fx), P.dx);
                const bm_v3 c = v3_mul(v3_add(momentum, m33_mul_v3(affine, dpos)), weight);
                const int64_t node = node_index(P, base[0] + i, base[1] + j, base[2] + k);
                atomicAdd(gp + node, (unsigned long long)bm_fixed64(c.x, P.momentum_shift));
                atomicAdd(gp + G + node, (unsigned long long)bm_fixed64(c.y, P.momentum_shift));
                atomicAdd(gp + 2 * G + node, (unsigned long long)bm_fixed64(c.z, P.momentum_shift));
                atomicAdd(gm + node, (unsigned long long)bm_fixed64(weight * P.mass, P.mass_shift));
            }
}

// grid_update (mlsmpm.py:122-137): v = p / m, sticky walls one node inside.
__global__ void k_mls_grid(bm_mls_params P, bm_mls_buffers B) {
    const int64_t G = (int64_t)P.dims[0] * P.dims[1] * P.dims[2];
    for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < G; node += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(node % P.dims[2]), j = (int)((node / P.dims[2]) % P.dims[1]), i = (int)(node / ((int64_t)P.dims[1] * P.dims[2]));
        const float m = bm_unfixed64(B.grid_mass[node], P.mass_shift);
        bm_v3 v = v3_zero();
        if (m > 0.0f)
            v = v3_div(v3(bm_unfixed64(B.grid_momentum[node], P.momentum_shift),
                          bm_unfixed64(B.grid_momentum[G + node], P.momentum_shift),
                          bm_unfixed64(B.grid_momentum[2 * G + node], P.momentum_shift)),
                       m);
        if (i < 1 || j < 1 || k < 1 || i >= P.dims[0] - 1 || j >= P.dims[1] - 1 || k >= P.dims[2] - 1) v = v3_zero();
        B.grid_v[node] = v.x;
        B.grid_v[G + node] = v.y;
        B.grid_v[2 * G + node] = v.z;
    }
}

// g2p (mlsmpm.py:157-229).
__global__ void k_mls_g2p(bm_mls_params P, bm_mls_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const int n = P.n;
    int base[3];
    bm_v3 fx;
    const bm_v3 x = ld3(B.x, n, p);
    if (!locate(P, x, base, &fx)) return;
    float w[3][3];
    spline_weights(fx, w);
    const int64_t G = (int64_t)P.dims[0] * P.dims[1] * P.dims[2];
    bm_v3 new_v = v3_zero();
    bm_m33 new_C = m33_zero();
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float weight = (w[i][0] * w[j][1]) * w[k][2];
                const bm_v3 dpos = v3_mul(v3_sub(v3((float)i, (float)j, (float)k), fx), P.dx);
                const int64_t node = node_index(P, base[0] + i, base[1] + j, base[2] + k);
                const bm_v3 gv = v3(B.grid_v[node], B.grid_v[G + node], B.grid_v[2 * G + node]);
                new_v = v3_add(new_v, v3_mul(gv, weight));
                new_C = m33_add(new_C, m33_scale(m33_outer(gv, dpos), (4.0f * weight) / (P.dx * P.dx)));
            }
    st3(B.v, n, p, new_v);
    st9(B.C, n, p, new_C);
    st3(B.x, n, p, v3_add(x, v3_mul(new_v, P.dt)));
    bm_m33 f = m33_mul(m33_add(m33_identity(), m33_scale(new_C, P.dt)), ld9(B.F, n, p));
    bm_m33 U, V;
    bm_v3 s;
    bm_svd3(f, &U, &s, &V);
    const float smallest = bm_minf(bm_minf(s.x, s.y), s.z);
    if (smallest <= 0.0f) atomicAdd(B.inversions, 1);
    if (smallest < kMinSingularValue) {
        s = v3(bm_maxf(s.x, kMinSingularValue), bm_maxf(s.y, kMinSingularValue), bm_maxf(s.z, kMinSingularValue));
        f = m33_mul(m33_mul(U, m33_diag(s)), m33_transpose(V));
    }
    const float reference_J = B.damage_reference[p];
    if (P.plastic) {
        bm_v3 e = v3(bm_logf(s.x), bm_logf(s.y), bm_logf(s.z));
        const float mean = ((e.x + e.y) + e.z) / 3.0f;
        const bm_v3 dev = v3_sub(e, v3(mean, mean, mean));
        const float norm = v3_len(dev);
        const float yield = B.yield_stress[p];
        const float limit = yield / (2.0f * P.mu) * sqrtf(2.0f / 3.0f);
        if (norm > limit) {
            e = v3_sub(e, v3_mul(dev, 1.0f - limit / norm));
            s = v3(bm_expf(e.x), bm_expf(e.y), bm_expf(e.z));
            f = m33_mul(m33_mul(U, m33_diag(s)), m33_transpose(V));
            if (P.softening > 0.0f && reference_J > 0.0f) {
                const float softened = bm_maxf(0.0f, yield - P.softening * (norm - limit));
                B.yield_stress[p] = softened;
                if (softened <= 0.0f) B.damage[p] = 1.0f;
            }
        }
    }
    st9(B.F, n, p, f);
    if (reference_J > 0.0f) {
        const float J = ((s.x * s.y) * s.z) / reference_J;
        if (J <= P.compressed || J >= P.stretched) B.damage[p] = 1.0f;
    }
}

void launch_substep(bm_mls* s, cudaStream_t st) {
    const bm_mls_params& P = s->P;
    launch_rigid(&s->contact, 0, st);
    k_mls_accumulate<<<1, 1, 0, st>>>(s->contact.B);
    cudaMemsetAsync(s->B.grid_mass, 0, sizeof(int64_t) * (size_t)s->nodes, st);
    cudaMemsetAsync(s->B.grid_momentum, 0, sizeof(int64_t) * 3 * (size_t)s->nodes, st);
    k_mls_p2g<<<grid_for(P.n), kBlock, 0, st>>>(P, s->B, s->contact.B.impulses);
    const unsigned gg = grid_for(s->nodes) < 8 * 152 ? grid_for(s->nodes) : 8 * 152;
    k_mls_grid<<<gg, kBlock, 0, st>>>(P, s->B);
    k_mls_g2p<<<grid_for(P.n), kBlock, 0, st>>>(P, s->B);
}

void launch_interval(bm_mls* s, int steps, cudaStream_t st) {
    launch_load_external(&s->contact, st);
    for (int i = 0; i < steps; ++i) launch_substep(s, st);
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_mls_create(const bm_mls_params* params, const bm_mls_buffers* buffers, const bm_params* contact,
                  const bm_buffers* contact_buffers, bm_mls** out) {
    if (!params || !buffers || !contact || !contact_buffers || !out) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    const bm_mls_params& P = *params;
    if (P.n < 1 || P.dims[0] < 3 || P.dims[1] < 3 || P.dims[2] < 3) return bm::fail(BM_ERR_ARGUMENT, "invalid MLS sizes");
    if (contact->n != P.n || contact->tool_count != 1) return bm::fail(BM_ERR_ARGUMENT, "contact must have n particles and one tool");
    const void* required[] = {buffers->x, buffers->v, buffers->C, buffers->F, buffers->yield_stress, buffers->damage,
                              buffers->damage_reference, buffers->grid_mass, buffers->grid_momentum, buffers->grid_v,
                              buffers->inversions, contact_buffers->x, contact_buffers->v, contact_buffers->histories,
                              contact_buffers->hist_mask, contact_buffers->damage, contact_buffers->impulses,
                              contact_buffers->tool, contact_buffers->tool_f, contact_buffers->mobility,
                              contact_buffers->acc, contact_buffers->interval, contact_buffers->speed,
                              contact_buffers->errors, contact_buffers->flags, contact_buffers->packed};
    for (const void* ptr : required)
        if (!ptr) return bm::fail(BM_ERR_ARGUMENT, "a required buffer is null");
    if (contact_buffers->x != buffers->x || contact_buffers->v != buffers->v)
        return bm::fail(BM_ERR_ARGUMENT, "contact particles must be the MLS particles");
    bm_mls* s = new (std::nothrow) bm_mls;
    if (!s) return bm::fail(BM_ERR_STATE, "out of host memory");
    s->P = P;
    s->B = *buffers;
    s->contact = bm_solver{};
    s->contact.P = *contact;
    s->contact.B = *contact_buffers;
    s->nodes = (int64_t)P.dims[0] * P.dims[1] * P.dims[2];
    *out = s;
    return BM_OK;
}

int bm_mls_destroy(bm_mls* s) {
    delete s;
    return BM_OK;
}

int bm_mls_substeps(bm_mls* s, int steps, void* stream) {
    if (!s || steps < 0) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    bm::launch_interval(s, steps, reinterpret_cast<cudaStream_t>(stream));
    return bm::check_cuda("mls_substeps");
}

int bm_mls_graph_create(bm_mls* s, int steps, void* stream, bm_graph** out) {
    if (!s || steps < 0 || !out) return bm::fail(BM_ERR_ARGUMENT, "invalid arguments");
    (void)stream;
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return bm::check_cuda("stream create");
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaStreamDestroy(cap);
        return bm::check_cuda("begin capture");
    }
    bm::launch_interval(s, steps, cap);
    const cudaError_t e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return bm::check_cuda("end capture");
    cudaGraphExec_t exec;
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaGraphDestroy(graph);
        return bm::check_cuda("graph instantiate");
    }
    bm_graph* g = new (std::nothrow) bm_graph;
    if (!g) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        return bm::fail(BM_ERR_STATE, "out of host memory");
    }
    g->graph = graph;
    g->exec = exec;
    *out = g;
    return BM_OK;
}

}  // extern "C"
