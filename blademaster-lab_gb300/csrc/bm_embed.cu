// Nodal embedding of a surface in the deformed material
// (surface_gpu.py:11-175 kernels, surface.py:887-993 semantics), in float64
// (or float32, the reference's display option).
//
// A node's field for a code is the weighted mean, over the node's support
// particles (tent weights of the reference configuration) whose codes are
// compatible with the code and with the code of the support's heaviest
// compatible particle (one side of an unassigned cut), of each particle's
// affine extrapolation x_p + F_p (node - ref_p) and of F_p.  With `extend`,
// a node without such a particle uses its second support ring.  A vertex is
// the trilinear interpolation of its own code's field over its grid cell.
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {
namespace {

template <typename T>
struct Field {
    T position[3];
    T gradient[9];
    T total;
    int extended;
};

template <typename T>
__device__ void ring_sum(const bm_embedding& E, const int32_t* offsets, const int32_t* indices, const T* weights,
                         int i, int64_t code, const T* x, const T* F, const int64_t* __restrict__ codes,
                         T& heaviest, int64_t& anchor, Field<T>& out) {
    const T* nodes = static_cast<const T*>(E.nodes);
    const T* reference = static_cast<const T*>(E.reference);
    const int begin = offsets[i], end = offsets[i + 1];
    for (int a = begin; a < end; ++a) {
        const int p = indices[a];
        if (compatible_codes(code, codes[p]) && weights[a] > heaviest) {
            heaviest = weights[a];
            anchor = codes[p];
        }
    }
    for (int a = begin; a < end; ++a) {
        const int p = indices[a];
        const int64_t c = codes[p];
        if (!compatible_codes(code, c) || !compatible_codes(anchor, c)) continue;
        const T w = weights[a];
        const T d0 = nodes[3 * i] - reference[3 * p], d1 = nodes[3 * i + 1] - reference[3 * p + 1],
                d2 = nodes[3 * i + 2] - reference[3 * p + 2];
        const T* f = F + 9 * (int64_t)p;
        for (int r = 0; r < 3; ++r) {
            const T e = x[3 * (int64_t)p + r] + ((f[3 * r] * d0 + f[3 * r + 1] * d1) + f[3 * r + 2] * d2);
            out.position[r] = out.position[r] + w * e;
        }
        for (int k = 0; k < 9; ++k) out.gradient[k] = out.gradient[k] + w * f[k];
        out.total = out.total + w;
    }
}

// node_field (surface_gpu.py:20-77) of node i for `code`.
template <typename T>
__device__ Field<T> node_field(const bm_embedding& E, int i, int64_t code, int extend, const T* x, const T* F,
                               const int64_t* __restrict__ codes) {
    Field<T> out;
    for (int r = 0; r < 3; ++r) out.position[r] = T(0);
    for (int k = 0; k < 9; ++k) out.gradient[k] = T(0);
    out.total = T(0);
    out.extended = 0;
    T heaviest = T(0);
    int64_t anchor = code;
    ring_sum<T>(E, E.offsets, E.indices, static_cast<const T*>(E.weights), i, code, x, F, codes, heaviest, anchor,
                out);
    if (out.total == T(0) && extend) {
        ring_sum<T>(E, E.extra_offsets, E.extra_indices, static_cast<const T*>(E.extra_weights), i, code, x, F,
                    codes, heaviest, anchor, out);
        if (out.total > T(0)) out.extended = 1;
    }
    return out;
}

template <typename T>
__device__ __forceinline__ T not_a_number();
template <>
__device__ __forceinline__ double not_a_number<double>() {
    return __longlong_as_double(0x7ff8000000000000ll);
}
template <>
__device__ __forceinline__ float not_a_number<float>() {
    return __int_as_float(0x7fc00000);
}

// evaluate_nodes (surface_gpu.py:79-129): per node, its field for its own
// code (node_codes) or for one code; NaN where nothing supports it.
template <typename T>
__global__ void k_embed_nodes(bm_embedding E, const T* x, const T* F, const int64_t* __restrict__ codes,
                              const int64_t* __restrict__ node_codes, int64_t code, int extend, T* positions,
                              T* gradients, int32_t* extensions) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= E.node_count) return;
    const Field<T> f = node_field<T>(E, i, node_codes ? node_codes[i] : code, extend, x, F, codes);
    if (f.extended) atomicAdd(extensions, 1);
    for (int r = 0; r < 3; ++r) positions[3 * (int64_t)i + r] = f.total > T(0) ? f.position[r] / f.total : not_a_number<T>();
    for (int k = 0; k < 9; ++k) gradients[9 * (int64_t)i + k] = f.total > T(0) ? f.gradient[k] / f.total : not_a_number<T>();
}

// embed_vertices (surface_gpu.py:131-175): trilinear interpolation of each
// vertex's own-code field over its grid cell; counts[0] extended corner
// lookups, counts[1] corners with weight > 1e-9 and no support.
template <typename T>
__global__ void k_embed_vertices(bm_embedding E, int vertex_count, const int64_t* __restrict__ vertex_codes,
                                 const int32_t* __restrict__ corners, const T* corner_weights, const T* x, const T* F,
                                 const int64_t* __restrict__ codes, T* vertices, int32_t* counts) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vertex_count) return;
    T result[3] = {T(0), T(0), T(0)};
    for (int k = 0; k < 8; ++k) {
        const Field<T> f = node_field<T>(E, corners[8 * (int64_t)v + k], vertex_codes[v], 1, x, F, codes);
        if (f.extended) atomicAdd(counts, 1);
        const T cw = corner_weights[8 * (int64_t)v + k];
        if (f.total > T(0)) {
            for (int r = 0; r < 3; ++r) result[r] = result[r] + cw * f.position[r] / f.total;
        } else if (cw > T(1.0e-9)) {
            atomicAdd(counts + 1, 1);
        }
    }
    for (int r = 0; r < 3; ++r) vertices[3 * (int64_t)v + r] = result[r];
}

int check_embedding(const bm_embedding* E) {
    if (!E || E->node_count < 0 || E->particle_count < 0 || (E->scalar_bytes != 4 && E->scalar_bytes != 8))
        return fail(BM_ERR_ARGUMENT, "embedding: invalid sizes or scalar_bytes (4 or 8)");
    if (E->node_count > 0 && (!E->nodes || !E->offsets || !E->indices || !E->weights))
        return fail(BM_ERR_ARGUMENT, "embedding: null nodes or support");
    return BM_OK;
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_embed_nodes(const bm_embedding* E, const void* x, const void* F, const int64_t* codes,
                   const int64_t* node_codes, int64_t code, int extend, void* positions, void* gradients,
                   int32_t* extensions, void* stream) {
    int rc = bm::check_embedding(E);
    if (rc != BM_OK) return rc;
    if (!x || !F || !codes || !positions || !gradients || !extensions) return bm::fail(BM_ERR_ARGUMENT, "null argument");
    if (extend && (!E->extra_offsets || !E->extra_indices || !E->extra_weights))
        return bm::fail(BM_ERR_ARGUMENT, "embedding: extend needs the second support ring");
    if (E->node_count == 0) return BM_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const unsigned g = bm::grid_for(E->node_count);
    if (E->scalar_bytes == 8)
        bm::k_embed_nodes<double><<<g, bm::kBlock, 0, st>>>(*E, (const double*)x, (const double*)F, codes, node_codes,
                                                             code, extend, (double*)positions, (double*)gradients,
                                                             extensions);
    else
        bm::k_embed_nodes<float><<<g, bm::kBlock, 0, st>>>(*E, (const float*)x, (const float*)F, codes, node_codes,
                                                           code, extend, (float*)positions, (float*)gradients,
                                                           extensions);
    return bm::check_cuda("embed nodes");
}

int bm_embed_vertices(const bm_embedding* E, int vertex_count, const int64_t* vertex_codes, const int32_t* corners,
                      const void* corner_weights, const void* x, const void* F, const int64_t* codes, void* vertices,
                      int32_t* counts, void* stream) {
    int rc = bm::check_embedding(E);
    if (rc != BM_OK) return rc;
    if (vertex_count < 0) return bm::fail(BM_ERR_ARGUMENT, "negative vertex count");
    if (vertex_count == 0) return BM_OK;
    if (!vertex_codes || !corners || !corner_weights || !x || !F || !codes || !vertices || !counts)
        return bm::fail(BM_ERR_ARGUMENT, "null argument");
    if (!E->extra_offsets || !E->extra_indices || !E->extra_weights)
        return bm::fail(BM_ERR_ARGUMENT, "embedding: vertices need the second support ring");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const unsigned g = bm::grid_for(vertex_count);
    if (E->scalar_bytes == 8)
        bm::k_embed_vertices<double><<<g, bm::kBlock, 0, st>>>(*E, vertex_count, vertex_codes, corners,
                                                                (const double*)corner_weights, (const double*)x,
                                                                (const double*)F, codes, (double*)vertices, counts);
    else
        bm::k_embed_vertices<float><<<g, bm::kBlock, 0, st>>>(*E, vertex_count, vertex_codes, corners,
                                                              (const float*)corner_weights, (const float*)x,
                                                              (const float*)F, codes, (float*)vertices, counts);
    return bm::check_cuda("embed vertices");
}

}  // extern "C"
