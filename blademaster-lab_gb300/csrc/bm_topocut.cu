// TopoCut topology discovery for the MLS baseline (topocut_topology.py:31-229):
// the particle signed distance field on a voxel grid with the knife
// trajectories carved out, its zero isosurface, and the cluster of every
// particle from the surface meshes.
//
//  * SDF: particles are binned (counting sort) in cubes whose edge is the
//    search reach, so a voxel finds every particle within the reach in the 27
//    bins around its own; value = max(min |v - x_p| - r, -v_z), raised to one
//    voxel inside any carved knife box (topocut_topology.py:31-64).
//  * Isosurface: marching tetrahedra.  Every cube is split into the six
//    tetrahedra that share its (0,0,0)-(1,1,1) diagonal, so neighbouring cubes
//    agree on every face and the surface is closed and crack-free without the
//    256-case cube table.  A vertex sits on a lattice edge (7 edge directions
//    per lattice point) and is shared by all triangles that cross that edge;
//    triangles are oriented from the inside (value < 0) to the outside.
//  * Clusters: per particle and per closed surface, the closest point and the
//    winding number (sum of the triangles' solid angles), signed distance
//    negative inside; the particle joins the surface with the smallest
//    signed distance below tau (topocut_topology.py:67-78).
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {
namespace {

struct Grid {
    int d0, d1, d2;
    float lx, ly, lz, voxel;
};

__device__ __forceinline__ Grid grid_of(const bm_topocut_grid& g) {
    Grid r;
    r.d0 = g.dims[0];
    r.d1 = g.dims[1];
    r.d2 = g.dims[2];
    r.lx = g.lower[0];
    r.ly = g.lower[1];
    r.lz = g.lower[2];
    r.voxel = g.voxel;
    return r;
}

__device__ __forceinline__ int bin_of(const bm_topocut_grid& g, bm_v3 x, int axis) {
    const float lower = g.lower[axis];
    const float c = axis == 0 ? x.x : (axis == 1 ? x.y : x.z);
    int b = (int)floorf((c - lower) / g.reach);
    return b < 0 ? 0 : (b >= g.bin_dims[axis] ? g.bin_dims[axis] - 1 : b);
}
__device__ __forceinline__ int bin_index(const bm_topocut_grid& g, bm_v3 x) {
    return (bin_of(g, x, 0) * g.bin_dims[1] + bin_of(g, x, 1)) * g.bin_dims[2] + bin_of(g, x, 2);
}

__global__ void k_tc_zero(int32_t* a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = 0;
}

__global__ void k_tc_bin_count(bm_topocut_grid g, const float* x, int n, int32_t* count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    atomicAdd(count + bin_index(g, v3(x[3 * p], x[3 * p + 1], x[3 * p + 2])), 1);
}

__global__ void k_tc_bin_fill(bm_topocut_grid g, const float* x, int n, const int32_t* start, int32_t* fill,
                              int32_t* items) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int b = bin_index(g, v3(x[3 * p], x[3 * p + 1], x[3 * p + 2]));
    items[start[b] + atomicAdd(fill + b, 1)] = p;
}

// box_sdf (topocut_topology.py:31-36).
__device__ __forceinline__ float box_sdf(bm_v3 v, bm_v3 pos, bm_q rot, bm_v3 half) {
    const bm_v3 q = q_rotate_inv(rot, v3_sub(v, pos));
    const bm_v3 d = v3(fabsf(q.x) - half.x, fabsf(q.y) - half.y, fabsf(q.z) - half.z);
    const float outside = v3_len(v3(fmaxf(d.x, 0.0f), fmaxf(d.y, 0.0f), fmaxf(d.z, 0.0f)));
    return outside + fminf(fmaxf(d.x, fmaxf(d.y, d.z)), 0.0f);
}

// particle_sdf (topocut_topology.py:39-64), one thread per voxel point.
__global__ void k_tc_sdf(bm_topocut_grid g, const float* x, const int32_t* start, const int32_t* items,
                         float* field) {
    const Grid G = grid_of(g);
    const int64_t points = (int64_t)G.d0 * G.d1 * G.d2;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= points) return;
    const int k = (int)(t % G.d2), j = (int)((t / G.d2) % G.d1), i = (int)(t / ((int64_t)G.d1 * G.d2));
    const bm_v3 v = v3(G.lx + G.voxel * (float)i, G.ly + G.voxel * (float)j, G.lz + G.voxel * (float)k);
    float nearest = g.reach;
    const int bx = bin_of(g, v, 0), by = bin_of(g, v, 1), bz = bin_of(g, v, 2);
    for (int a = bx - 1; a <= bx + 1; ++a) {
        if (a < 0 || a >= g.bin_dims[0]) continue;
        for (int b = by - 1; b <= by + 1; ++b) {
            if (b < 0 || b >= g.bin_dims[1]) continue;
            for (int c = bz - 1; c <= bz + 1; ++c) {
                if (c < 0 || c >= g.bin_dims[2]) continue;
                const int bin = (a * g.bin_dims[1] + b) * g.bin_dims[2] + c;
                for (int it = start[bin]; it < start[bin + 1]; ++it) {
                    const int p = items[it];
                    nearest = fminf(nearest, v3_len(v3_sub(v, v3(x[3 * p], x[3 * p + 1], x[3 * p + 2]))));
                }
            }
        }
    }
    float value = fmaxf(nearest - g.radius, -v.z);
    const bm_v3 half = v3(g.half[0], g.half[1], g.half[2] + 0.5f * G.voxel);
    for (int s = 0; s < g.pose_count; ++s) {
        const float* pose = g.poses + 7 * s;
        bm_q rot;
        rot.x = pose[3];
        rot.y = pose[4];
        rot.z = pose[5];
        rot.w = pose[6];
        // the edge lowered by half a voxel: a cut ending within a voxel of the board carves through
        const bm_v3 centre = v3_sub(v3(pose[0], pose[1], pose[2]), q_rotate(rot, v3(0.0f, 0.0f, 0.5f * G.voxel)));
        if (box_sdf(v, centre, rot, half) <= 0.0f) value = fmaxf(value, G.voxel);
    }
    field[t] = value;
}

// The six tetrahedra of a cube around its (0,0,0)-(1,1,1) diagonal, as corner
// codes x*4 + y*2 + z; along each, corner codes only gain bits, so an edge
// (u, v) runs from the lattice point of u in direction v - u (1..7).
__constant__ int kTets[6][4] = {{0, 4, 6, 7}, {0, 4, 5, 7}, {0, 2, 6, 7}, {0, 2, 3, 7}, {0, 1, 5, 7}, {0, 1, 3, 7}};

__device__ __forceinline__ int64_t point_id(const Grid& G, int i, int j, int k) {
    return ((int64_t)i * G.d1 + j) * G.d2 + k;
}
__device__ __forceinline__ int64_t edge_id(const Grid& G, int i, int j, int k, int u, int v) {
    return point_id(G, i + ((u >> 2) & 1), j + ((u >> 1) & 1), k + (u & 1)) * 7 + ((v - u) - 1);
}
__device__ __forceinline__ bm_v3 corner_pos(const Grid& G, int i, int j, int k, int q) {
    return v3(G.lx + G.voxel * (float)(i + ((q >> 2) & 1)), G.ly + G.voxel * (float)(j + ((q >> 1) & 1)),
              G.lz + G.voxel * (float)(k + (q & 1)));
}
// Point where the field crosses zero on edge (u, v) of the cube, u inside, v not.
__device__ __forceinline__ bm_v3 crossing(const Grid& G, int i, int j, int k, const float* f, int u, int v) {
    const bm_v3 pu = corner_pos(G, i, j, k, u), pv = corner_pos(G, i, j, k, v);
    const float t = f[u] / (f[u] - f[v]);
    return v3_add(pu, v3_mul(v3_sub(pv, pu), t));
}

__device__ __forceinline__ void cube_corners(const Grid& G, const float* field, int64_t c, int* i, int* j, int* k,
                                             float* f) {
    const int e2 = G.d2 - 1, e1 = G.d1 - 1;
    *k = (int)(c % e2);
    *j = (int)((c / e2) % e1);
    *i = (int)(c / ((int64_t)e1 * e2));
    for (int q = 0; q < 8; ++q)
        f[q] = field[point_id(G, *i + ((q >> 2) & 1), *j + ((q >> 1) & 1), *k + (q & 1))];
}

// Triangles per cube, and the lattice edges the surface crosses.
__global__ void k_tc_count(bm_topocut_grid g, const float* field, int32_t* cube_tris, int32_t* edge_used) {
    const Grid G = grid_of(g);
    const int64_t cubes = (int64_t)(G.d0 - 1) * (G.d1 - 1) * (G.d2 - 1);
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= cubes) return;
    int i, j, k;
    float f[8];
    cube_corners(G, field, c, &i, &j, &k, f);
    int tris = 0;
    for (int t = 0; t < 6; ++t) {
        int inside = 0;
        for (int a = 0; a < 4; ++a) inside += f[kTets[t][a]] < 0.0f ? 1 : 0;
        tris += (inside == 1 || inside == 3) ? 1 : (inside == 2 ? 2 : 0);
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b) {
                const int u = kTets[t][a], v = kTets[t][b];
                if ((f[u] < 0.0f) != (f[v] < 0.0f)) edge_used[edge_id(G, i, j, k, u, v)] = 1;
            }
    }
    cube_tris[c] = tris;
}

// Vertex of every crossed edge (vertex index = exclusive scan of edge_used).
__global__ void k_tc_vertices(bm_topocut_grid g, const float* field, const int32_t* edge_index,
                              const int32_t* edge_used_flags, int64_t edges, float* vertices) {
    const Grid G = grid_of(g);
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= edges || !edge_used_flags[e]) return;
    const int64_t pt = e / 7;
    const int dir = (int)(e % 7) + 1;
    const int k = (int)(pt % G.d2), j = (int)((pt / G.d2) % G.d1), i = (int)(pt / ((int64_t)G.d1 * G.d2));
    float f[8];
    f[0] = field[pt];
    f[dir] = field[point_id(G, i + ((dir >> 2) & 1), j + ((dir >> 1) & 1), k + (dir & 1))];
    // crossing() interpolates from the inside corner
    const bm_v3 p = f[0] < 0.0f ? crossing(G, i, j, k, f, 0, dir) : crossing(G, i, j, k, f, dir, 0);
    const int64_t at = edge_index[e];
    vertices[3 * at] = p.x;
    vertices[3 * at + 1] = p.y;
    vertices[3 * at + 2] = p.z;
}

__device__ __forceinline__ void emit_triangle(const Grid& G, int i, int j, int k, const float* f, const int* in,
                                              int n_in, const int* out, int n_out, int ua, int va, int ub, int vb,
                                              int uc, int vc, const int32_t* edge_index, int32_t* tri) {
    // orientation: normal from the inside corners' centroid towards the outside ones'
    const bm_v3 p0 = crossing(G, i, j, k, f, ua, va), p1 = crossing(G, i, j, k, f, ub, vb),
                p2 = crossing(G, i, j, k, f, uc, vc);
    bm_v3 ci = v3_zero(), co = v3_zero();
    for (int a = 0; a < n_in; ++a) ci = v3_add(ci, corner_pos(G, i, j, k, in[a]));
    for (int a = 0; a < n_out; ++a) co = v3_add(co, corner_pos(G, i, j, k, out[a]));
    const bm_v3 d = v3_sub(v3_mul(co, 1.0f / (float)n_out), v3_mul(ci, 1.0f / (float)n_in));
    const bool flip = v3_dot(v3_cross(v3_sub(p1, p0), v3_sub(p2, p0)), d) < 0.0f;
    auto index = [&](int u, int v) {
        const int lo = u < v ? u : v, hi = u < v ? v : u;
        return edge_index[edge_id(G, i, j, k, lo, hi)];
    };
    tri[0] = index(ua, va);
    tri[1] = flip ? index(uc, vc) : index(ub, vb);
    tri[2] = flip ? index(ub, vb) : index(uc, vc);
}

// Triangles of each cube at its offset (exclusive scan of cube_tris), tetrahedra in order.
__global__ void k_tc_emit(bm_topocut_grid g, const float* field, const int32_t* tri_start, const int32_t* edge_index,
                          int32_t* triangles) {
    const Grid G = grid_of(g);
    const int64_t cubes = (int64_t)(G.d0 - 1) * (G.d1 - 1) * (G.d2 - 1);
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= cubes) return;
    int i, j, k;
    float f[8];
    cube_corners(G, field, c, &i, &j, &k, f);
    int32_t* tri = triangles + 3 * (int64_t)tri_start[c];
    for (int t = 0; t < 6; ++t) {
        int in[4], out[4], n_in = 0, n_out = 0;
        for (int a = 0; a < 4; ++a) {
            const int q = kTets[t][a];
            if (f[q] < 0.0f) in[n_in++] = q;
            else out[n_out++] = q;
        }
        if (n_in == 1 || n_in == 3) {
            const int lone = n_in == 1 ? in[0] : out[0];
            const int* others = n_in == 1 ? out : in;
            // crossing() wants (inside, outside)
            if (n_in == 1)
                emit_triangle(G, i, j, k, f, in, n_in, out, n_out, lone, others[0], lone, others[1], lone, others[2],
                              edge_index, tri);
            else
                emit_triangle(G, i, j, k, f, in, n_in, out, n_out, others[0], lone, others[1], lone, others[2], lone,
                              edge_index, tri);
            tri += 3;
        } else if (n_in == 2) {
            const int a = in[0], b = in[1], c2 = out[0], d = out[1];
            // the quad a-c, a-d, b-d, b-c as two triangles
            emit_triangle(G, i, j, k, f, in, n_in, out, n_out, a, c2, a, d, b, d, edge_index, tri);
            emit_triangle(G, i, j, k, f, in, n_in, out, n_out, a, c2, b, d, b, c2, edge_index, tri + 3);
            tri += 6;
        }
    }
}

// ------------------------------------------------------------ clusters

// Closest point on triangle (a, b, c) to p (Ericson, Real-Time Collision
// Detection, 5.1.5: regions of the vertices, edges and face).
__device__ bm_v3 closest_on_triangle(bm_v3 p, bm_v3 a, bm_v3 b, bm_v3 c) {
    const bm_v3 ab = v3_sub(b, a), ac = v3_sub(c, a), ap = v3_sub(p, a);
    const float d1 = v3_dot(ab, ap), d2 = v3_dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    const bm_v3 bp = v3_sub(p, b);
    const float d3 = v3_dot(ab, bp), d4 = v3_dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return v3_add(a, v3_mul(ab, d1 / (d1 - d3)));
    const bm_v3 cp = v3_sub(p, c);
    const float d5 = v3_dot(ab, cp), d6 = v3_dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return v3_add(a, v3_mul(ac, d2 / (d2 - d6)));
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return v3_add(b, v3_mul(v3_sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    const float denom = 1.0f / ((va + vb) + vc);
    return v3_add(a, v3_add(v3_mul(ab, vb * denom), v3_mul(ac, vc * denom)));
}

// Solid angle of triangle (a, b, c) seen from p (Van Oosterom and Strackee).
__device__ float solid_angle(bm_v3 p, bm_v3 a, bm_v3 b, bm_v3 c) {
    const bm_v3 x = v3_sub(a, p), y = v3_sub(b, p), z = v3_sub(c, p);
    const float lx = v3_len(x), ly = v3_len(y), lz = v3_len(z);
    const float num = v3_dot(x, v3_cross(y, z));
    const float den = ((lx * ly * lz + v3_dot(x, y) * lz) + v3_dot(x, z) * ly) + v3_dot(y, z) * lx;
    return 2.0f * atan2f(num, den);
}

// nearest_cluster (topocut_topology.py:67-78), one thread per particle.
__global__ void k_tc_cluster(const float* x, int n, const float* vertices, const int32_t* triangles,
                             const int32_t* mesh_start, int mesh_count, float tau, float reach, int32_t* labels) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const bm_v3 xp = v3(x[3 * p], x[3 * p + 1], x[3 * p + 2]);
    float best = tau;
    int label = -1;
    for (int m = 0; m < mesh_count; ++m) {
        float closest = 3.0e38f, winding = 0.0f;
        for (int t = mesh_start[m]; t < mesh_start[m + 1]; ++t) {
            const int32_t* f = triangles + 3 * (int64_t)t;
            const bm_v3 a = v3(vertices[3 * f[0]], vertices[3 * f[0] + 1], vertices[3 * f[0] + 2]);
            const bm_v3 b = v3(vertices[3 * f[1]], vertices[3 * f[1] + 1], vertices[3 * f[1] + 2]);
            const bm_v3 c = v3(vertices[3 * f[2]], vertices[3 * f[2] + 1], vertices[3 * f[2] + 2]);
            closest = fminf(closest, v3_len(v3_sub(xp, closest_on_triangle(xp, a, b, c))));
            winding = winding + solid_angle(xp, a, b, c);
        }
        if (!(closest <= reach)) continue;
        // inside when the winding number (solid angle / 4 pi) exceeds one half
        const float d = winding > 2.0f * 3.14159265358979f ? -closest : closest;
        if (d < best) {
            best = d;
            label = m;
        }
    }
    labels[p] = label;
}

int check_grid(const bm_topocut_grid* g) {
    if (!g || g->dims[0] < 2 || g->dims[1] < 2 || g->dims[2] < 2 || g->bin_dims[0] < 1 || g->bin_dims[1] < 1 ||
        g->bin_dims[2] < 1 || !(g->voxel > 0.0f) || !(g->reach > 0.0f) || g->pose_count < 0 ||
        (g->pose_count > 0 && !g->poses))
        return fail(BM_ERR_ARGUMENT, "topocut: invalid grid");
    return BM_OK;
}

}  // namespace
}  // namespace bm

extern "C" {

int bm_topocut_sdf(const bm_topocut_grid* g, const float* x, int n, float* field, int32_t* bin_start,
                   int32_t* bin_fill, int32_t* items, int32_t* partials, int32_t* ticket, void* stream) {
    int rc = bm::check_grid(g);
    if (rc != BM_OK) return rc;
    if (n < 0 || (n > 0 && !x) || !field || !bin_start || !bin_fill || !items || !partials || !ticket)
        return bm::fail(BM_ERR_ARGUMENT, "topocut: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t bins = (int64_t)g->bin_dims[0] * g->bin_dims[1] * g->bin_dims[2];
    const int64_t points = (int64_t)g->dims[0] * g->dims[1] * g->dims[2];
    bm::k_tc_zero<<<bm::grid_for(bins + 1), bm::kBlock, 0, st>>>(bin_fill, bins);
    bm::k_tc_zero<<<bm::grid_for(bins + 1), bm::kBlock, 0, st>>>(bin_start, bins + 1);
    if (n > 0) bm::k_tc_bin_count<<<bm::grid_for(n), bm::kBlock, 0, st>>>(*g, x, n, bin_fill);
    bm::launch_exclusive_scan(bin_fill, bin_start, bins, partials, bin_start + bins, ticket, nullptr, st);
    bm::k_tc_zero<<<bm::grid_for(bins), bm::kBlock, 0, st>>>(bin_fill, bins);
    if (n > 0) bm::k_tc_bin_fill<<<bm::grid_for(n), bm::kBlock, 0, st>>>(*g, x, n, bin_start, bin_fill, items);
    bm::k_tc_sdf<<<bm::grid_for(points), bm::kBlock, 0, st>>>(*g, x, bin_start, items, field);
    return bm::check_cuda("topocut sdf");
}

int bm_topocut_count(const bm_topocut_grid* g, const float* field, int32_t* cube_tris, int32_t* tri_start,
                     int32_t* edge_used, int32_t* edge_index, int32_t* partials, int32_t* ticket, int32_t* totals,
                     void* stream) {
    int rc = bm::check_grid(g);
    if (rc != BM_OK) return rc;
    if (!field || !cube_tris || !tri_start || !edge_used || !edge_index || !partials || !ticket || !totals)
        return bm::fail(BM_ERR_ARGUMENT, "topocut: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t cubes = (int64_t)(g->dims[0] - 1) * (g->dims[1] - 1) * (g->dims[2] - 1);
    const int64_t edges = (int64_t)g->dims[0] * g->dims[1] * g->dims[2] * 7;
    bm::k_tc_zero<<<bm::grid_for(edges), bm::kBlock, 0, st>>>(edge_used, edges);
    bm::k_tc_count<<<bm::grid_for(cubes), bm::kBlock, 0, st>>>(*g, field, cube_tris, edge_used);
    bm::launch_exclusive_scan(cube_tris, tri_start, cubes, partials, totals, ticket, nullptr, st);
    bm::launch_exclusive_scan(edge_used, edge_index, edges, partials, totals + 1, ticket, nullptr, st);
    return bm::check_cuda("topocut count");
}

int bm_topocut_emit(const bm_topocut_grid* g, const float* field, const int32_t* tri_start, const int32_t* edge_used,
                    const int32_t* edge_index, float* vertices, int32_t* triangles, void* stream) {
    int rc = bm::check_grid(g);
    if (rc != BM_OK) return rc;
    if (!field || !tri_start || !edge_used || !edge_index || !vertices || !triangles)
        return bm::fail(BM_ERR_ARGUMENT, "topocut: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t cubes = (int64_t)(g->dims[0] - 1) * (g->dims[1] - 1) * (g->dims[2] - 1);
    const int64_t edges = (int64_t)g->dims[0] * g->dims[1] * g->dims[2] * 7;
    bm::k_tc_vertices<<<bm::grid_for(edges), bm::kBlock, 0, st>>>(*g, field, edge_index, edge_used, edges, vertices);
    bm::k_tc_emit<<<bm::grid_for(cubes), bm::kBlock, 0, st>>>(*g, field, tri_start, edge_index, triangles);
    return bm::check_cuda("topocut emit");
}

int bm_topocut_cluster(const float* x, int n, const float* vertices, const int32_t* triangles,
                       const int32_t* mesh_start, int mesh_count, float tau, float reach, int32_t* labels,
                       void* stream) {
    if (n < 0 || mesh_count < 0 || !labels || (n > 0 && !x) || (mesh_count > 0 && (!vertices || !triangles || !mesh_start)))
        return bm::fail(BM_ERR_ARGUMENT, "topocut: invalid cluster arguments");
    if (n == 0) return BM_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    bm::k_tc_cluster<<<bm::grid_for(n), bm::kBlock, 0, st>>>(x, n, vertices, triangles, mesh_start, mesh_count, tau,
                                                            reach, labels);
    return bm::check_cuda("topocut cluster");
}

}  // extern "C"
