// Topology-aware TLMPM transfers and constitutive update on the GB300
// (blademaster_warp/material.py).
//
// Layout: particles are sorted by reference cell, so the particles that weigh
// a grid node are the contents of its eight adjacent cells, contiguous in
// memory.  The reference scatters (p, a) contributions with float atomics into
// a hash of (node, code) keys; here each cell's particles first reduce their
// contributions to each of the cell's corners with a fixed warp-shuffle tree
// (cell pass), and one thread per node then adds the partials of its adjacent
// cells in a fixed order (node pass), so the sums are deterministic and no
// float atomic touches the primary fields.  A node's fields (one per distinct
// cut code among its contributors, ascending code) live at slot
// f * node_count + node; each particle carries the field index of each of its
// eight stencil nodes in one uint64 (fidx).
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {

// ---------------------------------------------------------------- topology

// Solver._register_topology, node pass: the distinct codes among a node's
// contributors in ascending order (material.register, material.py:50-66).
// With list_multi the node joins the multi-field node list when it has
// more than one field.
__device__ void register_node(const bm_params& P, const bm_buffers& B, const int64_t* __restrict__ field_codes, int n,
                              bool list_multi = true);

__global__ void k_register_begin(bm_buffers B, int force) { begin_registration(B, force); }

__global__ void k_register_nodes(bm_params P, bm_buffers B, const int64_t* __restrict__ field_codes) {
    if (B.flags[BM_FLAG_REG_MODE] != 1) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < P.active_nodes; t += gridDim.x * blockDim.x)
        register_node(P, B, field_codes, B.active[t]);
}

__device__ void register_node(const bm_params& P, const bm_buffers& B, const int64_t* __restrict__ field_codes, int n,
                              bool list_multi) {
    int nf = 0;
    int64_t prev = 0;
    bool have_prev = false;
    for (;;) {
        int64_t best = 0;
        bool found = false;
        for_contributions(P, B, n, [&](int p, int) {
            const int64_t c = field_codes[p];
            if ((!have_prev || c > prev) && (!found || c < best)) {
                best = c;
                found = true;
            }
        });
        if (!found) break;
        if (nf >= P.fmax) {
            atomicAdd(&B.errors[0], 1);
            break;
        }
        const int s = nf * P.node_count + n;
        B.fcode[s] = best;
        uint64_t ones, twos;
        digit_masks(best, &ones, &twos);
        B.fones[s] = ones;
        B.ftwos[s] = twos;
        ++nf;
        prev = best;
        have_prev = true;
    }
    B.nfield[n] = nf;
    if (list_multi && nf > 1) B.multi_nodes[atomicAdd(&B.flags[BM_FLAG_MULTI], 1)] = n;
}

// Particle pass: the field index of the particle's code at each stencil node.
__device__ uint64_t register_particle(const bm_params& P, const bm_buffers& B, const int64_t* __restrict__ field_codes,
                                      int p);

__global__ void k_register_particles(bm_params P, bm_buffers B, const int64_t* __restrict__ field_codes) {
    if (B.flags[BM_FLAG_REG_MODE] != 1) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) register_particle(P, B, field_codes, p);
}

__device__ uint64_t register_particle(const bm_params& P, const bm_buffers& B, const int64_t* __restrict__ field_codes,
                                      int p) {
    const int64_t code = field_codes[p];
    const int base = B.base_node[p];
    uint64_t fidx = 0u;
    for (int a = 0; a < 8; ++a) {
        const int node = base + node_offset(P, a);
        const int nf = B.nfield[node];
        int f = 0;
        while (f < nf && B.fcode[(int64_t)f * P.node_count + node] != code) ++f;
        if (f >= nf) f = 0;  // only after a field overflow, already counted in errors[0]
        fidx |= (uint64_t)f << (8 * a);
    }
    B.fidx[p] = fidx;
    return fidx;
}

__global__ void k_clear_flag(bm_buffers B, int which) { B.flags[which] = 0; }

// ------------------------------------------------------------------- P2G
//
// Summation order (shared with the oracle): the contribution of the <= 8
// particles of a cell to one of its corner nodes is summed by a fixed tree
// over the cell's 8 particle slots, ((s0+s1)+(s2+s3))+((s4+s5)+(s6+s7)), with
// absent particles and particles of another field contributing +0; a node
// then adds the partials of its adjacent cells in ascending cell index
// (corner index a = 7 .. 0), skipping cells without a particle of the field.
//
// The corner flags (cell_field[node][a]: the field of a uniform corner, 255
// when the cell's particles map to different fields there, 254 when there is
// no cell) depend only on the field indices, so registration writes them and
// counts the cells with a mixed corner.  Per substep, the cell pass writes one
// partial per corner; single-field nodes read eight partials; multi-field
// nodes are handled one warp each and sum a mixed corner's particles of each
// field by the same tree straight from the cell's particles.

constexpr int kMixed = 255;
constexpr int kAbsentCorner = 254;
constexpr unsigned kFull = 0xffffffffu;

// Reduce-scatter over the 8 lanes of a cell group: vals[c][v] holds this
// lane's contribution to corner c; on return out[v] holds, in lane s, the sum
// over the group for corner s.  Each sum is the tree
// ((s0+s1)+(s2+s3))+((s4+s5)+(s6+s7)) over the group's lanes (each addition
// commutes), with 7 V shuffles instead of 24 V for a full butterfly per corner.
template <int V>
__device__ __forceinline__ void reduce_scatter8(const float (&vals)[8][V], float (&out)[V]) {
    const int s = threadIdx.x & 7;
    const bool b0 = s & 1, b1 = (s >> 1) & 1, b2 = (s >> 2) & 1;
    float k1[4][V], k2[2][V];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float mine = b0 ? vals[2 * j + 1][v] : vals[2 * j][v];
            const float other = b0 ? vals[2 * j][v] : vals[2 * j + 1][v];
            k1[j][v] = mine + __shfl_xor_sync(kFull, other, 1);
        }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float mine = b1 ? k1[2 * i + 1][v] : k1[2 * i][v];
            const float other = b1 ? k1[2 * i][v] : k1[2 * i + 1][v];
            k2[i][v] = mine + __shfl_xor_sync(kFull, other, 2);
        }
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const float mine = b2 ? k2[1][v] : k2[0][v];
        const float other = b2 ? k2[0][v] : k2[1][v];
        out[v] = mine + __shfl_xor_sync(kFull, other, 4);
    }
}
__device__ __forceinline__ int cell_count(const bm_params& P) { return P.cell_dims[0] * P.cell_dims[1] * P.cell_dims[2]; }
// The cell whose corner a is node n, or -1.
__device__ __forceinline__ int cell_at(const bm_params& P, int n, int a) {
    const int nyz = P.node_dims[1] * P.node_dims[2];
    const int ci = n / nyz - ((a >> 2) & 1), cj = (n / P.node_dims[2]) % P.node_dims[1] - ((a >> 1) & 1),
              ck = n % P.node_dims[2] - (a & 1);
    if (ci < 0 || cj < 0 || ck < 0 || ci >= P.cell_dims[0] || cj >= P.cell_dims[1] || ck >= P.cell_dims[2]) return -1;
    return (ci * P.cell_dims[1] + cj) * P.cell_dims[2] + ck;
}
// Node of corner (0, 0, 0) of cell c.
__device__ __forceinline__ int cell_base_node(const bm_params& P, int c) {
    const int ck = c % P.cell_dims[2], cj = (c / P.cell_dims[2]) % P.cell_dims[1], ci = c / (P.cell_dims[1] * P.cell_dims[2]);
    return (ci * P.node_dims[1] + cj) * P.node_dims[2] + ck;
}

// Registration, cell pass: corner flags of every occupied cell and the list of
// cells with a mixed corner.  Thread (cell, slot); lane s decides corner s.
__global__ void k_register_cells(bm_params P, bm_buffers B) {
    if (B.flags[BM_FLAG_REG_MODE] != 1) return;
    const int cells = cell_count(P);
    const int stride = gridDim.x * blockDim.x;
    for (int t0 = blockIdx.x * blockDim.x; t0 < 8 * cells; t0 += stride) {
        const int t = t0 + threadIdx.x;
        const int c = t >> 3, s = t & 7;
        int count = 0, p = 0;
        if (c < cells) {
            const int b = B.cell_start[c];
            count = B.cell_start[c + 1] - b;
            p = b + s;
        }
        const uint64_t fidx = s < count ? B.fidx[p] : 0u;
        const int group = threadIdx.x & 24;
        int lo = kMixed, hi = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint64_t fk = __shfl_sync(kFull, fidx, group + k);
            if (k < count) {
                const int f = field_of(fk, s);
                lo = min(lo, f);
                hi = max(hi, f);
            }
        }
        const bool mixed = count > 0 && lo != hi;
        if (count > 0) B.cell_field[(cell_base_node(P, c) + node_offset(P, s)) * 8 + s] = (uint8_t)(mixed ? kMixed : lo);
        const unsigned any = __ballot_sync(kFull, mixed);
        if (s == 0 && ((any >> group) & 0xffu)) B.mixed_cells[atomicAdd(&B.flags[BM_FLAG_MIXED_CELLS], 1)] = c;
    }
}

// Incremental registration (flags[BM_FLAG_REG_MODE] == 2).  The side labelling
// lists the stencil nodes of every particle it relabels (reg_nodes); only
// those nodes, the particles of the cells around them and those cells'
// corner flags are registered again.  Every other node, particle and cell
// keeps what it has, which equals a full registration's, because none of
// their contributors' codes changed.  The multi-field node list is rebuilt
// from the field counts (its order is immaterial: each node is summed alone).

// register_node for node n by one warp: lane l takes slots 2 (l & 3) and
// 2 (l & 3) + 1 of the cell at corner l >> 2, so the node's contributions
// load in one round trip; each field is then the smallest code above the
// previous field's, found by a warp minimum.  Same fields as register_node.
__device__ void register_node_warp(const bm_params& P, const bm_buffers& B, const int64_t* __restrict__ field_codes,
                                   int n) {
    const int lane = threadIdx.x & 31, a = lane >> 2;
    const int64_t none = INT64_MAX;  // codes stay below 3^40 < 2^63
    int64_t mine[2] = {none, none};
    const int c = cell_at(P, n, a);
    if (c >= 0) {
        const int begin = B.cell_start[c], count = B.cell_start[c + 1] - begin;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int slot = 2 * (lane & 3) + k;
            if (slot < count) mine[k] = field_codes[begin + slot];
        }
    }
    int nf = 0;
    int64_t prev = -1;  // codes are non-negative
    for (;;) {
        int64_t best = none;
#pragma unroll
        for (int k = 0; k < 2; ++k)
            if (mine[k] > prev && mine[k] < best) best = mine[k];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const int64_t other = __shfl_xor_sync(kFull, best, d);
            best = other < best ? other : best;
        }
        if (best == none) break;
        if (nf >= P.fmax) {
            if (lane == 0) atomicAdd(&B.errors[0], 1);
            break;
        }
        if (lane == 0) {
            const int s = nf * P.node_count + n;
            B.fcode[s] = best;
            uint64_t ones, twos;
            digit_masks(best, &ones, &twos);
            B.fones[s] = ones;
            B.ftwos[s] = twos;
        }
        ++nf;
        prev = best;
    }
    if (lane == 0) B.nfield[n] = nf;
}

__global__ void k_register_nodes_listed(bm_params P, bm_buffers B, const int64_t* __restrict__ field_codes) {
    if (B.flags[BM_FLAG_REG_MODE] != 2) return;
    const int count = min(B.flags[BM_FLAG_REG_NODES], P.node_count);
    const int lane = threadIdx.x & 31, warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < count; t += warps) {
        const int n = B.reg_nodes[t];
        register_node_warp(P, B, field_codes, n);
        if (lane < 8) {
            const int c = cell_at(P, n, lane);
            if (c >= 0 && B.cell_start[c + 1] != B.cell_start[c] && atomicExch(&B.reg_cell_mark[c], 1) == 0)
                B.reg_cells[atomicAdd(&B.flags[BM_FLAG_REG_CELLS], 1)] = c;
        }
    }
}

// Field indices of a listed cell's particles, then the cell's corner flags
// (as k_register_cells: the common field of a corner, or kMixed), by one
// warp: lane l takes particle slot l >> 2 of the cell and its corners
// 2 (l & 3) and 2 (l & 3) + 1.  A cell holds at most 8 particles.
__global__ void k_register_cells_listed(bm_params P, bm_buffers B, const int64_t* __restrict__ field_codes) {
    if (B.flags[BM_FLAG_REG_MODE] != 2) return;
    const int count = min(B.flags[BM_FLAG_REG_CELLS], cell_count(P));
    const int lane = threadIdx.x & 31, slot = lane >> 2, pair = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < count; t += warps) {
        const int c = B.reg_cells[t];
        const int begin = B.cell_start[c], cnt = B.cell_start[c + 1] - begin;
        const bool present = slot < cnt;
        const int p = begin + (present ? slot : 0);
        const int64_t code = field_codes[p];
        const int base = B.base_node[p];
        int f[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int node = base + node_offset(P, 2 * pair + k);
            const int nf = B.nfield[node];
            int i = 0;
            while (i < nf && B.fcode[(int64_t)i * P.node_count + node] != code) ++i;
            f[k] = i >= nf ? 0 : i;  // only after a field overflow, already counted in errors[0]
        }
        uint64_t part = ((uint64_t)f[0] << (16 * pair)) | ((uint64_t)f[1] << (16 * pair + 8));
        part |= __shfl_xor_sync(kFull, part, 1);
        part |= __shfl_xor_sync(kFull, part, 2);
        if (present && pair == 0) B.fidx[p] = part;
        // corner a = 2 pair + k over the present particles: lanes of equal pair, stride 4
        int lo[2], hi[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            lo[k] = present ? f[k] : kMixed;
            hi[k] = present ? f[k] : 0;
#pragma unroll
            for (int d = 4; d < 32; d <<= 1) {
                lo[k] = min(lo[k], __shfl_xor_sync(kFull, lo[k], d));
                hi[k] = max(hi[k], __shfl_xor_sync(kFull, hi[k], d));
            }
        }
        if (slot == 0) {
            const int cbase = cell_base_node(P, c);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int a = 2 * pair + k;
                B.cell_field[(cbase + node_offset(P, a)) * 8 + a] = (uint8_t)(lo[k] != hi[k] ? kMixed : lo[k]);
            }
        }
    }
}

// After either registration: clear the marks of the listed nodes and cells;
// after an incremental one, list the multi-field nodes again.
__global__ void k_register_finish(bm_params P, bm_buffers B) {
    const int mode = B.flags[BM_FLAG_REG_MODE];
    if (mode == 0) return;
    const int nodes = min(B.flags[BM_FLAG_REG_NODES], P.node_count);
    const int cells = min(B.flags[BM_FLAG_REG_CELLS], cell_count(P));
    const int scan = mode == 2 ? P.active_nodes : 0;
    const int total = max(max(nodes, cells), scan);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < nodes) B.reg_node_mark[B.reg_nodes[t]] = 0;
        if (t < cells) B.reg_cell_mark[B.reg_cells[t]] = 0;
        if (t < scan) {
            const int n = B.active[t];
            if (B.nfield[n] > 1) B.multi_nodes[atomicAdd(&B.flags[BM_FLAG_MULTI], 1)] = n;
        }
    }
}

__global__ void k_register_reset(bm_buffers B) {
    B.flags[BM_FLAG_REG_NODES] = 0;
    B.flags[BM_FLAG_REG_CELLS] = 0;
    B.flags[BM_FLAG_REG_MODE] = 0;
}


struct P2GContrib {
    float m;
    bm_v3 mom, J;
};
// One particle's p2g contribution to its corner a (material.py:149-152).
__device__ __forceinline__ P2GContrib p2g_contrib(const bm_params& P, const bm_buffers& B, bm_v3 v, bm_v3 imp,
                                                  const bm_m33& scaled_stress, int sid, int a) {
    const float w = stencil_w(B, sid, a);
    const bm_v3 g = stencil_g(B, sid, a);
    P2GContrib c;
    c.m = P.mass * w;
    c.mom = v3_mul(v, c.m);
    c.J = v3_sub(v3_mul(imp, w), m33_mul_v3(scaled_stress, g));
    return c;
}

// Cell pass of p2g: thread (cell, slot); the 8-slot tree sum of every corner
// written to cell_part[.][a][corner node] (meaningful where the corner is uniform).
__global__ void __launch_bounds__(256) k_p2g_cells(bm_params P, bm_buffers B) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cells = cell_count(P);
    const int c = t >> 3, s = t & 7;
    const int N = P.n, NC = P.node_count;
    int count = 0, p = 0;
    if (c < cells) {
        const int b = B.cell_start[c];
        count = B.cell_start[c + 1] - b;
        p = b + s;
    }
    const bool present = s < count;
    float vals[8][7];
    int base = 0;
    if (present) {
        const bm_v3 v = ld3(B.v, N, p), imp = ld3(B.impulses, N, p);
        const bm_m33 S = m33_scale(ld9(B.stress, N, p), P.dt * P.volume);
        const int sid = B.stencil_id[p];
        base = B.base_node[p];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const P2GContrib k = p2g_contrib(P, B, v, imp, S, sid, a);
            vals[a][0] = k.m;
            vals[a][1] = k.mom.x;
            vals[a][2] = k.mom.y;
            vals[a][3] = k.mom.z;
            vals[a][4] = k.J.x;
            vals[a][5] = k.J.y;
            vals[a][6] = k.J.z;
        }
    } else {
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int v = 0; v < 7; ++v) vals[a][v] = 0.0f;
    }
    float sum[7];
    reduce_scatter8<7>(vals, sum);
    base = __shfl_sync(kFull, base, threadIdx.x & 24);  // lane 0 of the group is present when count > 0
    if (count > 0) {
        const int plane = 8 * NC;
        float* part = B.cell_part + s * NC + base + node_offset(P, s);
#pragma unroll
        for (int v = 0; v < 7; ++v) part[v * plane] = sum[v];
    }
}

// A multi-field node staged in shared memory by its warp.  val[a][8 s + v]
// holds the V values that slot s of the cell at corner a gives the node: the
// contribution of that slot's particle at a mixed corner, the cell pass's
// partial (in slot 0) at a uniform one.  field[a][s] is the field those
// values belong to (-1: none) and flag[a] the corner's cell_field flag.  The
// row pad puts the eight corners on different banks.
struct NodeStage {
    float val[8][8 * 8 + 1];
    int field[8][9];
    int flag[8];
};

// Stage 1, lane (g, s) = (lane / 8, lane % 8): slot s of corners 7 - g and
// 3 - g.  Every load is issued without a branch (particle 0 stands in where
// a slot is not needed), so the cell words, the particles and the stencil
// rows of all 64 (corner, slot) pairs take three dependent round trips.
// With kOwnCorners a uniform corner is staged from its particles too (the
// pass then needs nothing from the cell pass and may run beside it);
// otherwise it takes the cell pass's partial in slot 0.
template <int V, bool kOwnCorners = false>
__device__ __forceinline__ void stage_node(const bm_params& P, const bm_buffers& B, int n, NodeStage& st) {
    const int lane = threadIdx.x & 31, g = lane >> 3, s = lane & 7;
    const int N = P.n, NC = P.node_count, plane = 8 * NC;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int a = 7 - (4 * h + g);
        const int c = cell_at(P, n, a);
        const int flag = B.cell_field[n * 8 + a];
        int b = 0, count = 0;
        if (c >= 0) {
            b = B.cell_start[c];
            count = B.cell_start[c + 1] - b;
        }
        const bool mixed = flag == kMixed && s < count;
        const bool uniform = flag != kMixed && flag != kAbsentCorner && (kOwnCorners ? s < count : s == 0);
        const bool own = mixed || (kOwnCorners && uniform);  // slot s's particle is staged
        const int p = own ? b + s : 0;
        const uint64_t fidx = B.fidx[p];
        const int sid = B.stencil_id[p];
        float e[V];
        if (V == 7) {
            const P2GContrib k = p2g_contrib(P, B, ld3(B.v, N, p), ld3(B.impulses, N, p),
                                             m33_scale(ld9(B.stress, N, p), P.dt * P.volume), sid, a);
            const float c7[7] = {k.m, k.mom.x, k.mom.y, k.mom.z, k.J.x, k.J.y, k.J.z};
#pragma unroll
            for (int v = 0; v < V; ++v) e[v] = c7[v];
        } else {
            const bm_v3 r = v3_mul(ld3(B.v, N, p), P.mass * stencil_w(B, sid, a));
            const float c3[3] = {r.x, r.y, r.z};
#pragma unroll
            for (int v = 0; v < V; ++v) e[v] = c3[v];
        }
        const float* part = B.cell_part + a * NC + n;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float u = kOwnCorners ? 0.0f : part[v * plane];
            st.val[a][8 * s + v] = own ? e[v] : (uniform ? u : 0.0f);
        }
        st.field[a][s] = mixed ? field_of(fidx, a) : (uniform ? flag : -1);
        // a uniform corner staged from its particles is summed like a mixed one
        if (s == 0) st.flag[a] = (kOwnCorners && flag != kAbsentCorner) ? kMixed : flag;
    }
}

// Stage 2: the values corner a gives field f - the tree sum
// ((s0+s1)+(s2+s3))+((s4+s5)+(s6+s7)) over the slots of field f at a mixed
// corner (+0 for the others, the cell pass's tree), the cell partial at a
// uniform corner of field f; false if the corner gives f nothing.
template <int V>
__device__ __forceinline__ bool staged_corner(const NodeStage& st, int a, int f, float (&out)[V]) {
    const int flag = st.flag[a];
    if (flag != kMixed) {
#pragma unroll
        for (int v = 0; v < V; ++v) out[v] = st.val[a][v];
        return flag == f;
    }
    unsigned match = 0u;
#pragma unroll
    for (int s = 0; s < 8; ++s)
        if (st.field[a][s] == f) match |= 1u << s;
    float half[2][V];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float e[4][V];
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int v = 0; v < V; ++v) e[k][v] = ((match >> (4 * h + k)) & 1u) ? st.val[a][8 * (4 * h + k) + v] : 0.0f;
#pragma unroll
        for (int v = 0; v < V; ++v) half[h][v] = (e[0][v] + e[1][v]) + (e[2][v] + e[3][v]);
    }
#pragma unroll
    for (int v = 0; v < V; ++v) out[v] = half[0][v] + half[1][v];
    return match != 0u;
}

// Stages 2 and 3 for fields f0 .. f0 + 3: lane (a, k) = (lane / 4, lane % 4)
// forms corner a's values for field f0 + k; then every lane adds, for its
// field f0 + lane % 4, the corners that have that field in ascending cell
// index (a = 7 .. 0).
template <int V>
__device__ __forceinline__ void staged_sums(const NodeStage& st, int nf, int f0, float (&sum)[V]) {
    const int lane = threadIdx.x & 31, k = lane & 3, f = f0 + k;
    float cv[V];
    const bool have = f < nf && staged_corner<V>(st, lane >> 2, f, cv);
    const unsigned haves = __ballot_sync(kFull, have);
#pragma unroll
    for (int v = 0; v < V; ++v) sum[v] = 0.0f;
#pragma unroll
    for (int a = 7; a >= 0; --a) {
        const int src = 4 * a + k;
        const bool use = (haves >> src) & 1u;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const float x = __shfl_sync(kFull, cv[v], src);
            if (use) sum[v] = sum[v] + x;
        }
    }
}

// p2g node sums + couple_and_velocity (material.py:127-152, 252-284) for the
// single-field nodes, one thread per active node (a single-field node has no
// mixed corner: each corner is field 0 or has no cell).  Also clears the
// topology flag consumed by registration.
__global__ void __launch_bounds__(256) k_p2g_grid(bm_params P, bm_buffers B, int write_sums) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) B.flags[BM_FLAG_TOPOLOGY_DIRTY] = 0;
    if (t >= P.active_nodes) return;
    const int n = B.active[t];
    if (B.nfield[n] != 1) return;
    const int NC = P.node_count, S = P.fmax * NC, plane = 8 * NC;
    const uint64_t flags = *reinterpret_cast<const uint64_t*>(B.cell_field + 8 * n);
    float part[8][7];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int v = 0; v < 7; ++v) part[a][v] = B.cell_part[v * plane + a * NC + n];
    float m = 0.0f;
    bm_v3 mom = v3_zero(), J = v3_zero();
#pragma unroll
    for (int a = 7; a >= 0; --a) {
        if (((flags >> (8 * a)) & 0xffu) != 0u) continue;  // no cell at this corner
        m = m + part[a][0];
        mom = v3_add(mom, v3(part[a][1], part[a][2], part[a][3]));
        J = v3_add(J, v3(part[a][4], part[a][5], part[a][6]));
    }
    B.grid_mass[n] = m;
    if (write_sums) {
        st3(B.momentum, S, n, mom);
        st3(B.grid_impulse, S, n, J);
    }
    if (m <= 0.0f) {
        st3(B.old_v, S, n, v3_zero());
        st3(B.new_v, S, n, v3_zero());
        return;
    }
    const bm_v3 pm = v3_add(mom, v3_div(v3_zero(), m));
    const bm_v3 jm = v3_add(J, v3_div(v3_zero(), m));
    st3(B.old_v, S, n, v3_div(pm, m));
    st3(B.new_v, S, n, v3_div(v3_add(pm, jm), m));
}

// Multi-field nodes, one warp per listed node: the node is staged (stage 1),
// then fields are summed four at a time (stages 2 and 3).  With at most four
// fields, lanes 0 .. 3 then hold every field's sums and evaluate the exchange
// (couple_and_velocity_at) by shuffles; otherwise the sums go to memory and
// lane f evaluates field f's exchange from there.
__global__ void __launch_bounds__(256) k_p2g_multi(bm_params P, bm_buffers B, int write_sums) {
    __shared__ NodeStage stage[kBlock / 32];
    NodeStage& st = stage[threadIdx.x >> 5];
    const int count = B.flags[BM_FLAG_MULTI];
    const int NC = P.node_count, S = P.fmax * NC;
    const int lane = threadIdx.x & 31, k = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < count; w += warps) {
        const int n = B.multi_nodes[w];
        const int nf = B.nfield[n];
        const int slot = k * NC + n;
        uint64_t oa = 0u, ta = 0u;
        if (nf <= 4 && k < nf) {
            oa = B.fones[slot];
            ta = B.ftwos[slot];
        }
        stage_node<7>(P, B, n, st);
        __syncwarp();
        for (int f0 = 0; f0 < nf; f0 += 4) {
            float sum[7];
            staged_sums<7>(st, nf, f0, sum);
            const int f = f0 + k;
            if (nf <= 4) {
                // every field's sums are in lanes 0 .. nf-1: exchange in ascending field
                // order by shuffles, as the general path below does from memory
                const float ma = sum[0];
                const bm_v3 pa = v3(sum[1], sum[2], sum[3]), ja = v3(sum[4], sum[5], sum[6]);
                float total = 0.0f;
                bm_v3 dm = v3_zero(), di = v3_zero();
                for (int g = 0; g < nf; ++g) {
                    const float mb = __shfl_sync(kFull, ma, g);
                    const bm_v3 pb = v3(__shfl_sync(kFull, pa.x, g), __shfl_sync(kFull, pa.y, g), __shfl_sync(kFull, pa.z, g));
                    const bm_v3 jb = v3(__shfl_sync(kFull, ja.x, g), __shfl_sync(kFull, ja.y, g), __shfl_sync(kFull, ja.z, g));
                    const uint64_t ob = __shfl_sync(kFull, oa, g), tb = __shfl_sync(kFull, ta, g);
                    total = total + mb;
                    if (g != f && compatible_masks(oa, ta, ob, tb)) {
                        dm = v3_add(dm, v3_sub(v3_mul(pb, ma), v3_mul(pa, mb)));
                        di = v3_add(di, v3_sub(v3_mul(jb, ma), v3_mul(ja, mb)));
                    }
                }
                if (lane < nf) {
                    B.grid_mass[slot] = ma;
                    if (write_sums) {
                        st3(B.momentum, S, slot, pa);
                        st3(B.grid_impulse, S, slot, ja);
                    }
                    if (ma <= 0.0f) {
                        st3(B.old_v, S, slot, v3_zero());
                        st3(B.new_v, S, slot, v3_zero());
                    } else {
                        const bm_v3 pm = v3_add(pa, v3_div(dm, total));
                        const bm_v3 jm = v3_add(ja, v3_div(di, total));
                        st3(B.old_v, S, slot, v3_div(pm, ma));
                        st3(B.new_v, S, slot, v3_div(v3_add(pm, jm), ma));
                    }
                }
                continue;
            }
            if (lane < 4 && f < nf) {
                const int sf = f * NC + n;
                B.grid_mass[sf] = sum[0];
                st3(B.momentum, S, sf, v3(sum[1], sum[2], sum[3]));
                st3(B.grid_impulse, S, sf, v3(sum[4], sum[5], sum[6]));
            }
        }
        __syncwarp();  // the stage is rewritten for the next node; the sums are visible to the warp
        if (nf <= 4) continue;
        // exchange (couple_and_velocity_at): lane f handles field f
        for (int f = lane; f < nf; f += 32) {
            const int sa = f * NC + n;
            const float ma = B.grid_mass[sa];
            if (ma <= 0.0f) {
                st3(B.old_v, S, sa, v3_zero());
                st3(B.new_v, S, sa, v3_zero());
                continue;
            }
            const bm_v3 pa = ld3(B.momentum, S, sa), ja = ld3(B.grid_impulse, S, sa);
            const uint64_t oa2 = B.fones[sa], ta2 = B.ftwos[sa];
            float total = 0.0f;
            bm_v3 dm = v3_zero(), di = v3_zero();
            for (int g = 0; g < nf; ++g) {
                const int sb = g * NC + n;
                const float mb = B.grid_mass[sb];
                total = total + mb;
                if (g != f && compatible_masks(oa2, ta2, B.fones[sb], B.ftwos[sb])) {
                    dm = v3_add(dm, v3_sub(v3_mul(ld3(B.momentum, S, sb), ma), v3_mul(pa, mb)));
                    di = v3_add(di, v3_sub(v3_mul(ld3(B.grid_impulse, S, sb), ma), v3_mul(ja, mb)));
                }
            }
            const bm_v3 pm = v3_add(pa, v3_div(dm, total));
            const bm_v3 jm = v3_add(ja, v3_div(di, total));
            st3(B.old_v, S, sa, v3_div(pm, ma));
            st3(B.new_v, S, sa, v3_div(v3_add(pm, jm), ma));
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------- G2P

// material.g2p_at (material.py:343-367), the pair-list displacement check of
// contact.check_pair_list (contact.py:716-735) on the new x, v, and the cell
// partials of the MUSL re-scatter (material.py:400-401), thread (cell, slot).
__global__ void __launch_bounds__(256) k_g2p(bm_params P, bm_buffers B, float half_skin, int check_list) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cells = cell_count(P);
    const int c = t >> 3, s = t & 7;
    const int N = P.n, S = P.fmax * P.node_count, NC = P.node_count;
    int count = 0, p = 0;
    if (c < cells) {
        const int b = B.cell_start[c];
        count = B.cell_start[c + 1] - b;
        p = b + s;
    }
    const bool present = s < count;
    float vals[8][3];
    int base = 0;
    if (present) {
        const int sid = B.stencil_id[p];
        const uint64_t fidx = B.fidx[p];
        base = B.base_node[p];
        bm_v3 pic = v3_zero(), dv = v3_zero();
        float w[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int slot = field_of(fidx, a) * NC + base + node_offset(P, a);
            w[a] = stencil_w(B, sid, a);
            const bm_v3 nv = ld3(B.new_v, S, slot);
            pic = v3_add(pic, v3_mul(nv, w[a]));
            dv = v3_add(dv, v3_mul(v3_sub(nv, ld3(B.old_v, S, slot)), w[a]));
        }
        const bm_v3 v = v3_add(v3_mul(pic, 1.0f - P.flip), v3_mul(v3_add(ld3(B.v, N, p), dv), P.flip));
        const bm_v3 x = v3_add(ld3(B.x, N, p), v3_mul(pic, P.dt));
        st3(B.v, N, p, v);
        st3(B.x, N, p, x);
        if (check_list && v3_len(v3_sub(x, ld3(B.built_x, N, p))) + P.dt * v3_len(v) > half_skin)
            B.flags[BM_FLAG_PAIR_DIRTY] = 1;
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const bm_v3 r = v3_mul(v, P.mass * w[a]);
            vals[a][0] = r.x;
            vals[a][1] = r.y;
            vals[a][2] = r.z;
        }
    } else {
#pragma unroll
        for (int a = 0; a < 8; ++a) vals[a][0] = vals[a][1] = vals[a][2] = 0.0f;
    }
    float sum[3];
    reduce_scatter8<3>(vals, sum);
    base = __shfl_sync(kFull, base, threadIdx.x & 24);
    if (count > 0) {
        float* part = B.cell_part + s * NC + base + node_offset(P, s);
        const int plane = 8 * NC;
        part[0] = sum[0];
        part[plane] = sum[1];
        part[2 * plane] = sum[2];
    }
}

// ---------------------------------------------------------- remap + couple

// Node pass of the MUSL re-scatter, then couple (material.py:155-193) for the
// single-field nodes; stores coupled / mass for the F update.
__global__ void __launch_bounds__(256) k_remap_couple(bm_params P, bm_buffers B) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int n = B.active[t];
    if (B.nfield[n] != 1) return;
    const int NC = P.node_count, S = P.fmax * NC, plane = 8 * NC;
    const uint64_t flags = *reinterpret_cast<const uint64_t*>(B.cell_field + 8 * n);
    float part[8][3];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int v = 0; v < 3; ++v) part[a][v] = B.cell_part[v * plane + a * NC + n];
    bm_v3 r = v3_zero();
#pragma unroll
    for (int a = 7; a >= 0; --a) {
        if (((flags >> (8 * a)) & 0xffu) != 0u) continue;
        r = v3_add(r, v3(part[a][0], part[a][1], part[a][2]));
    }
    const float m = B.grid_mass[n];
    if (m <= 0.0f) {
        st3(B.remap_v, S, n, v3_zero());
        return;
    }
    const bm_v3 coupled = v3_add(r, v3_div(v3_zero(), m));
    st3(B.remap_v, S, n, v3_div(coupled, m));
}

__global__ void __launch_bounds__(256, 4) k_remap_multi(bm_params P, bm_buffers B) {
    __shared__ NodeStage stage[kBlock / 32];
    NodeStage& st = stage[threadIdx.x >> 5];
    const int count = B.flags[BM_FLAG_MULTI];
    const int NC = P.node_count, S = P.fmax * NC;
    const int lane = threadIdx.x & 31, k = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < count; w += warps) {
        const int n = B.multi_nodes[w];
        const int nf = B.nfield[n];
        const int slot = k * NC + n;
        float ma = 0.0f;
        uint64_t oa = 0u, ta = 0u;
        if (nf <= 4 && k < nf) {
            ma = B.grid_mass[slot];
            oa = B.fones[slot];
            ta = B.ftwos[slot];
        }
        stage_node<3>(P, B, n, st);
        __syncwarp();
        for (int f0 = 0; f0 < nf; f0 += 4) {
            float sum[3];
            staged_sums<3>(st, nf, f0, sum);
            const int f = f0 + k;
            if (nf <= 4) {
                // couple (couple_at) by shuffles, ascending field order as in the general path
                const bm_v3 va = v3(sum[0], sum[1], sum[2]);
                float total = 0.0f;
                bm_v3 ex = v3_zero();
                for (int g = 0; g < nf; ++g) {
                    const float mb = __shfl_sync(kFull, ma, g);
                    const bm_v3 vb = v3(__shfl_sync(kFull, va.x, g), __shfl_sync(kFull, va.y, g), __shfl_sync(kFull, va.z, g));
                    const uint64_t ob = __shfl_sync(kFull, oa, g), tb = __shfl_sync(kFull, ta, g);
                    total = total + mb;
                    if (g != f && compatible_masks(oa, ta, ob, tb)) ex = v3_add(ex, v3_sub(v3_mul(vb, ma), v3_mul(va, mb)));
                }
                if (lane < nf) {
                    st3(B.remapped, S, slot, va);
                    if (ma <= 0.0f) st3(B.remap_v, S, slot, v3_zero());
                    else st3(B.remap_v, S, slot, v3_div(v3_add(va, v3_div(ex, total)), ma));
                }
                continue;
            }
            if (lane < 4 && f < nf) st3(B.remapped, S, f * NC + n, v3(sum[0], sum[1], sum[2]));
        }
        __syncwarp();  // the stage is rewritten for the next node; the sums are visible to the warp
        if (nf <= 4) continue;
        for (int f = lane; f < nf; f += 32) {
            const int sa = f * NC + n;
            const float mf = B.grid_mass[sa];
            if (mf <= 0.0f) {
                st3(B.remap_v, S, sa, v3_zero());
                continue;
            }
            const bm_v3 va = ld3(B.remapped, S, sa);
            const uint64_t oa2 = B.fones[sa], ta2 = B.ftwos[sa];
            float total = 0.0f;
            bm_v3 ex = v3_zero();
            for (int g = 0; g < nf; ++g) {
                const int sb = g * NC + n;
                const float mb = B.grid_mass[sb];
                total = total + mb;
                if (g != f && compatible_masks(oa2, ta2, B.fones[sb], B.ftwos[sb]))
                    ex = v3_add(ex, v3_sub(v3_mul(ld3(B.remapped, S, sb), mf), v3_mul(va, mb)));
            }
            st3(B.remap_v, S, sa, v3_div(v3_add(va, v3_div(ex, total)), mf));
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------- constitutive

// Fixed-corotated first Piola stress through the polar rotation:
// P = 2 mu (f - R) + lam (J - 1) J f^-T, equal to material.corotated_stress
// (material.py:78-91) with Fp = I.
__device__ __forceinline__ bm_m33 corotated_polar(const bm_m33& f, float J, float mu, float lam) {
    bm_m33 inv_t;  // f^-T, the polar iteration's first inverse transpose
    const bm_m33 R = bm_polar3_inv(f, &inv_t);
    const float c = lam * (J - 1.0f) * J, two_mu = 2.0f * mu;
    bm_m33 out;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) out.m[i][j] = two_mu * (f.m[i][j] - R.m[i][j]) + c * inv_t.m[i][j];
    return out;
}

// material.stress_at (material.py:94-112) of the deformation gradient F of
// particle p (the caller's copy of buffers.F[p]).
__device__ __forceinline__ void stress_of(const bm_params& P, const bm_buffers& B, int p, const bm_m33& F) {
    const int N = P.n;
    bm_m33 f = F, pinv = m33_identity();
    if (P.use_fp) {
        pinv = m33_inverse(ld9(B.Fp, N, p));
        f = m33_mul(F, pinv);
    }
    const float J = m33_det(f);
    if (J <= 0.0f || !bm_isfinitef(J)) {
        atomicAdd(&B.errors[1], 1);
        st9(B.stress, N, p, m33_zero());
        return;
    }
    if (P.use_fp) st9(B.stress, N, p, m33_mul(corotated_polar(f, J, P.mu, P.lam), m33_transpose(pinv)));
    else st9(B.stress, N, p, corotated_polar(f, J, P.mu, P.lam));
}
__device__ void stress_at(const bm_params& P, const bm_buffers& B, int p) { stress_of(P, B, p, ld9(B.F, P.n, p)); }

// material.plastic_at (material.py:404-431).
__device__ bool plastic_at(const bm_params& P, const bm_buffers& B, int p, float yield_stress, bm_m33* U, bm_v3* s,
                           bm_m33* V) {
    const int N = P.n;
    const bm_m33 F = ld9(B.F, N, p);
    bm_svd3(m33_mul(F, m33_inverse(ld9(B.Fp, N, p))), U, s, V);
    if (bm_minf(bm_minf(s->x, s->y), s->z) <= 0.0f) {
        atomicAdd(&B.errors[1], 1);
        return false;
    }
    const bm_v3 e = v3(bm_logf(s->x), bm_logf(s->y), bm_logf(s->z));
    const float mean = ((e.x + e.y) + e.z) / 3.0f;
    const bm_v3 dev = v3_sub(e, v3(mean, mean, mean));
    const float norm = v3_len(dev);
    const float limit = yield_stress / (2.0f * P.mu) * sqrtf(2.0f / 3.0f);
    if (norm > limit) {
        const bm_v3 ep = v3_sub(e, v3_mul(dev, 1.0f - limit / norm));
        *s = v3(bm_expf(ep.x), bm_expf(ep.y), bm_expf(ep.z));
        const bm_m33 next_f = m33_mul(m33_mul(*U, m33_diag(*s)), m33_transpose(*V));
        st9(B.Fp, N, p, m33_mul(m33_inverse(next_f), F));
    }
    return true;
}

// material.maxwell_at (material.py:485-533).
__device__ void maxwell_at(const bm_params& P, const bm_buffers& B, int p, const bm_m33& U, bm_v3 sigma,
                           const bm_m33& V, float relax) {
    const int N = P.n;
    const bm_m33 f = m33_mul(m33_mul(U, m33_diag(sigma)), m33_transpose(V));
    double D[9];
    for (int r = 0; r < 9; ++r) D[r] = B.viscous[r * N + p];
    bm_m33 Df;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Df.m[r][c] = (float)D[3 * r + c];
    const bm_m33 fm = m33_mul(f, m33_inverse(m33_add(m33_identity(), Df)));
    bm_m33 Um, Vm;
    bm_v3 sm;
    bm_svd3(fm, &Um, &sm, &Vm);
    if (bm_minf(bm_minf(sm.x, sm.y), sm.z) <= 0.0f) {
        atomicAdd(&B.errors[1], 1);
        st9(B.stress, N, p, m33_zero());
        return;
    }
    const bm_v3 e = v3(bm_logf(sm.x), bm_logf(sm.y), bm_logf(sm.z));
    const float mean = ((e.x + e.y) + e.z) / 3.0f;
    bm_v3 dev = v3_sub(e, v3(mean, mean, mean));
    if (relax > 0.0f) {
        const bm_v3 step = v3_mul(dev, relax);
        dev = v3_sub(dev, step);
        // f_m <- f_m W with W = Vm diag(exp(-step)) Vm^T, i.e. Fv <- W^-1 Fv (material.py:518-521)
        const bm_v3 growth = v3(bm_expm1f(step.x), bm_expm1f(step.y), bm_expm1f(step.z));
        const bm_m33 delta = m33_mul(m33_mul(Vm, m33_diag(growth)), m33_transpose(Vm));
        double dd[9], nd[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dd[3 * r + c] = (double)delta.m[r][c];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                double prod = 0.0;
                for (int k = 0; k < 3; ++k) prod = prod + dd[3 * r + k] * D[3 * k + c];
                nd[3 * r + c] = (D[3 * r + c] + dd[3 * r + c]) + prod;
            }
        for (int r = 0; r < 9; ++r) B.viscous[r * N + p] = nd[r];
    }
    const bm_m33 kirchhoff = m33_mul(m33_mul(Um, m33_diag(v3_mul(dev, 2.0f * P.mu_maxwell))), m33_transpose(Um));
    const float mu_eq = P.mu - P.mu_maxwell;
    const float lam_eq = P.lam + 2.0f / 3.0f * P.mu_maxwell;
    const bm_m33 equilibrium = corotated_svd(U, sigma, V, m33_inverse(ld9(B.Fp, N, p)), mu_eq, lam_eq);
    st9(B.stress, N, p, m33_add(equilibrium, m33_mul(kirchhoff, m33_transpose(m33_inverse(ld9(B.F, N, p))))));
}

// material.maxwell_stress_at (material.py:536-566).
// material.maxwell_stress_at (material.py:536-566); with project == 0 the
// stress of the current F, Fp and Fv alone (compute_stress_maxwell,
// material.py:569-589: no return map, relax must be 0).
__device__ void maxwell_stress_at(const bm_params& P, const bm_buffers& B, int p, float relax, int project = 1) {
    const int N = P.n;
    bm_m33 U, V;
    bm_v3 sigma;
    if (project && P.yield_stress > 0.0f) {
        if (!plastic_at(P, B, p, P.yield_stress, &U, &sigma, &V)) {
            st9(B.stress, N, p, m33_zero());
            return;
        }
        maxwell_at(P, B, p, U, sigma, V, relax);
        return;
    }
    const bm_m33 f = m33_mul(ld9(B.F, N, p), m33_inverse(ld9(B.Fp, N, p)));
    const float J = m33_det(f);
    if (J <= 0.0f || !bm_isfinitef(J)) {
        atomicAdd(&B.errors[1], 1);
        st9(B.stress, N, p, m33_zero());
        return;
    }
    bm_svd3(f, &U, &sigma, &V);
    maxwell_at(P, B, p, U, sigma, V, relax);
}

__device__ void constitutive(const bm_params& P, const bm_buffers& B, int p) {
    if (P.maxwell) {
        maxwell_stress_at(P, B, p, P.maxwell_relax);
    } else if (P.plastic) {
        bm_m33 U, V;
        bm_v3 s;
        if (plastic_at(P, B, p, P.yield_stress, &U, &s, &V))
            st9(B.stress, P.n, p, corotated_svd(U, s, V, m33_inverse(ld9(B.Fp, P.n, p)), P.mu, P.lam));
        else
            st9(B.stress, P.n, p, m33_zero());
    } else {
        stress_at(P, B, p);
    }
}

// material.compute_stress / compute_stress_maxwell (material.py:115-124, 569-589).
__global__ void k_refresh_stress(bm_params P, bm_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    if (P.maxwell) maxwell_stress_at(P, B, p, 0.0f, 0);
    else stress_at(P, B, p);
}

// material.plastic_project (material.py:434-442) on caller arrays.
__global__ void k_plastic_project(float* F, float* Fp, int n, float mu, float yield_stress, int32_t* errors) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    bm_params P = {};
    P.n = n;
    P.mu = mu;
    bm_buffers B = {};
    B.F = F;
    B.Fp = Fp;
    B.errors = errors;
    bm_m33 U, V;
    bm_v3 s;
    plastic_at(P, B, p, yield_stress, &U, &s, &V);
}

// contact.assign (contact.py:996-1039) for every knife, knife k labelling the
// digit 3^(cut_index + k).  The band tests run before the digit test (both
// must hold, neither has side effects), so the int64 division only runs for
// particles in a knife's band.
__device__ void assign_sides(const bm_params& P, const bm_buffers& B, int p, int cut_index, int cutting, bm_v3 xp,
                             bm_v3 vp, unsigned knives) {
    if (cutting == 0) return;
    int64_t code = 0;
    bool loaded = false, changed = false;
    const float band = 6.0f * P.spacing;
    for (int k = 0; k < P.tool_count; ++k) {
        if (((knives >> k) & 1u) == 0u) continue;
        const ToolF T = load_tool(B.tool_f + BM_TOOL_F_WORDS * k);
        const bm_v3 d = v3_sub(xp, T.edge);
        // cheap conservative band test on the knife axes (1 um beyond the exact bounds)
        if (fabsf(v3_dot(d, T.ax)) > band + 1.0e-6f || fabsf(v3_dot(d, T.ay)) > P.half[1] + 1.0e-6f) continue;
        const bm_v3 local = q_rotate_inv(T.rot, d);
        if (!(fabsf(local.x) <= band && fabsf(local.y) <= P.half[1])) continue;
        const float front = -local.z;
        const float advance = v3_dot(v3_sub(T.edge_vel, vp), T.down);
        const float back = 2.0f * P.spacing + bm_maxf(advance * P.dt, 0.0f);
        const bool behind = front >= -back && front <= 0.0f;
        bool pinched = false;
        if (!behind) {
            const bool on_board = (P.board_half[0] == 0.0f || fabsf(xp.x) <= P.board_half[0]) &&
                                  (P.board_half[1] == 0.0f || fabsf(xp.y) <= P.board_half[1]);
            if (on_board) {
                const bm_v3 edge_here = v3_add(T.edge, q_rotate(T.rot, v3(0.0f, local.y, 0.0f)));
                pinched = edge_here.z <= P.radius && xp.z <= edge_here.z + P.radius;
            }
        }
        if (!(behind || pinched)) continue;
        if (!loaded) {
            code = B.codes[p];
            loaded = true;
        }
        int64_t digit = 1;
        for (int e = 0; e < cut_index + k; ++e) digit *= 3;
        if ((code / digit) % 3 != 0) continue;
        code += digit * (local.x < 0.0f ? 1 : 2);
        changed = true;
    }
    if (changed) {
        B.codes[p] = code;
        B.flags[BM_FLAG_TOPOLOGY_DIRTY] = 1;
        // the pair lists of p and its neighbours are recomputed before the next pair pass
        const int at = atomicAdd(&B.flags[BM_FLAG_CHANGED], 1);
        if (at < P.n) B.changed[at] = p;
        // and the nodes it weighs are registered again at the next registration
        const int base = B.base_node[p];
        for (int a = 0; a < 8; ++a) {
            const int n = base + node_offset(P, a);
            if (atomicExch(&B.reg_node_mark[n], 1) == 0) B.reg_nodes[atomicAdd(&B.flags[BM_FLAG_REG_NODES], 1)] = n;
        }
    }
}

// Knives that may label some particle of this warp (the same mask in every
// lane).  assign_sides labels a particle only inside the knife's band (within
// 6 h on the knife's x axis and the half length on its y axis) and either
// just behind the edge (local z in [0, back], back = 2 h + max(advance dt, 0)
// with advance <= |edge velocity| + |v|) or pinched at the board (the edge
// within one radius of z = 0 and the particle within one radius above it).
// A knife is left out when the warp's bounding box, widened by 2 um for
// rounding, misses the band or misses both the slab behind the edge and the
// pinch region; every particle of the warp then fails assign_sides' tests.
__device__ unsigned band_knives(const bm_params& P, const bm_buffers& B, bm_v3 x, float speed, bool active) {
    bm_v3 c, e;
    float vmax;
    bool any;
    warp_box(x, speed, active, &c, &e, &vmax, &any);
    if (!any) return 0u;
    const int k = threadIdx.x & 31;
    bool near = false;
    if (k < P.tool_count) {
        const ToolF T = load_tool(B.tool_f + BM_TOOL_F_WORDS * k);
        const bm_v3 d = v3_sub(c, T.edge);
        const float slack = 2.0e-6f;
        const bool band = !(fabsf(v3_dot(d, T.ax)) - box_reach(T.ax, e) > 6.0f * P.spacing + slack ||
                            fabsf(v3_dot(d, T.ay)) - box_reach(T.ay, e) > P.half[1] + slack);
        const float z = v3_dot(d, T.az), reach = box_reach(T.az, e);
        const float back = 2.0f * P.spacing + P.dt * (v3_len(T.edge_vel) + vmax);
        // written as "not certainly outside", so a NaN in the box keeps the knife
        const bool behind = !(z + reach < -slack || z - reach > back + slack);
        const float sway = P.half[1] * fabsf(T.ay.z);  // edge height change along the blade
        const bool pinch = !(T.edge.z - sway > P.radius + slack || c.z - e.z > T.edge.z + sway + P.radius + slack);
        near = band && (behind || pinch);
    }
    return __ballot_sync(0xffffffffu, near);
}

// contact.assign (contact.py:996-1039) for every knife, after this substep's
// tool update: the warp's knife-band cull, then each particle's band and digit
// tests.  Reads x and v last in the substep, which leaves them in L2 for the
// next substep's contact pass.
__global__ void __launch_bounds__(256) k_assign(bm_params P, bm_buffers B, int cut_index, int cutting) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < P.n;
    const int N = P.n;
    // the whole warp takes part in the knife mask, so no lane leaves before it
    const bm_v3 xp = active ? ld3(B.x, N, p) : v3_zero(), vp = active ? ld3(B.v, N, p) : v3_zero();
    const unsigned knives = band_knives(P, B, xp, v3_len(vp), active);
    if (active && knives != 0u) assign_sides(P, B, p, cut_index, cutting, xp, vp, knives);
}

// update_F_plastic / update_F_maxwell (material.py:445-475, 592-618); thread
// 0 advances the substep counter of the friction-history ping-pong.  The
// elastic update (kMinBlocks 4: polar stress only, launched when neither
// plasticity nor the Maxwell element is on) runs at 4 blocks per SM (64
// registers); the SVD-based plastic and Maxwell updates get the registers
// their Jacobi sweeps need (kMinBlocks 1), where a 64-register cap spills them.
template <int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) k_fupdate(bm_params P, bm_buffers B, int do_update, int advance_step) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (advance_step && p == 0) B.flags[BM_FLAG_STEP] += 1;
    const bool active = p < P.n;
    const int N = P.n, S = P.fmax * P.node_count;
    if (!active) return;
    if (do_update) {
        const int sid = B.stencil_id[p], base = B.base_node[p];
        const uint64_t fidx = B.fidx[p];
        // update_F sums over slots with mass > 0.  The remap passes store a zero
        // velocity in every registered slot without mass, and adding the (+-0)
        // outer product of a zero velocity leaves the sum unchanged (it starts
        // at +0 and never becomes -0), so all 8 corners are read unconditionally.
        bm_m33 rate = m33_zero();
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int s = slot_of(P, base, fidx, a);
            rate = m33_add(rate, m33_outer(ld3(B.remap_v, S, s), stencil_g(B, sid, a)));
        }
        const bm_m33 F = m33_add(ld9(B.F, N, p), m33_scale(rate, P.dt));
        st9(B.F, N, p, F);
        // the elastic stress from the new F in registers, the SVD-based laws from buffers.F
        if (kMinBlocks == 4) stress_of(P, B, p, F);
        else constitutive(P, B, p);
    }
}

// material.validate_interval (material.py:6-20).
__global__ void k_validate(bm_params P, bm_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const int N = P.n;
    const float d = m33_det(ld9(B.F, N, p));
    int bad = (d <= 0.0f || !bm_isfinitef(d)) ? 1 : 0;
    for (int i = 0; i < 3; ++i) {
        if (!bm_isfinitef(B.x[i * N + p])) ++bad;
        if (!bm_isfinitef(B.v[i * N + p])) ++bad;
    }
    if (bad) atomicAdd(&B.errors[1], bad);
}

// viscous_impulse (material.py:321-340): per-particle viscous stress, then a
// per-slot gather added to grid_impulse in ascending particle order.
__global__ void k_viscous_stress(bm_params P, bm_buffers B, float* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const int N = P.n, S = P.fmax * P.node_count;
    const int sid = B.stencil_id[p], base = B.base_node[p];
    const uint64_t fidx = B.fidx[p];
    bm_m33 rate = m33_zero();
    for (int a = 0; a < 8; ++a)
        rate = m33_add(rate, m33_outer(ld3(B.old_v, S, slot_of(P, base, fidx, a)), stencil_g(B, sid, a)));
    const bm_m33 F = ld9(B.F, N, p);
    const bm_m33 inv = m33_inverse(F);
    const bm_m33 L = m33_mul(rate, inv);
    st9(out, N, p, m33_mul(m33_scale(m33_add(L, m33_transpose(L)), P.dynamic_viscosity * m33_det(F)), m33_transpose(inv)));
}

__global__ void k_viscous_gather(bm_params P, bm_buffers B, const float* __restrict__ vstress) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int n = B.active[t];
    const int nf = B.nfield[n];
    const int N = P.n, S = P.fmax * P.node_count;
    const float scale = -P.dt * P.volume;
    for (int f = 0; f < nf; ++f) {
        const int slot = f * P.node_count + n;
        bm_v3 J = ld3(B.grid_impulse, S, slot);
        for_contributions(P, B, n, [&](int p, int a) {
            if (field_of(B.fidx[p], a) != f) return;
            J = v3_add(J, m33_mul_v3(m33_scale(ld9(vstress, N, p), scale), stencil_g(B, B.stencil_id[p], a)));
        });
        st3(B.grid_impulse, S, slot, J);
    }
}

// couple (material.py:155-193) of `state` into `result` and grid_vel
// (material.py:212-249) on every field of every active node.  mode 0: couple
// state -> result; mode 1: old/new velocity from momentum `state` and
// impulse `result`.
__global__ void k_couple_slots(bm_params P, bm_buffers B, const float* __restrict__ state, float* __restrict__ result) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int n = B.active[t];
    const int nf = B.nfield[n];
    const int S = P.fmax * P.node_count;
    for (int f = 0; f < nf; ++f) {
        const int a = f * P.node_count + n;
        const float ma = B.grid_mass[a];
        if (ma <= 0.0f) continue;
        const bm_v3 sa = ld3(state, S, a);
        const uint64_t oa = B.fones[a], ta = B.ftwos[a];
        float total = 0.0f;
        bm_v3 ex = v3_zero();
        for (int g = 0; g < nf; ++g) {
            const int b = g * P.node_count + n;
            const float mb = B.grid_mass[b];
            total = total + mb;
            if (g != f && compatible_masks(oa, ta, B.fones[b], B.ftwos[b]))
                ex = v3_add(ex, v3_sub(v3_mul(ld3(state, S, b), ma), v3_mul(sa, mb)));
        }
        st3(result, S, a, v3_add(sa, v3_div(ex, total)));
    }
}

__global__ void k_grid_vel(bm_params P, bm_buffers B, const float* __restrict__ momentum, const float* __restrict__ impulse) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int n = B.active[t];
    const int nf = B.nfield[n];
    const int S = P.fmax * P.node_count;
    for (int f = 0; f < nf; ++f) {
        const int s = f * P.node_count + n;
        const float m = B.grid_mass[s];
        if (m > 0.0f) {
            const bm_v3 pm = ld3(momentum, S, s);
            st3(B.old_v, S, s, v3_div(pm, m));
            st3(B.new_v, S, s, v3_div(v3_add(pm, ld3(impulse, S, s)), m));
        }
    }
}

// --------------------------------------------------------------- launches

void launch_register(const bm_solver* s, const int64_t* field_codes, int force, cudaStream_t st, int begin) {
    const bm_params& P = s->P;
    const unsigned wide = 8 * 152;  // grid-stride: cheap to launch when the gate is off
    const unsigned gn = grid_for(P.active_nodes) < wide ? grid_for(P.active_nodes) : wide;
    const unsigned gp = grid_for(P.n) < wide ? grid_for(P.n) : wide;
    const int cells8 = 8 * P.cell_dims[0] * P.cell_dims[1] * P.cell_dims[2];
    const unsigned gc = grid_for(cells8) < wide ? grid_for(cells8) : wide;
    if (begin) k_register_begin<<<1, 1, 0, st>>>(s->B, force);
    // full registration (each kernel returns at once unless the mode is 1)
    k_register_nodes<<<gn, kBlock, 0, st>>>(P, s->B, field_codes);
    k_register_particles<<<gp, kBlock, 0, st>>>(P, s->B, field_codes);
    k_register_cells<<<gc, kBlock, 0, st>>>(P, s->B);
    // incremental registration (mode 2): a few hundred nodes and cells at most per substep
    k_register_nodes_listed<<<152, kBlock, 0, st>>>(P, s->B, field_codes);
    k_register_cells_listed<<<152, kBlock, 0, st>>>(P, s->B, field_codes);
    k_register_finish<<<gn, kBlock, 0, st>>>(P, s->B);
    k_register_reset<<<1, 1, 0, st>>>(s->B);
}

// Runs launch(q) on aux beside the work queued on st after this call, or on st
// when aux is null; join_aux then makes st wait for it.
template <class Launch>
static void fork_aux(const bm_solver* s, cudaStream_t st, cudaStream_t aux, Launch launch) {
    if (!aux) {
        launch(st);
        return;
    }
    cudaEventRecord(s->aux_fork, st);
    cudaStreamWaitEvent(aux, s->aux_fork, 0);
    launch(aux);
    cudaEventRecord(s->aux_join, aux);
}
static void join_aux(const bm_solver* s, cudaStream_t st, cudaStream_t aux) {
    if (aux) cudaStreamWaitEvent(st, s->aux_join, 0);
}

void launch_material(const bm_solver* s, int write_sums, cudaStream_t st, cudaStream_t aux) {
    const bm_params& P = s->P;
    const bm_buffers& B = s->B;
    const int cells8 = 8 * P.cell_dims[0] * P.cell_dims[1] * P.cell_dims[2];
    const int sums = P.viscous ? 1 : write_sums;
    const int tc = spread_block(cells8);
    // the multi-field nodes stage every corner from the particles, so they
    // run beside the cell pass and the single-field node pass
    k_p2g_cells<<<grid_for(cells8, tc), tc, 0, st>>>(P, B);
    fork_aux(s, st, aux, [&](cudaStream_t q) { k_p2g_multi<<<4 * 152, kBlock, 0, q>>>(P, B, sums); });
    k_p2g_grid<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, sums);
    join_aux(s, st, aux);
    if (P.viscous) {
        // solver.py:433-459: couple momentum, velocities, viscous impulse, couple impulse, velocities.
        k_couple_slots<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, B.momentum, B.remapped);
        k_grid_vel<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, B.remapped, B.grid_impulse);
        k_viscous_stress<<<grid_for(P.n), kBlock, 0, st>>>(P, B, s->viscous_scratch);
        k_viscous_gather<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, s->viscous_scratch);
        // coupled impulse into remap_v as scratch (overwritten by the remap below)
        k_couple_slots<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, B.grid_impulse, B.remap_v);
        k_grid_vel<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B, B.remapped, B.remap_v);
    }
}

void launch_g2p(const bm_solver* s, cudaStream_t st) {
    const bm_params& P = s->P;
    const int cells8 = 8 * P.cell_dims[0] * P.cell_dims[1] * P.cell_dims[2];
    const int tc = spread_block(cells8);
    k_g2p<<<grid_for(cells8, tc), tc, 0, st>>>(P, s->B, 0.5f * P.pair_skin, P.pair_search == 0 ? 1 : 0);
}

void launch_remap(const bm_solver* s, cudaStream_t st, cudaStream_t aux) {
    const bm_params& P = s->P;
    fork_aux(s, st, aux, [&](cudaStream_t q) { k_remap_multi<<<4 * 152, kBlock, 0, q>>>(P, s->B); });
    k_remap_couple<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, s->B);
    join_aux(s, st, aux);
}

void launch_fupdate(const bm_solver* s, int do_update, int advance_step, cudaStream_t st) {
    const int tb = spread_block(s->P.n);
    if (!(do_update || advance_step)) return;
    if (s->P.maxwell || s->P.plastic)
        k_fupdate<1><<<grid_for(s->P.n, tb), tb, 0, st>>>(s->P, s->B, do_update, advance_step);
    else
        k_fupdate<4><<<grid_for(s->P.n, tb), tb, 0, st>>>(s->P, s->B, do_update, advance_step);
}

void launch_assign(const bm_solver* s, int cut_index, int cutting, cudaStream_t st) {
    const int tb = spread_block(s->P.n);
    if (cutting) k_assign<<<grid_for(s->P.n, tb), tb, 0, st>>>(s->P, s->B, cut_index, cutting);
}

void launch_refresh_stress(const bm_solver* s, cudaStream_t st) {
    k_refresh_stress<<<grid_for(s->P.n), kBlock, 0, st>>>(s->P, s->B);
}

void launch_validate(const bm_solver* s, cudaStream_t st) {
    k_validate<<<grid_for(s->P.n), kBlock, 0, st>>>(s->P, s->B);
}

void launch_clear_flag(const bm_solver* s, int which, cudaStream_t st) { k_clear_flag<<<1, 1, 0, st>>>(s->B, which); }

void launch_plastic_project(float* F, float* Fp, int n, float mu, float yield_stress, int32_t* errors, cudaStream_t st) {
    k_plastic_project<<<grid_for(n), kBlock, 0, st>>>(F, Fp, n, mu, yield_stress, errors);
}

}  // namespace bm
