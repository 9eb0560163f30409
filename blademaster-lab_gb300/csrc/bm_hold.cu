// Held-blade grid constraint (blademaster_warp/blade_constraint.py): for an
// external tool in hold mode, after the grid velocities and before G2P, the
// broad-face contacts of knife 0 get non-negative normal impulses that stop
// grid transport through the faces (W lambda >= rhs, lambda >= 0, solved by
// projected gradient with a row-sum diagonal bound and k / (k + 3)
// extrapolation, batches of 48 iterations, at most 8 batches).
//
// Contacts are few (particles within a proxy radius of a face), so the
// iterations run in one 1024-thread block: every phase is separated by a
// block barrier and no thread waits on another block.  Grid sums run per
// (node, field) over the contacts at that node in ascending particle order
// (adjacent cells in ascending index, particles of a cell in order), a fixed
// order shared with the CPU oracle, so the results are bit-identical to it.
// The scatter and couple results use the remapped / remap_v planes as
// scratch: they are free between the grid velocities and the remap.
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {
namespace {

constexpr unsigned kAll = 0xffffffffu;
enum HoldRow { kSide = 0, kNormal = 1, kLever = 4, kRhs = 7, kBound = 8, kImpulse = 9, kExtrapolated = 10 };

__device__ __forceinline__ float* row(const bm_buffers& B, int n, int r) { return B.hold + (int64_t)r * n; }

// prepare (blade_constraint.py:13-70).
__global__ void k_hold_prepare(bm_params P, bm_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool needs = false;
    if (p < P.n) {
        const int N = P.n, S = P.fmax * P.node_count;
        const ToolF T = load_tool(B.tool_f);
        const bm_v3 local = q_rotate_inv(T.rot, v3_sub(ld3(B.x, N, p), T.pos));
        float* side_row = row(B, N, kSide);
        int mark = 0;
        float side = 0.0f;
        if (!(fabsf(local.y) >= P.half[1] || local.z <= -P.half[2] + P.bevel || local.z >= P.half[2])) {
            const int sid = B.stencil_id[p], base = B.base_node[p];
            const uint64_t fidx = B.fidx[p];
            bm_v3 grid_v = v3_zero();
#pragma unroll
            for (int a = 0; a < 8; ++a)
                grid_v = v3_add(grid_v, v3_mul(ld3(B.new_v, S, slot_of(P, base, fidx, a)), stencil_w(B, sid, a)));
            side = side_row[p];
            if (side == 0.0f || fabsf(local.x) > P.half[0] + P.blade_offset) side = local.x < 0.0f ? -1.0f : 1.0f;
            const bm_v3 n = q_rotate(T.rot, v3(side, 0.0f, 0.0f));
            const float gap = side * local.x - P.half[0];
            if (gap > P.blade_offset && gap + P.dt * v3_dot(grid_v, n) > 0.0f) {
                side = 0.0f;
            } else {
                mark = 1;
                st3(row(B, N, kNormal), N, p, n);
                st3(row(B, N, kLever), N, p, q_rotate(T.rot, v3(side * P.half[0], local.y, local.z)));
                const float rhs = -bm_maxf(gap, 0.0f) / P.dt - v3_dot(grid_v, n);
                row(B, N, kRhs)[p] = rhs;
                row(B, N, kImpulse)[p] = 0.0f;
                row(B, N, kExtrapolated)[p] = 0.0f;
                needs = rhs > 1.0e-7f;
            }
        }
        side_row[p] = side;
        B.hold_mark[p] = mark;
    }
    if (__any_sync(kAll, needs) && (threadIdx.x & 31) == 0) B.flags[BM_FLAG_HOLD_NEEDS] = 1;
}

// Contact list (ascending) and the grid nodes the contacts touch.
__global__ void k_hold_list(bm_params P, bm_buffers B) {
    if (B.flags[BM_FLAG_HOLD_NEEDS] == 0) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) {
        if (B.hold_mark[p] == 0) continue;
        B.hold_list[B.hold_pos[p]] = p;
        const int base = B.base_node[p];
        for (int a = 0; a < 8; ++a) {
            const int node = base + node_offset(P, a);
            if (atomicExch(&B.hold_node_mark[node], 1) == 0) B.hold_nodes[atomicAdd(&B.flags[BM_FLAG_HOLD_NODES], 1)] = node;
        }
    }
}

// Inclusive scan of one int per thread of a 1024-thread block.
__device__ int block_scan(int v, int* s) {
    const int t = threadIdx.x;
    s[t] = v;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const int add = t >= d ? s[t - d] : 0;
        __syncthreads();
        s[t] += add;
        __syncthreads();
    }
    const int r = s[t];
    __syncthreads();
    return r;
}

enum Source { kOnes = 0, kFromExtrapolated = 1, kFromImpulse = 2 };

// scatter (blade_constraint.py:93-111) of w j for the contacts, then couple
// (material.py:155-179) at every listed node: G in `remapped`, C in `remap_v`.
__device__ void scatter_couple(const bm_params& P, const bm_buffers& B, int nodes, Source src) {
    const int N = P.n, NC = P.node_count, S = P.fmax * NC;
    for (int t = threadIdx.x; t < nodes; t += blockDim.x) {
        const int X = B.hold_nodes[t], nf = B.nfield[X];
        const int begin = B.hold_node_start[t], end = B.hold_node_start[t + 1];
        for (int f = 0; f < nf; ++f) {
            bm_v3 g = v3_zero();
            for (int k = begin; k < end; ++k) {
                const int e = B.hold_entry[k], p = e >> 3, a = e & 7;
                if (field_of(B.fidx[p], a) != f) continue;
                bm_v3 j = v3(1.0f, 0.0f, 0.0f);
                if (src != kOnes)
                    j = v3_mul(ld3(row(B, N, kNormal), N, p), row(B, N, src == kFromImpulse ? kImpulse : kExtrapolated)[p]);
                g = v3_add(g, v3_mul(j, stencil_w(B, B.stencil_id[p], a)));
            }
            st3(B.remapped, S, f * NC + X, g);
        }
        for (int f = 0; f < nf; ++f) {
            const int sa = f * NC + X;
            const float ma = B.grid_mass[sa];
            if (ma <= 0.0f) {
                st3(B.remap_v, S, sa, v3_zero());
                continue;
            }
            const bm_v3 ga = ld3(B.remapped, S, sa);
            const uint64_t oa = B.fones[sa], ta = B.ftwos[sa];
            float total = 0.0f;
            bm_v3 ex = v3_zero();
            for (int h = 0; h < nf; ++h) {
                const int sb = h * NC + X;
                const float mb = B.grid_mass[sb];
                total = total + mb;
                if (h != f && compatible_masks(oa, ta, B.fones[sb], B.ftwos[sb]))
                    ex = v3_add(ex, v3_sub(v3_mul(ld3(B.remapped, S, sb), ma), v3_mul(ga, mb)));
            }
            st3(B.remap_v, S, sa, v3_add(ga, v3_div(ex, total)));
        }
    }
}

// response_at (blade_constraint.py:114-127) from C.
__device__ bm_v3 response(const bm_params& P, const bm_buffers& B, int p) {
    const int S = P.fmax * P.node_count, sid = B.stencil_id[p], base = B.base_node[p];
    const uint64_t fidx = B.fidx[p];
    bm_v3 r = v3_zero();
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        const int s = slot_of(P, base, fidx, a);
        const float m = B.grid_mass[s];
        if (m > 0.0f) r = v3_add(r, v3_div(v3_mul(ld3(B.remap_v, S, s), stencil_w(B, sid, a)), m));
    }
    return r;
}

// BladeConstraint._iterations (blade_constraint.py:296-324) in one block.
__global__ void __launch_bounds__(1024) k_hold_solve(bm_params P, bm_buffers B) {
    if (B.flags[BM_FLAG_HOLD_NEEDS] == 0) return;
    __shared__ int scan[1024];
    __shared__ float warp_max[32];
    const int N = P.n, S = P.fmax * P.node_count;
    const int m = B.flags[BM_FLAG_HOLD_COUNT], nodes = B.flags[BM_FLAG_HOLD_NODES];
    const int t0 = threadIdx.x;
    // contacts per listed node, in ascending particle order
    const int chunk = (nodes + 1023) / 1024, begin = t0 * chunk, end = min(begin + chunk, nodes);
    int mine = 0;
    for (int t = begin; t < end; ++t) {
        int count = 0;
        for_contributions(P, B, B.hold_nodes[t], [&](int p, int) { count += B.hold_mark[p]; });
        B.hold_node_start[t] = count;
        mine += count;
    }
    int run = block_scan(mine, scan) - mine;
    for (int t = begin; t < end; ++t) {
        const int count = B.hold_node_start[t];
        B.hold_node_start[t] = run;
        run += count;
    }
    if (t0 == 1023) B.hold_node_start[nodes] = run;
    __syncthreads();
    for (int t = t0; t < nodes; t += 1024) {
        int k = B.hold_node_start[t];
        for_contributions(P, B, B.hold_nodes[t], [&](int p, int a) {
            if (B.hold_mark[p]) B.hold_entry[k++] = (p << 3) | a;
        });
    }
    __syncthreads();
    // row_bound (blade_constraint.py:73-90) from the coupled active weights
    scatter_couple(P, B, nodes, kOnes);
    __syncthreads();
    for (int i = t0; i < m; i += 1024) {
        const int p = B.hold_list[i], sid = B.stencil_id[p], base = B.base_node[p];
        const uint64_t fidx = B.fidx[p];
        float total = 0.0f;
        for (int a = 0; a < 8; ++a) {
            const int s = slot_of(P, base, fidx, a);
            const float mass = B.grid_mass[s];
            if (mass > 0.0f) total = total + stencil_w(B, sid, a) * B.remap_v[s] / mass;
        }
        row(B, N, kBound)[p] = total;
    }
    __syncthreads();
    int batches = 0;
    float residual = 0.0f;
    for (;;) {
        for (int i = t0; i < m; i += 1024) {
            const int p = B.hold_list[i];
            row(B, N, kExtrapolated)[p] = row(B, N, kImpulse)[p];
        }
        __syncthreads();
        for (int it = 0; it < 48; ++it) {
            const float acc = (float)((double)it / (double)(it + 3));
            scatter_couple(P, B, nodes, kFromExtrapolated);
            __syncthreads();
            for (int i = t0; i < m; i += 1024) {
                const int p = B.hold_list[i];
                const bm_v3 r = response(P, B, p);
                const float previous = row(B, N, kImpulse)[p];
                const float current =
                    bm_maxf(0.0f, row(B, N, kExtrapolated)[p] +
                                      (row(B, N, kRhs)[p] - v3_dot(ld3(row(B, N, kNormal), N, p), r)) /
                                          bm_maxf(row(B, N, kBound)[p], 1.0e-12f));
                row(B, N, kImpulse)[p] = current;
                row(B, N, kExtrapolated)[p] = current + acc * (current - previous);
            }
            __syncthreads();
        }
        scatter_couple(P, B, nodes, kFromImpulse);
        __syncthreads();
        // record_residual (blade_constraint.py:155-168): the largest inward residual
        float worst = 0.0f;
        for (int i = t0; i < m; i += 1024) {
            const int p = B.hold_list[i];
            worst = bm_maxf(worst, bm_maxf(0.0f, row(B, N, kRhs)[p] - v3_dot(ld3(row(B, N, kNormal), N, p), response(P, B, p))));
        }
        for (int d = 16; d > 0; d >>= 1) worst = fmaxf(worst, __shfl_xor_sync(kAll, worst, d));
        if ((t0 & 31) == 0) warp_max[t0 >> 5] = worst;
        __syncthreads();
        residual = 0.0f;
        for (int w = 0; w < 32; ++w) residual = fmaxf(residual, warp_max[w]);
        __syncthreads();
        batches += 1;
        if (!(residual > 1.0e-6f && batches < 8)) break;
    }
    // apply_reaction (blade_constraint.py:197-205): reaction -= sum j, torque -= sum lever x j
    for (int i0 = 0; i0 < m; i0 += 1024) {
        const int i = i0 + t0;
        bm_v3 j = v3_zero(), tq = v3_zero();
        if (i < m) {
            const int p = B.hold_list[i];
            j = v3_mul(ld3(row(B, N, kNormal), N, p), row(B, N, kImpulse)[p]);
            tq = v3_cross(ld3(row(B, N, kLever), N, p), j);
        }
        if (__any_sync(kAll, i < m)) {
            warp_accumulate(B.acc + BM_ACC_REACTION(0), bm_fx_from_float(-j.x));
            warp_accumulate(B.acc + BM_ACC_REACTION(0) + 2, bm_fx_from_float(-j.y));
            warp_accumulate(B.acc + BM_ACC_REACTION(0) + 4, bm_fx_from_float(-j.z));
            warp_accumulate(B.acc + BM_ACC_TORQUE(0), bm_fx_from_float(-tq.x));
            warp_accumulate(B.acc + BM_ACC_TORQUE(0) + 2, bm_fx_from_float(-tq.y));
            warp_accumulate(B.acc + BM_ACC_TORQUE(0) + 4, bm_fx_from_float(-tq.z));
        }
    }
    if (t0 == 0) {
        const float previous = __int_as_float(B.flags[BM_FLAG_HOLD_RESIDUAL]);
        B.flags[BM_FLAG_HOLD_RESIDUAL] = __float_as_int(bm_maxf(previous, residual));
    }
    (void)S;
}

// apply_grid (blade_constraint.py:187-194): new_v += C / m for every slot with
// mass; C is zero away from the listed nodes.
__global__ void k_hold_apply(bm_params P, bm_buffers B) {
    if (B.flags[BM_FLAG_HOLD_NEEDS] == 0) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.active_nodes) return;
    const int X = B.active[t], nf = B.nfield[X], NC = P.node_count, S = P.fmax * NC;
    const bool listed = B.hold_node_mark[X] != 0;
    for (int f = 0; f < nf; ++f) {
        const int s = f * NC + X;
        const float m = B.grid_mass[s];
        if (m <= 0.0f) continue;
        const bm_v3 c = listed ? ld3(B.remap_v, S, s) : v3_zero();
        st3(B.new_v, S, s, v3_add(ld3(B.new_v, S, s), v3_div(c, m)));
    }
}

// Clears the node marks and the per-substep counters.
__global__ void k_hold_finish(bm_params P, bm_buffers B) {
    const int nodes = min(B.flags[BM_FLAG_HOLD_NODES], P.node_count);
    for (int t = threadIdx.x; t < nodes; t += blockDim.x) B.hold_node_mark[B.hold_nodes[t]] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        B.flags[BM_FLAG_HOLD_NEEDS] = 0;
        B.flags[BM_FLAG_HOLD_NODES] = 0;
    }
}

}  // namespace

void launch_hold(const bm_solver* s, cudaStream_t st) {
    const bm_params& P = s->P;
    const bm_buffers& B = s->B;
    const int32_t* gate = &B.flags[BM_FLAG_HOLD_NEEDS];
    const unsigned wide = 4 * 152;
    const unsigned gn = grid_for(P.n) < wide ? grid_for(P.n) : wide;
    const int tb = spread_block(P.n);
    k_hold_prepare<<<grid_for(P.n, tb), tb, 0, st>>>(P, B);
    launch_exclusive_scan(B.hold_mark, B.hold_pos, P.n, s->scan_partials, &B.flags[BM_FLAG_HOLD_COUNT], scan_ticket(B), gate,
                          st);
    k_hold_list<<<gn, kBlock, 0, st>>>(P, B);
    k_hold_solve<<<1, 1024, 0, st>>>(P, B);
    k_hold_apply<<<grid_for(P.active_nodes), kBlock, 0, st>>>(P, B);
    k_hold_finish<<<1, 1024, 0, st>>>(P, B);
}

}  // namespace bm
