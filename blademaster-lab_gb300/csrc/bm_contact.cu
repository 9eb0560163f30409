// Rigid (gravity, board, knife) and particle-pair contact, cutting damage,
// side labels (blademaster_warp/contact.py).
//
// Reactions, torques, board impulse and cutting work are summed exactly in
// 128-bit fixed point (warp-reduced, one atomic pair per warp), so their
// values do not depend on the order of accumulation.  Pair impulses are
// evaluated from both sides of each pair (the two evaluations are exact
// negations) and each particle adds its own in ascending partner order, so
// no float atomic touches the impulses.  The pair search is a skin list
// rebuilt only when a particle moved half the skin or a cut code changed
// (contact.py:716-822): particles are binned by a counting sort of hashed
// cells, and each particle keeps its sorted partners on both sides.
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {

// contact.friction (contact.py:21-43).
__device__ __forceinline__ void friction(bm_v3 n, bm_v3 relative, float jn, bm_v3 history, float me, float dt,
                                         float mus, float mud, float gk, float gc, bm_v3* impulse, bm_v3* new_history) {
    const bm_v3 vt = v3_sub(relative, v3_mul(n, v3_dot(relative, n)));
    const bm_v3 ht = v3_sub(history, v3_mul(n, v3_dot(history, n)));
    const float k = gk * me / (dt * dt);
    const float damping = 2.0f * gc * sqrtf(me * k);
    const bm_v3 trial = v3_mul(v3_sub(v3_mul(ht, -k), v3_mul(vt, damping)), dt);
    const float magnitude = v3_len(trial);
    if (magnitude <= mus * jn) {
        *impulse = trial;
        *new_history = v3_add(ht, v3_mul(vt, dt));
        return;
    }
    const bm_v3 applied = v3_mul(trial, mud * jn / magnitude);
    *impulse = applied;
    *new_history = v3_div(v3_neg(v3_add(v3_div(applied, dt), v3_mul(vt, damping))), k);
}

// contact.blade_query (contact.py:46-120).
__device__ void blade_query(bm_v3 local, const float* half, float bevel, bm_v3* closest_out, bm_v3* normal_out,
                            float* distance_out) {
    bm_v3 closest = v3(bm_clampf(local.x, -half[0], half[0]), bm_clampf(local.y, -half[1], half[1]),
                       bm_clampf(local.z, -half[2], half[2]));
    bm_v3 delta = v3_sub(local, closest), normal = v3_zero();
    float distance = v3_len(delta);
    if (bevel == 0.0f) {
        if (distance > 1.0e-12f) {
            normal = v3_div(delta, distance);
        } else {
            const bm_v3 margin = v3(half[0] - fabsf(local.x), half[1] - fabsf(local.y), half[2] - fabsf(local.z));
            int axis = 0;
            if (margin.y < v3_get(margin, axis)) axis = 1;
            if (margin.z < v3_get(margin, axis)) axis = 2;
            v3_set(&normal, axis, 1.0f);
            if (v3_get(local, axis) < 0.0f) v3_set(&normal, axis, -1.0f);
            v3_set(&closest, axis, v3_get(normal, axis) * half[axis]);
            distance = -v3_get(margin, axis);
        }
    } else {
        const float qx = fabsf(local.x), qy = local.z;
        const float sign = local.x < 0.0f ? -1.0f : 1.0f;
        const float ex = half[0], ey = bevel;
        const float len_sq = ex * ex + ey * ey;
        const float t = bm_clampf((qx * ex + (qy + half[2]) * ey) / len_sq, 0.0f, 1.0f);
        float nx = t * half[0], ny = -half[2] + t * bevel;
        float best_sq = (qx - nx) * (qx - nx) + (qy - ny) * (qy - ny);
        float ox = bevel / sqrtf(len_sq), oy = -half[0] / sqrtf(len_sq);
        float cx = half[0], cy = bm_clampf(qy, -half[2] + bevel, half[2]);
        float dsq = (qx - cx) * (qx - cx) + (qy - cy) * (qy - cy);
        if (dsq < best_sq) {
            best_sq = dsq;
            nx = cx;
            ny = cy;
            ox = 1.0f;
            oy = 0.0f;
        }
        cx = bm_clampf(qx, 0.0f, half[0]);
        cy = half[2];
        dsq = (qx - cx) * (qx - cx) + (qy - cy) * (qy - cy);
        if (dsq < best_sq) {
            best_sq = dsq;
            nx = cx;
            ny = cy;
            ox = 0.0f;
            oy = 1.0f;
        }
        const bool inside = qx <= half[0] && qy <= half[2] && half[0] * (qy + half[2]) >= bevel * qx;
        const float best = sqrtf(best_sq);
        nx = sign * nx;
        ox = sign * ox;
        closest = v3(nx, bm_clampf(local.y, -half[1], half[1]), ny);
        if (inside && fabsf(local.y) <= half[1]) {
            normal = v3(ox, 0.0f, oy);
            distance = -best;
            if (half[1] - fabsf(local.y) < best) {
                const float s2 = local.y < 0.0f ? -1.0f : 1.0f;
                closest = local;
                closest.y = s2 * half[1];
                normal = v3(0.0f, s2, 0.0f);
                distance = -(half[1] - fabsf(local.y));
            }
        } else {
            if (inside) {
                closest.x = local.x;
                closest.z = local.z;
            }
            delta = v3_sub(local, closest);
            distance = v3_len(delta);
            normal = v3(ox, 0.0f, oy);
            if (distance > 1.0e-12f) normal = v3_div(delta, distance);
        }
    }
    *closest_out = closest;
    *normal_out = normal;
    *distance_out = distance;
}

// contact.penalty_impulse (contact.py:123-147).
__device__ __forceinline__ void penalty_impulse(float gap, bm_v3 relative, bm_v3 n, float me, bm_v3 history, float dt,
                                                float sn, float mus, float mud, float gk, float gc, bm_v3* impulse,
                                                bm_v3* new_history) {
    const float predicted = gap + dt * bm_minf(v3_dot(relative, n), 0.0f);
    if (predicted >= 0.0f) {
        *impulse = v3_zero();
        *new_history = v3_zero();
        return;
    }
    const float jn = sn * me / dt * (-predicted);
    bm_v3 jt, ht;
    friction(n, relative, jn, history, me, dt, mus, mud, gk, gc, &jt, &ht);
    *impulse = v3_add(v3_mul(n, jn), jt);
    *new_history = ht;
}

// contact.blade_effective_mass (contact.py:150-178).
__device__ __forceinline__ float blade_effective_mass(const bm_params& P, const float* __restrict__ mobility,
                                                      bm_v3 lever, bm_v3 n, bm_q q) {
    float inverse = 1.0f / P.blade_mass;
    if (P.tool_model < 0) {
        const bm_v3 rn = v3_cross(lever, n);
        const float u[6] = {n.x, n.y, n.z, rn.x, rn.y, rn.z};
        inverse = 0.0f;
#pragma unroll
        for (int row = 0; row < 6; ++row)
#pragma unroll
            for (int col = 0; col < 6; ++col) inverse = inverse + u[row] * mobility[6 * row + col] * u[col];
    } else if (P.tool_model > 0) {
        const bm_v3 rn = q_rotate_inv(q, v3_cross(lever, n));
        inverse = inverse + v3_dot(rn, v3_cw(v3(P.inertia_inv[0], P.inertia_inv[1], P.inertia_inv[2]), rn));
    }
    return 1.0f / (1.0f / P.mass + inverse);
}

// contact.resist_cut (contact.py:181-232); work added to *work.
__device__ __forceinline__ bm_v3 resist_cut(bm_v3 j, bm_v3 xp, bm_v3 vp, bm_v3 origin, bm_v3 tool_velocity, bm_q q,
                                            bm_v3 tool_angular, const float* half, float radius, float spacing,
                                            float* damage, float threshold, int cutting, bm_fx* work) {
    const bm_v3 edge = v3_add(origin, q_rotate(q, v3(0.0f, 0.0f, -half[2])));
    const bm_v3 down = q_rotate(q, v3(0.0f, 0.0f, -1.0f));
    const bm_v3 edge_velocity = v3_add(tool_velocity, v3_cross(tool_angular, v3_sub(edge, origin)));
    const float front = v3_dot(v3_sub(xp, edge), down);
    float advance = v3_dot(v3_sub(edge_velocity, vp), down);
    if ((cutting & BM_CUT_ADVANCE) != 0) advance = v3_dot(edge_velocity, down);
    const bm_v3 local_edge = q_rotate_inv(q, v3_sub(xp, edge));
    const bool ahead = front >= 0.0f && front <= 2.0f * radius && fabsf(local_edge.x) <= 6.0f * spacing &&
                       fabsf(local_edge.y) <= half[1];
    if (!ahead) return j;
    const float push = bm_maxf(v3_dot(j, down), 0.0f);
    if (*damage >= 1.0f) return v3_sub(j, v3_mul(down, push));
    if (advance > 0.0f) {
        const float delta = push * advance;
        *work = bm_fx_add(*work, bm_fx_from_float(delta));
        *damage = bm_minf(1.0f, *damage + delta / threshold);
    }
    return j;
}

// contact.blade_at (contact.py:235-329) for knife k: returns the impulse on
// the particle and sets the reaction / torque contributions (zero if none).
// Two exact shortcuts keep far particles cheap without changing any result:
// a particle outside the knife's box grown by the contact reach gets the
// reference's "no contact" outcome directly, and bit 1 + k of `mask` says
// whether its stored knife history may be non-zero (a zero history is
// neither read nor rewritten).
__device__ bm_v3 blade_at(const bm_params& P, const bm_buffers& B, int p, int k, const ToolF& T, int cutting,
                          bm_v3 xp, bm_v3 vp, float vlen, float radius_of_blade, unsigned* mask, bm_v3* reaction,
                          bm_v3* torque, bm_fx* work) {
    const int64_t N = P.n;
    float* hist = B.histories + (int64_t)(1 + k) * 3 * N;
    const unsigned bit = 1u << (1 + k);
    *reaction = v3_zero();
    *torque = v3_zero();
    const float max_closing = (vlen + T.speed) + T.spin_reach;
    const bm_v3 d = v3_sub(xp, T.pos);
    bool far = v3_len(d) - radius_of_blade - P.blade_offset > P.dt * max_closing;
    bm_v3 local = v3_zero();
    if (!far) {
        // Contact needs every |local_i| <= half_i + offset + dt * max_closing;
        // the margin is widened to cover rounding of the exact test below, and
        // the axis projections (a cheaper route to local) get 10 ppm more.
        const float margin = (P.blade_offset + P.dt * max_closing) * 1.01f + 1.0e-6f;
        const float axis_margin = margin + 1.0e-5f * radius_of_blade;
        far = fabsf(v3_dot(d, T.ax)) - P.half[0] > axis_margin || fabsf(v3_dot(d, T.ay)) - P.half[1] > axis_margin ||
              fabsf(v3_dot(d, T.az)) - P.half[2] > axis_margin;
        if (!far) {
            local = q_rotate_inv(T.rot, d);
            far = fabsf(local.x) - P.half[0] > margin || fabsf(local.y) - P.half[1] > margin ||
                  fabsf(local.z) - P.half[2] > margin;
        }
    }
    if (far) {
        if (*mask & bit) {
            st3(hist, N, p, v3_zero());
            *mask &= ~bit;
        }
        return v3_zero();
    }
    float* damage = B.damage + (int64_t)k * N + p;
    bm_v3 closest_local, normal_local;
    float distance;
    blade_query(local, P.half, P.bevel, &closest_local, &normal_local, &distance);
    const float front = -P.half[2] - local.z;
    if ((cutting & BM_CUT_HOLD) != 0 && *damage < 1.0f && fabsf(local.x) <= P.half[0] + P.blade_offset &&
        fabsf(local.y) <= P.half[1] && front >= 0.0f) {
        closest_local = v3(local.x, local.y, -P.half[2]);
        normal_local = v3(0.0f, 0.0f, -1.0f);
        distance = front;
    }
    const bm_v3 lever = q_rotate(T.rot, closest_local);
    const bm_v3 n = q_rotate(T.rot, normal_local);
    const bm_v3 relative = v3_sub(v3_sub(vp, T.vel), v3_cross(T.omega, lever));
    if (distance - P.blade_offset + P.dt * bm_minf(v3_dot(relative, n), 0.0f) >= 0.0f) {
        if (*mask & bit) {
            st3(hist, N, p, v3_zero());
            *mask &= ~bit;
        }
        return v3_zero();
    }
    const float me = blade_effective_mass(P, B.mobility, lever, n, T.rot);
    const bm_v3 h_old = (*mask & bit) ? ld3(hist, N, p) : v3_zero();
    bm_v3 j, h;
    penalty_impulse(distance - P.blade_offset, relative, n, me, h_old, P.dt, P.normal_scale, P.friction_static,
                    P.friction_dynamic, P.tangent_stiffness, P.tangent_damping, &j, &h);
    st3(hist, N, p, h);
    *mask |= bit;
    if (v3_len_sq(j) > 0.0f) {
        if (cutting != 0)
            j = resist_cut(j, xp, vp, T.pos, T.vel, T.rot, T.omega, P.half, P.blade_offset, P.spacing, damage,
                           P.threshold, cutting, work);
        *reaction = v3_neg(j);
        *torque = v3_neg(v3_cross(lever, j));
        return j;
    }
    return v3_zero();
}

__device__ __forceinline__ void warp_accumulate3(uint64_t* acc, bm_v3 v, bool any) {
    if (!__any_sync(0xffffffffu, any)) return;
    warp_accumulate(acc, bm_fx_from_float(v.x));
    warp_accumulate(acc + 2, bm_fx_from_float(v.y));
    warp_accumulate(acc + 4, bm_fx_from_float(v.z));
}

// Knives that may be in contact with some particle of this warp (the same
// mask in every lane).  A knife is left out when, on one of its axes, the
// warp's bounding box lies farther from it than blade_at's per-particle axis
// pre-test allows at the warp's largest particle speed, plus 1 um for
// rounding: every particle of the warp then takes blade_at's "far" outcome.
// Lane 0 also raises the substep's maximum particle speed
// (rigid_and_speed's atomic_max, contact.py:497).
__device__ unsigned rigid_knives(const bm_params& P, const bm_buffers& B, bm_v3 x, float speed, bool active,
                                 float radius_of_blade) {
    bm_v3 c, e;
    float vmax;
    bool any;
    warp_box(x, speed, active, &c, &e, &vmax, &any);
    if (!any) return 0u;
    const int k = threadIdx.x & 31;
    if (k == 0) atomic_max_nonneg(B.speed, vmax);
    bool near = false;
    if (k < P.tool_count) {
        const ToolF T = load_tool(B.tool_f + BM_TOOL_F_WORDS * k);
        const float max_closing = (vmax + T.speed) + T.spin_reach;
        const float margin = (P.blade_offset + P.dt * max_closing) * 1.01f + 1.0e-6f;
        const float axis_margin = margin + 1.0e-5f * radius_of_blade + 1.0e-6f;
        const bm_v3 d = v3_sub(c, T.pos);
        near = !(fabsf(v3_dot(d, T.ax)) - box_reach(T.ax, e) - P.half[0] > axis_margin ||
                 fabsf(v3_dot(d, T.ay)) - box_reach(T.ay, e) - P.half[1] > axis_margin ||
                 fabsf(v3_dot(d, T.az)) - box_reach(T.az, e) - P.half[2] > axis_margin);
    }
    return __ballot_sync(0xffffffffu, near);
}

// contact.rigid_and_speed + extra_blade (contact.py:422-566) for every knife.
__global__ void __launch_bounds__(256, 4) k_rigid(bm_params P, bm_buffers B, int cutting) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = p < P.n;
    const int64_t N = P.n;
    bm_fx work = fx_zero();
    float speed = 0.0f;
    bm_v3 total = v3_zero(), jb = v3_zero(), xp = v3_zero(), vp = v3_zero();
    bool board_hit = false;
    unsigned mask = 0u, mask_in = 0u;
    const float radius_of_blade = blade_radius(P);
    if (active) {
        xp = ld3(B.x, N, p);
        vp = ld3(B.v, N, p);
        mask = mask_in = B.hist_mask[p];
        speed = v3_len(vp);
        total = v3(0.0f, 0.0f, -9.81f * P.mass * P.dt);
        float board_gap = xp.z - P.radius;
        if (P.board_half[0] > 0.0f && fabsf(xp.x) > P.board_half[0]) board_gap = 1.0e30f;
        if (P.board_half[1] > 0.0f && fabsf(xp.y) > P.board_half[1]) board_gap = 1.0e30f;
        bm_v3 hb;
        const bm_v3 h_old = (mask & 1u) ? ld3(B.histories, N, p) : v3_zero();
        penalty_impulse(board_gap, vp, v3(0.0f, 0.0f, 1.0f), P.mass, h_old, P.dt, P.board_scale, P.friction_static,
                        P.friction_dynamic, P.tangent_stiffness, P.tangent_damping, &jb, &hb);
        const bool nonzero = hb.x != 0.0f || hb.y != 0.0f || hb.z != 0.0f;
        if (nonzero || (mask & 1u)) st3(B.histories, N, p, hb);
        mask = nonzero ? (mask | 1u) : (mask & ~1u);
        if (v3_len_sq(jb) > 0.0f) {
            total = v3_add(total, jb);
            board_hit = true;
        }
    }
    warp_accumulate3(B.acc + BM_ACC_BOARD, jb, board_hit);
    const unsigned knives = rigid_knives(P, B, xp, speed, active, radius_of_blade);
    for (int k = 0; k < P.tool_count; ++k) {
        if (((knives >> k) & 1u) == 0u) {
            // no particle of the block is near knife k: blade_at's far outcome
            const unsigned bit = 1u << (1 + k);
            if (active && (mask & bit)) {
                st3(B.histories + (int64_t)(1 + k) * 3 * N, N, p, v3_zero());
                mask &= ~bit;
            }
            continue;
        }
        bm_v3 reaction = v3_zero(), torque = v3_zero();
        if (active) {
            const ToolF T = load_tool(B.tool_f + BM_TOOL_F_WORDS * k);
            total = v3_add(total, blade_at(P, B, p, k, T, cutting, xp, vp, speed, radius_of_blade, &mask, &reaction,
                                           &torque, &work));
        }
        const bool hit = v3_len_sq(reaction) > 0.0f || v3_len_sq(torque) > 0.0f;
        warp_accumulate3(B.acc + BM_ACC_REACTION(k), reaction, hit);
        warp_accumulate3(B.acc + BM_ACC_TORQUE(k), torque, hit);
    }
    if (__any_sync(0xffffffffu, work.lo != 0u || work.hi != 0u)) warp_accumulate(B.acc + BM_ACC_WORK, work);
    if (active) {
        st3(B.impulses, N, p, total);
        if (mask != mask_in) B.hist_mask[p] = (uint16_t)mask;
    }
}

// ------------------------------------------------------------ pair contact

__device__ __forceinline__ int64_t hash_slot(int64_t key, int64_t capacity) {
    return (int64_t)(((uint64_t)key * (uint64_t)2654435761u) % (uint64_t)capacity);
}
// material.insert_key (material.py:37-47).
__device__ int64_t insert_key(int64_t* keys, int64_t key, int64_t capacity) {
    int64_t slot = hash_slot(key, capacity);
    for (int64_t probe = 0; probe < capacity; ++probe) {
        const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(&keys[slot]),
                                                  (unsigned long long)(-1ll), (unsigned long long)key);
        if ((long long)prev == -1ll || (long long)prev == key) return slot;
        slot = (slot + 1) % capacity;
    }
    return -1;
}
// contact.find_key (contact.py:569-580).
__device__ int64_t find_key(const int64_t* keys, int64_t key, int64_t capacity) {
    int64_t slot = hash_slot(key, capacity);
    for (int64_t probe = 0; probe < capacity; ++probe) {
        const int64_t k = keys[slot];
        if (k == -1) return -1;
        if (k == key) return slot;
        slot = (slot + 1) % capacity;
    }
    return -1;
}

// contact.pair_at (contact.py:583-640) from the side of p; returns whether the
// pair is in contact and the impulse on p.  The owner (p < q) records the new
// friction history and counts coincident pairs.
__device__ bool pair_impulse(const bm_params& P, const bm_buffers& B, int p, int q, int old, int nw, bm_v3* out) {
    const int64_t N = P.n;
    const bm_v3 delta = v3_sub(ld3(B.x, N, p), ld3(B.x, N, q));
    const float dist = v3_len(delta);
    if (dist >= 2.0f * P.radius + P.dt * v3_len(v3_sub(ld3(B.v, N, p), ld3(B.v, N, q)))) return false;
    if (compatible_codes(B.codes[p], B.codes[q]) &&
        v3_len(v3_sub(ld3(B.ref, N, p), ld3(B.ref, N, q))) < 2.0f * P.spacing)
        return false;
    const bool owner = p < q;
    if (dist < 1.0e-12f) {
        if (owner) atomicAdd(&B.errors[2], 1);
        return false;
    }
    const bm_v3 normal = v3_div(delta, dist);
    const bm_v3 relative = v3_sub(ld3(B.v, N, p), ld3(B.v, N, q));
    const float predicted = 2.0f * P.radius - dist - P.dt * bm_minf(v3_dot(relative, normal), 0.0f);
    if (predicted <= 0.0f) return false;
    const int64_t lo = owner ? p : q, hi = owner ? q : p;
    const int64_t key = lo * N + hi;
    const int64_t cap = P.pair_capacity;
    const int64_t oslot = find_key(B.pair_keys + (int64_t)old * cap, key, cap);
    bm_v3 history = v3_zero();
    if (oslot >= 0) {
        const float* h = B.pair_history + 3 * ((int64_t)old * cap + oslot);
        history = v3(h[0], h[1], h[2]);
    }
    if (!owner) history = v3_neg(history);
    int64_t nslot = -1;
    if (owner) {
        nslot = insert_key(B.pair_keys + (int64_t)nw * cap, key, cap);
        if (nslot < 0) {
            atomicAdd(&B.errors[0], 1);
            return false;
        }
    }
    const float half_mass = P.mass / 2.0f;
    const float jn = P.normal_scale * half_mass / P.dt * predicted;
    bm_v3 jt, ht;
    friction(normal, relative, jn, history, half_mass, P.dt, P.friction_static, P.friction_dynamic,
             P.tangent_stiffness, P.tangent_damping, &jt, &ht);
    if (owner) {
        float* h = B.pair_history + 3 * ((int64_t)nw * cap + nslot);
        h[0] = ht.x;
        h[1] = ht.y;
        h[2] = ht.z;
        const int at = atomicAdd(&B.pair_count[nw], 1);
        if (at < cap) B.pair_used[(int64_t)nw * cap + at] = (int32_t)nslot;
    }
    *out = v3_add(v3_mul(normal, jn), jt);
    return true;
}

__device__ __forceinline__ int cell_coord(float x, float size) { return (int)floorf(x / size); }
// Cell coordinates packed 21 bits each (cells more than 2^20 apart may alias,
// which only adds candidates that the distance test rejects).
__device__ __forceinline__ int64_t cell_key(int cx, int cy, int cz) {
    return (int64_t)((((uint64_t)cx & 0x1FFFFFu) << 42) | (((uint64_t)cy & 0x1FFFFFu) << 21) | ((uint64_t)cz & 0x1FFFFFu));
}
// contact.list_bucket (contact.py:743-745).
__device__ __forceinline__ int list_bucket(int cx, int cy, int cz, int mask) {
    return (int)((((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u)) &
                 (uint32_t)mask);
}

// Solver prologue of a substep: clear_pair_slots (contact.py:643-652) of the
// table written this substep, and clear_step (contact.py:1058-1068).  It
// also opens the substep's gated work, whose flags are final by now: the
// largest-displacement bound of a full pair-list build (reset when the list
// is rebuilt this substep), and with registration >= 0 the counters of a
// topology registration (when the topology is dirty, or always with
// registration == 1), which the registration kernels then fill.
__global__ void k_prologue(bm_params P, bm_buffers B, int clear_step, int registration) {
    const int step = B.flags[BM_FLAG_STEP];
    const int nw = (step + 1) & 1;
    const int64_t cap = P.pair_capacity;
    const int count = min(B.pair_count[nw], P.pair_capacity);
    for (int i = threadIdx.x; i < count; i += blockDim.x) B.pair_keys[(int64_t)nw * cap + B.pair_used[(int64_t)nw * cap + i]] = -1;
    if (clear_step) {
        for (int i = threadIdx.x; i < BM_ACC_WORK; i += blockDim.x) {
            // reaction and torque of every knife, and the board (not the cumulative work)
            const bool reaction = i < 2 * 3 * P.tool_count;
            const bool torque = i >= BM_ACC_TORQUE(0) && i < BM_ACC_TORQUE(0) + 2 * 3 * P.tool_count;
            const bool board = i >= BM_ACC_BOARD && i < BM_ACC_BOARD + 6;
            if (reaction || torque || board) B.acc[i] = 0u;
        }
        if (threadIdx.x == 0) B.speed[0] = 0.0f;
    }
    if (threadIdx.x == 0) {
        if (P.pair_search != 0 || B.flags[BM_FLAG_PAIR_DIRTY] != 0) {
            B.flags[BM_FLAG_MAX_DISP] = 0;  // +0.0f
            B.flags[BM_FLAG_PAIR_SPEED] = 0;
        }
        if (registration >= 0) begin_registration(B, registration);
    }
    __syncthreads();
    if (threadIdx.x == 0) B.pair_count[nw] = 0;
}

// First kernel of a full pair-list build.  Block 0 resets the build's
// counters; every block zeroes bucket counts and raises, over all particles,
// the largest displacement |x - ref| (the build's reference-distance bound,
// see build_list; k_prologue reset it).  The reach uses the substep's largest
// particle speed (rigid_and_speed's maximum, contact.py:497): inside a
// substep (find_speed) it is found here from the same velocities the contact
// pass reads, so that the build need not wait for that pass; a pair pass
// called on its own takes the stored maximum (buffers.speed), as the
// reference's particle_contacts does.
__global__ void k_pair_begin(bm_params P, bm_buffers B, int64_t buckets, const int32_t* gate_flag, int find_speed) {
    if (gate_flag && *gate_flag == 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.flags[BM_FLAG_CANDIDATES] = 0;
        B.flags[BM_FLAG_PAIR_BUILDS] += 1;
        B.flags[BM_FLAG_CHANGED] = 0;  // a full build uses the current codes
        if (!find_speed) B.flags[BM_FLAG_PAIR_SPEED] = __float_as_int(B.speed[0]);
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < buckets; i += stride) B.bucket_fill[i] = 0;
    const int N = P.n;
    float d = 0.0f;
    const float inf = __int_as_float(0x7f800000);
    // the speed maximum as the contact pass forms it (a NaN speed wins there
    // too): warp maxima, combined by integer maximum of their bit patterns,
    // here over the warp's grid-stride iterations first and then by one
    // atomic per warp (the same value as one atomic per iteration)
    int speed_bits = 0;
    bool speed_any = false;
    for (int p0 = blockIdx.x * blockDim.x; p0 < N; p0 += gridDim.x * blockDim.x) {
        const int p = p0 + threadIdx.x;
        const bool active = p < N;
        float speed = -inf;
        if (active) {
            d = fmaxf(d, v3_len(v3_sub(ld3(B.x, N, p), ld3(B.ref, N, p))));
            if (find_speed) speed = v3_len(ld3(B.v, N, p));
        }
        if (find_speed) {  // block-uniform; every lane takes part in both warp collectives
            const float vmax = warp_max(speed);
            if (__any_sync(0xffffffffu, active)) {
                speed_bits = max(speed_bits, __float_as_int(vmax));
                speed_any = true;
            }
        }
    }
    if ((threadIdx.x & 31) == 0 && speed_any) atomicMax(&B.flags[BM_FLAG_PAIR_SPEED], speed_bits);
    for (int s = 16; s > 0; s >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, s));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(reinterpret_cast<float*>(&B.flags[BM_FLAG_MAX_DISP]), d);
}

// contact.set_pair_reach (contact.py:748-761) for the list search, or the hash
// search reach 2 radius + 2 dt speed (contact.py:684), from the speed
// k_pair_begin found.  Every thread evaluates it; block 0 stores it for the
// build's later kernels and the relists.
__device__ __forceinline__ float pair_reach(const bm_params& P, float speed) {
    if (P.pair_search == 0) {
        float value = 2.0f * P.radius + P.pair_skin;
        if (P.dt * speed > 0.5f * P.pair_skin) value += 2.0f * P.dt * speed;
        return value;
    }
    return 2.0f * P.radius + 2.0f * speed * P.dt;
}

__global__ void k_bin_count(bm_params P, bm_buffers B, float* reach_out, const int32_t* gate_flag) {
    if (gate_flag && *gate_flag == 0) return;
    const int64_t N = P.n;
    const float reach = pair_reach(P, __int_as_float(B.flags[BM_FLAG_PAIR_SPEED]));
    if (blockIdx.x == 0 && threadIdx.x == 0) *reach_out = reach;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) {
        const bm_v3 x = ld3(B.x, N, p);
        const int cx = cell_coord(x.x, reach), cy = cell_coord(x.y, reach), cz = cell_coord(x.z, reach);
        const int b = list_bucket(cx, cy, cz, P.bucket_mask);
        B.particle_bucket[p] = b;
        B.particle_key[p] = cell_key(cx, cy, cz);
        atomicAdd(&B.bucket_fill[b], 1);
    }
}

// Block-wide inclusive scan of one value per thread (blockDim.x == 1024).
__device__ __forceinline__ int32_t block_scan_1024(int32_t v, int32_t* s) {
    const int t = threadIdx.x;
    s[t] = v;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const int32_t add = t >= d ? s[t - d] : 0;
        __syncthreads();
        s[t] += add;
        __syncthreads();
    }
    const int32_t r = s[t];
    __syncthreads();
    return r;
}

// Exclusive scan of the tile sums (one block of 1024 threads); the total of
// all tiles goes to *total_out.  The sums are read through L2: other blocks
// of the same kernel wrote them.
__device__ void scan_partials_block(int32_t* partials, int64_t tiles, int32_t* total_out) {
    __shared__ int32_t s[1024];
    const int64_t chunk = (tiles + 1023) / 1024;
    const int64_t begin = threadIdx.x * chunk, end = min(begin + chunk, tiles);
    int32_t sum = 0;
    for (int64_t i = begin; i < end; ++i) sum += __ldcg(partials + i);
    const int32_t inc = block_scan_1024(sum, s);
    int32_t run = inc - sum;
    for (int64_t i = begin; i < end; ++i) {
        const int32_t v = __ldcg(partials + i);
        partials[i] = run;
        run += v;
    }
    if (threadIdx.x == 1023 && total_out) *total_out = inc;
}

// Exclusive scan of `count` ints: tiles of 1024 (grid-stride over tiles),
// then the block that finishes last (a ticket counter; no block waits)
// scans the tile sums and resets the ticket; k_scan_add adds the tile
// offsets.
__global__ void k_scan_tiles(const int32_t* in, int32_t* out, int64_t count, int32_t* partials, int32_t* total_out,
                             int32_t* ticket, const int32_t* gate_flag) {
    if (gate_flag && *gate_flag == 0) return;
    __shared__ int32_t s[1024];
    __shared__ int last;
    const int64_t tiles = (count + 1023) / 1024;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t i = tile * 1024 + threadIdx.x;
        const int32_t v = i < count ? in[i] : 0;
        const int32_t inc = block_scan_1024(v, s);
        if (i < count) out[i] = inc - v;
        if (threadIdx.x == 1023) partials[tile] = inc;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    scan_partials_block(partials, tiles, total_out);
    if (threadIdx.x == 0) *ticket = 0;
}
__global__ void k_scan_add(int32_t* out, int64_t count, const int32_t* partials, const int32_t* gate_flag) {
    if (gate_flag && *gate_flag == 0) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        out[i] += partials[i / 1024];
}

__global__ void k_bin_scatter(bm_params P, bm_buffers B, const int32_t* gate_flag) {
    if (gate_flag && *gate_flag == 0) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x) {
        const int b = B.particle_bucket[p];
        const int at = B.bucket_start[b] + atomicSub(&B.bucket_fill[b], 1) - 1;
        B.bucket_items[at] = p;
        B.bucket_key[at] = B.particle_key[p];
        const bm_v3 x = ld3(B.x, P.n, p);
        reinterpret_cast<float4*>(B.bucket_pos)[at] = make_float4(x.x, x.y, x.z, 0.0f);
    }
}

__device__ void build_list(const bm_params& P, const bm_buffers& B, int p, float reach, const float* __restrict__ pos);
__device__ void pair_particle(const bm_params& P, const bm_buffers& B, int p, float reach);

// contact.build_pair_list (contact.py:778-822): partners on both sides within
// the reach that pair_at does not skip as compatible neighbours, ascending.
__global__ void k_build_lists(bm_params P, bm_buffers B, const float* reach_in, const int32_t* gate_flag) {
    if (gate_flag && *gate_flag == 0) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n; p += gridDim.x * blockDim.x)
        build_list(P, B, p, *reach_in, B.x);
}

__device__ void build_list(const bm_params& P, const bm_buffers& B, int p, float reach, const float* __restrict__ pos) {
    const int N = P.n;
    const bm_v3 xp = ld3(pos, N, p), rp = ld3(B.ref, N, p);
    const int64_t cp = B.codes[p];
    if (pos == B.x) st3(B.built_x, N, p, xp);
    B.built_codes[p] = cp;
    // A particle without cut digits is compatible with every code, so its only
    // possible partners are particles farther than 2 h from it in the
    // reference configuration.  Any particle q within the reach has
    // |ref_p - ref_q| <= |x_p - ref_p| + reach + |x_q - ref_q|, and the last
    // term is at most the build's largest displacement: when that sum stays
    // below 2 h (less 0.1 % for rounding) the list is empty without a search.
    if (cp == 0) {
        const float largest = __int_as_float(B.flags[BM_FLAG_MAX_DISP]);
        if ((v3_len(v3_sub(xp, rp)) + largest) + reach < 0.999f * (2.0f * P.spacing)) {
            B.partner_count[p] = 0;
            if (pos == B.x) B.listed[p] = 0;
            return;
        }
    }
    const int hx = cell_coord(xp.x, reach), hy = cell_coord(xp.y, reach), hz = cell_coord(xp.z, reach);
    int32_t* list = B.partners + (int64_t)p * BM_PAIR_LANES;
    const float4* bpos = reinterpret_cast<const float4*>(B.bucket_pos);
    int count = 0;
    for (int i = 0; i < 27; ++i) {
        const int cx = hx + i % 3 - 1, cy = hy + (i / 3) % 3 - 1, cz = hz + i / 9 - 1;
        const int b = list_bucket(cx, cy, cz, P.bucket_mask);
        const int64_t key = cell_key(cx, cy, cz);
        const int begin = B.bucket_start[b], end = B.bucket_start[b + 1];
        for (int it = begin; it < end; ++it) {
            if (B.bucket_key[it] != key) continue;
            const int q = B.bucket_items[it];
            if (q == p) continue;
            const float4 xq4 = bpos[it];
            const bm_v3 xq = v3(xq4.x, xq4.y, xq4.z);
            if (!(v3_len(v3_sub(xq, xp)) < reach)) continue;
            if (v3_len(v3_sub(rp, ld3(B.ref, N, q))) < 2.0f * P.spacing && compatible_codes(cp, B.codes[q])) continue;
            if (count < 0) continue;
            if (count == BM_PAIR_LANES) {
                count = -1;
                continue;
            }
            int j = count++;
            while (j > 0 && list[j - 1] > q) {
                list[j] = list[j - 1];
                --j;
            }
            list[j] = q;
        }
    }
    B.partner_count[p] = count;
    if (pos == B.x) B.listed[p] = 0;
    if (count != 0 && B.listed[p] == 0) {
        B.listed[p] = 1;
        const int at = atomicAdd(&B.flags[BM_FLAG_CANDIDATES], 1);
        if (at < P.candidate_capacity) B.candidates[at] = p;
    }
}

// build_list for particle p by one warp: lane i < 27 scans neighbour cell i
// of the build grid and adds the partners it finds to `found` (this warp's
// shared-memory list); the list overflows past BM_PAIR_LANES partners as in
// build_list, otherwise each lane ranks its entries into ascending order.
// The result equals build_list's; a relist touches few particles, so the
// 27 bucket walks run side by side instead of one after another.
__device__ void build_list_warp(const bm_params& P, const bm_buffers& B, int p, float reach, int32_t* found,
                                int* found_count) {
    const int N = P.n, lane = threadIdx.x & 31;
    const bm_v3 xp = ld3(B.built_x, N, p), rp = ld3(B.ref, N, p);
    const int64_t cp = B.codes[p];
    if (lane == 0) B.built_codes[p] = cp;
    if (cp == 0) {
        const float largest = __int_as_float(B.flags[BM_FLAG_MAX_DISP]);
        if ((v3_len(v3_sub(xp, rp)) + largest) + reach < 0.999f * (2.0f * P.spacing)) {
            if (lane == 0) B.partner_count[p] = 0;
            return;
        }
    }
    if (lane == 0) *found_count = 0;
    __syncwarp();
    if (lane < 27) {
        const int hx = cell_coord(xp.x, reach), hy = cell_coord(xp.y, reach), hz = cell_coord(xp.z, reach);
        const int cx = hx + lane % 3 - 1, cy = hy + (lane / 3) % 3 - 1, cz = hz + lane / 9 - 1;
        const int b = list_bucket(cx, cy, cz, P.bucket_mask);
        const int64_t key = cell_key(cx, cy, cz);
        const float4* bpos = reinterpret_cast<const float4*>(B.bucket_pos);
        const int begin = B.bucket_start[b], end = B.bucket_start[b + 1];
        for (int it = begin; it < end; ++it) {
            if (B.bucket_key[it] != key) continue;
            const int q = B.bucket_items[it];
            if (q == p) continue;
            const float4 xq4 = bpos[it];
            if (!(v3_len(v3_sub(v3(xq4.x, xq4.y, xq4.z), xp)) < reach)) continue;
            if (v3_len(v3_sub(rp, ld3(B.ref, N, q))) < 2.0f * P.spacing && compatible_codes(cp, B.codes[q])) continue;
            const int at = atomicAdd(found_count, 1);
            if (at < BM_PAIR_LANES) found[at] = q;
        }
    }
    __syncwarp();
    const int total = *found_count;
    int count = total > BM_PAIR_LANES ? -1 : total;
    if (count > 0) {
        int32_t* list = B.partners + (int64_t)p * BM_PAIR_LANES;
        for (int j = lane; j < count; j += 32) {
            const int q = found[j];
            int rank = 0;
            for (int k = 0; k < count; ++k) rank += found[k] < q;
            list[rank] = q;
        }
    }
    if (lane == 0) {
        B.partner_count[p] = count;
        if (count != 0 && B.listed[p] == 0) {
            B.listed[p] = 1;
            const int at = atomicAdd(&B.flags[BM_FLAG_CANDIDATES], 1);
            if (at < P.candidate_capacity) B.candidates[at] = p;
        }
    }
    __syncwarp();  // `found` is reused by this warp's next particle
}

// Cut codes changed since the last list update: mark each changed particle
// and every particle within the build reach of it (build positions and
// buckets), so their lists are recomputed with the new codes.  Codes only
// gain digits, so compatibility only turns false and lists only grow; the
// positions are still within half a skin of the build (else a full build ran).
// One warp per changed particle, lane i < 27 walking neighbour cell i.
__global__ void k_relist_mark(bm_params P, bm_buffers B, const float* reach_in, int clear_dirty) {
    const int changed = min(B.flags[BM_FLAG_CHANGED], P.n);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (clear_dirty) B.flags[BM_FLAG_PAIR_DIRTY] = 0;  // any full build ran before this kernel
        if (changed != 0) B.flags[BM_FLAG_RELISTS] += 1;
    }
    if (changed == 0) return;
    const int N = P.n, lane = threadIdx.x & 31;
    const float reach = *reach_in;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < changed; t += warps) {
        const int p = B.changed[t];
        const bm_v3 xp = ld3(B.built_x, N, p);
        if (lane == 0 && atomicExch(&B.relist[p], 1) == 0) B.relist_list[atomicAdd(&B.flags[BM_FLAG_RELIST], 1)] = p;
        if (lane < 27) {
            const int hx = cell_coord(xp.x, reach), hy = cell_coord(xp.y, reach), hz = cell_coord(xp.z, reach);
            const int cx = hx + lane % 3 - 1, cy = hy + (lane / 3) % 3 - 1, cz = hz + lane / 9 - 1;
            const int b = list_bucket(cx, cy, cz, P.bucket_mask);
            const int64_t key = cell_key(cx, cy, cz);
            const float4* bpos = reinterpret_cast<const float4*>(B.bucket_pos);
            for (int it = B.bucket_start[b]; it < B.bucket_start[b + 1]; ++it) {
                if (B.bucket_key[it] != key) continue;
                const int q = B.bucket_items[it];
                const float4 xq4 = bpos[it];
                if (!(v3_len(v3_sub(v3(xq4.x, xq4.y, xq4.z), xp)) < reach)) continue;
                if (atomicExch(&B.relist[q], 1) == 0) B.relist_list[atomicAdd(&B.flags[BM_FLAG_RELIST], 1)] = q;
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_relist(bm_params P, bm_buffers B, const float* reach_in) {
    __shared__ int32_t found[8][BM_PAIR_LANES];
    __shared__ int found_count[8];
    const int count = min(B.flags[BM_FLAG_RELIST], P.n);
    if (count == 0) return;
    const int w = threadIdx.x >> 5;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + w; t < count; t += warps) {
        const int p = B.relist_list[t];
        build_list_warp(P, B, p, *reach_in, found[w], &found_count[w]);
        if ((threadIdx.x & 31) == 0) B.relist[p] = 0;
    }
}

// contact.pairs_listed (contact.py:825-925): each candidate adds its pair
// impulses to its rigid impulse in ascending partner order.  The lists are
// current by now, so the changed-code and relist counts are reset here.
__global__ void k_pairs(bm_params P, bm_buffers B, const float* reach_in) {
    const int candidates = min(B.flags[BM_FLAG_CANDIDATES], P.candidate_capacity);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.flags[BM_FLAG_CHANGED] = 0;
        B.flags[BM_FLAG_RELIST] = 0;
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < candidates; t += gridDim.x * blockDim.x)
        pair_particle(P, B, B.candidates[t], *reach_in);
}

__device__ void pair_particle(const bm_params& P, const bm_buffers& B, int p, float reach) {
    const int64_t N = P.n;
    const int step = B.flags[BM_FLAG_STEP];
    const int old = step & 1, nw = (step + 1) & 1;
    bm_v3 total = ld3(B.impulses, N, p);
    bool touched = false;
    const int count = B.partner_count[p];
    if (count >= 0) {
        const int32_t* list = B.partners + (int64_t)p * BM_PAIR_LANES;
        for (int i = 0; i < count; ++i) {
            bm_v3 j;
            if (pair_impulse(P, B, p, list[i], old, nw, &j)) {
                total = v3_add(total, j);
                touched = true;
            }
        }
    } else {
        // More partners than lanes: the buckets of the last list rebuild at the
        // rebuild position, visited in ascending particle order by repeated selection.
        const bm_v3 bx = ld3(B.built_x, N, p);
        const int hx = cell_coord(bx.x, reach), hy = cell_coord(bx.y, reach), hz = cell_coord(bx.z, reach);
        int last = -1;
        for (;;) {
            int next = INT32_MAX;
            for (int i = 0; i < 27; ++i) {
                const int cx = hx + i % 3 - 1, cy = hy + (i / 3) % 3 - 1, cz = hz + i / 9 - 1;
                const int b = list_bucket(cx, cy, cz, P.bucket_mask);
                for (int it = B.bucket_start[b]; it < B.bucket_start[b + 1]; ++it) {
                    const int q = B.bucket_items[it];
                    if (q == p || q <= last || q >= next) continue;
                    const bm_v3 xq = ld3(B.built_x, N, q);
                    if (cell_coord(xq.x, reach) != cx || cell_coord(xq.y, reach) != cy || cell_coord(xq.z, reach) != cz)
                        continue;
                    next = q;
                }
            }
            if (next == INT32_MAX) break;
            bm_v3 j;
            if (pair_impulse(P, B, p, next, old, nw, &j)) {
                total = v3_add(total, j);
                touched = true;
            }
            last = next;
        }
    }
    if (touched) st3(B.impulses, N, p, total);
}

// contact.count_embedded (contact.py:1042-1055) into flags[BM_FLAG_EMBEDDED].
__global__ void k_count_embedded(bm_params P, bm_buffers B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool inside = false;
    if (p < P.n) {
        const ToolF T = load_tool(B.tool_f);
        const bm_v3 local = q_rotate_inv(T.rot, v3_sub(ld3(B.x, P.n, p), T.pos));
        inside = fabsf(local.x) <= 6.0f * P.spacing && fabsf(local.y) <= P.half[1] && fabsf(local.z) <= P.half[2];
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, inside);
    if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(&B.flags[BM_FLAG_EMBEDDED], __popc(ballot));
}

// ------------------------------------------------------------------ probes

__global__ void k_blade_query(const float* local, int n, float h0, float h1, float h2, float bevel, float* closest,
                              float* normal, float* distance) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float half[3] = {h0, h1, h2};
    bm_v3 c, nn;
    float d;
    blade_query(v3(local[3 * i], local[3 * i + 1], local[3 * i + 2]), half, bevel, &c, &nn, &d);
    closest[3 * i] = c.x;
    closest[3 * i + 1] = c.y;
    closest[3 * i + 2] = c.z;
    normal[3 * i] = nn.x;
    normal[3 * i + 1] = nn.y;
    normal[3 * i + 2] = nn.z;
    distance[i] = d;
}

__global__ void k_friction(const float* normal, const float* relative, const float* jn, const float* history, int n,
                           float me, float dt, float mus, float mud, float gk, float gc, float* impulse,
                           float* new_history) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bm_v3 j, h;
    friction(v3(normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]),
             v3(relative[3 * i], relative[3 * i + 1], relative[3 * i + 2]), jn[i],
             v3(history[3 * i], history[3 * i + 1], history[3 * i + 2]), me, dt, mus, mud, gk, gc, &j, &h);
    impulse[3 * i] = j.x;
    impulse[3 * i + 1] = j.y;
    impulse[3 * i + 2] = j.z;
    new_history[3 * i] = h.x;
    new_history[3 * i + 1] = h.y;
    new_history[3 * i + 2] = h.z;
}

__global__ void k_resist_cut(const float* j, const float* x, const float* v, const float* origin, const float* tool_velocity,
                             const float* q, const float* tool_angular, float h0, float h1, float h2, float radius,
                             float spacing, float* damage, float threshold, int cutting, uint64_t* work_acc,
                             float* result, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float half[3] = {h0, h1, h2};
    bm_fx work = fx_zero();
    if (i < n) {
        bm_q qq;
        qq.x = q[0];
        qq.y = q[1];
        qq.z = q[2];
        qq.w = q[3];
        const bm_v3 r = resist_cut(v3(j[3 * i], j[3 * i + 1], j[3 * i + 2]), v3(x[3 * i], x[3 * i + 1], x[3 * i + 2]),
                                   v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]), v3(origin[0], origin[1], origin[2]),
                                   v3(tool_velocity[3 * i], tool_velocity[3 * i + 1], tool_velocity[3 * i + 2]), qq,
                                   v3(tool_angular[0], tool_angular[1], tool_angular[2]), half, radius, spacing,
                                   &damage[i], threshold, cutting, &work);
        result[3 * i] = r.x;
        result[3 * i + 1] = r.y;
        result[3 * i + 2] = r.z;
    }
    warp_accumulate(work_acc, work);
}

// --------------------------------------------------------------- launches

void launch_prologue(const bm_solver* s, int clear_step, cudaStream_t st, int registration) {
    k_prologue<<<1, 1024, 0, st>>>(s->P, s->B, clear_step, registration);
}

void launch_rigid(const bm_solver* s, int cut_bits, cudaStream_t st) {
    const int tb = spread_block(s->P.n);
    k_rigid<<<grid_for(s->P.n, tb), tb, 0, st>>>(s->P, s->B, cut_bits);
}

void launch_pairs(const bm_solver* s, cudaStream_t st) { launch_pairs_using(s, s->scan_partials, st); }

void launch_pairs_using(const bm_solver* s, int32_t* partials, cudaStream_t st) {
    launch_pair_lists(s, partials, 0, st);
    launch_pair_impulses(s, st);
}

void launch_pair_lists(const bm_solver* s, int32_t* partials, int find_speed, cudaStream_t st) {
    const int force = s->P.pair_search != 0;
    launch_pair_build(s, partials, !force, find_speed, st);
    if (!force) launch_relist(s, 1, st);
}

void launch_pair_build(const bm_solver* s, int32_t* partials, int gated, int find_speed, cudaStream_t st) {
    const bm_params& P = s->P;
    const bm_buffers& B = s->B;
    const int32_t* gate = gated ? &B.flags[BM_FLAG_PAIR_DIRTY] : nullptr;
    float* reach = reinterpret_cast<float*>(B.scratch);
    const int64_t buckets = s->buckets;
    const int64_t tiles = (buckets + 1023) / 1024;
    const unsigned wide = 4 * 152;  // grid-stride: cheap to launch when the gate is off
    const unsigned gb = grid_for(buckets) < wide ? grid_for(buckets) : wide;
    const unsigned gn = grid_for(P.n) < wide ? grid_for(P.n) : wide;
    const unsigned gt = tiles < 152 ? (unsigned)tiles : 152;
    k_pair_begin<<<gn > gb ? gn : gb, kBlock, 0, st>>>(P, B, buckets, gate, find_speed);
    k_bin_count<<<gn, kBlock, 0, st>>>(P, B, reach, gate);
    k_scan_tiles<<<gt, 1024, 0, st>>>(B.bucket_fill, B.bucket_start, buckets, partials, B.bucket_start + buckets,
                                      scan_ticket(B), gate);
    k_scan_add<<<gb, kBlock, 0, st>>>(B.bucket_start, buckets, partials, gate);
    k_bin_scatter<<<gn, kBlock, 0, st>>>(P, B, gate);
    k_build_lists<<<gn, kBlock, 0, st>>>(P, B, reach, gate);
}

void launch_relist(const bm_solver* s, int clear_dirty, cudaStream_t st) {
    float* reach = reinterpret_cast<float*>(s->B.scratch);
    k_relist_mark<<<152, kBlock, 0, st>>>(s->P, s->B, reach, clear_dirty);
    k_relist<<<152, kBlock, 0, st>>>(s->P, s->B, reach);
}

void launch_pair_impulses(const bm_solver* s, cudaStream_t st) {
    const bm_params& P = s->P;
    const unsigned wide = 4 * 152;
    const unsigned gc = grid_for(P.candidate_capacity) < wide ? grid_for(P.candidate_capacity) : wide;
    k_pairs<<<gc, kBlock, 0, st>>>(P, s->B, reinterpret_cast<float*>(s->B.scratch));
}

void launch_exclusive_scan(const int32_t* in, int32_t* out, int64_t count, int32_t* partials, int32_t* total_out,
                           int32_t* ticket, const int32_t* gate, cudaStream_t st) {
    const int64_t tiles = (count + 1023) / 1024;
    const unsigned gt = tiles < 152 ? (unsigned)(tiles < 1 ? 1 : tiles) : 152;
    const unsigned ga = grid_for(count) < 4 * 152 ? grid_for(count) : 4 * 152;
    k_scan_tiles<<<gt, 1024, 0, st>>>(in, out, count, partials, total_out, ticket, gate);
    k_scan_add<<<ga, kBlock, 0, st>>>(out, count, partials, gate);
}

void launch_count_embedded(const bm_solver* s, int reset, cudaStream_t st) {
    if (reset) cudaMemsetAsync(&s->B.flags[BM_FLAG_EMBEDDED], 0, sizeof(int32_t), st);
    k_count_embedded<<<grid_for(s->P.n), kBlock, 0, st>>>(s->P, s->B);
}

void launch_blade_query(const float* local, int n, const float* half, float bevel, float* closest, float* normal,
                        float* distance, cudaStream_t st) {
    k_blade_query<<<grid_for(n), kBlock, 0, st>>>(local, n, half[0], half[1], half[2], bevel, closest, normal, distance);
}

void launch_friction(const float* normal, const float* relative, const float* jn, const float* history, int n, float me,
                     float dt, float mus, float mud, float gk, float gc, float* impulse, float* new_history,
                     cudaStream_t st) {
    k_friction<<<grid_for(n), kBlock, 0, st>>>(normal, relative, jn, history, n, me, dt, mus, mud, gk, gc, impulse,
                                               new_history);
}

void launch_resist_cut(const float* j, const float* x, const float* v, const float* origin, const float* tool_velocity,
                       const float* q, const float* tool_angular, const float* half, float radius, float spacing,
                       float* damage, float threshold, int cutting, uint64_t* work_acc, float* result, int n,
                       cudaStream_t st) {
    k_resist_cut<<<grid_for(n, 32), 32, 0, st>>>(j, x, v, origin, tool_velocity, q, tool_angular, half[0], half[1],
                                                 half[2], radius, spacing, damage, threshold, cutting, work_acc, result,
                                                 n);
}

}  // namespace bm
