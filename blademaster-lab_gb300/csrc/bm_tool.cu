// Rigid knife integration and the external-tool interval bookkeeping
// (blademaster_warp/tool.py), in float64 on one thread per knife.  The
// particle kernels read a float32 mirror of the knife state (tool_f).
#include "bm_device.cuh"
#include "bm_internal.h"

namespace bm {

// Float32 knife record read by the particle kernels; the derived entries are
// evaluated with the same operations the particle code would apply.
__device__ void write_mirror(const bm_params& P, const bm_buffers& B, int k) {
    const double* t = B.tool + 13 * k;
    float* f = B.tool_f + BM_TOOL_F_WORDS * k;
    for (int i = 0; i < 13; ++i) f[i] = (float)t[i];
    const bm_v3 pos = v3(f[0], f[1], f[2]), vel = v3(f[3], f[4], f[5]), omega = v3(f[10], f[11], f[12]);
    bm_q q;
    q.x = f[6];
    q.y = f[7];
    q.z = f[8];
    q.w = f[9];
    f[13] = v3_len(vel);
    f[14] = v3_len(omega) * blade_radius(P);
    const bm_v3 edge = v3_add(pos, q_rotate(q, v3(0.0f, 0.0f, -P.half[2])));
    const bm_v3 down = q_rotate(q, v3(0.0f, 0.0f, -1.0f));
    const bm_v3 edge_vel = v3_add(vel, v3_cross(omega, v3_sub(edge, pos)));
    f[15] = edge.x;
    f[16] = edge.y;
    f[17] = edge.z;
    f[18] = down.x;
    f[19] = down.y;
    f[20] = down.z;
    f[21] = edge_vel.x;
    f[22] = edge_vel.y;
    f[23] = edge_vel.z;
    const bm_v3 ax = q_rotate(q, v3(1.0f, 0.0f, 0.0f)), ay = q_rotate(q, v3(0.0f, 1.0f, 0.0f)),
                az = q_rotate(q, v3(0.0f, 0.0f, 1.0f));
    f[24] = ax.x;
    f[25] = ax.y;
    f[26] = ax.z;
    f[27] = ay.x;
    f[28] = ay.y;
    f[29] = ay.z;
    f[30] = az.x;
    f[31] = az.y;
    f[32] = az.z;
    f[33] = f[34] = f[35] = 0.0f;
}

// tool.vertex (tool.py:118-138).
__device__ bm_v3d vertex(int i, const bm_params& P) {
    const int j = i % 5;
    double x = 0.0, z = -P.half_d[2], y;
    if (j == 1) {
        x = P.half_d[0];
        z += P.bevel_d;
    } else if (j == 2) {
        x = P.half_d[0];
        z = P.half_d[2];
    } else if (j == 3) {
        x = -P.half_d[0];
        z = P.half_d[2];
    } else if (j == 4) {
        x = -P.half_d[0];
        z += P.bevel_d;
    }
    y = -P.half_d[1];
    if (i >= 5) y = P.half_d[1];
    return v3d(x, y, z);
}

// ----------------------------------------------------- warp-parallel step
//
// Float64 instructions issue slowly on this part (a warp instruction costs
// the same whether one lane or 32 are active), so one warp runs each knife and
// spreads the float64 work over its lanes.  Lane c (mod 3 for vectors, mod 4
// for quaternions) evaluates component c of a vector expression with exactly
// the operations of the one-thread form in bm_scalar.h, the operands picked
// without a branch; shuffles then give every lane the whole vector.  Results
// are therefore bit-identical to evaluating the expressions on one thread.

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double pick3(bm_v3d a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }
__device__ __forceinline__ double pick4(bm_qd q, int c) { return c == 0 ? q.x : (c == 1 ? q.y : (c == 2 ? q.z : q.w)); }
__device__ __forceinline__ bm_v3d gather3(double mine) {
    return v3d(__shfl_sync(kFull, mine, 0), __shfl_sync(kFull, mine, 1), __shfl_sync(kFull, mine, 2));
}
__device__ __forceinline__ bm_qd gather4(double mine) {
    return qd(__shfl_sync(kFull, mine, 0), __shfl_sync(kFull, mine, 1), __shfl_sync(kFull, mine, 2),
              __shfl_sync(kFull, mine, 3));
}
// Component c of v3d_cross(a, b).
__device__ __forceinline__ double cross_c(bm_v3d a, bm_v3d b, int c) {
    const int i = c == 2 ? 0 : c + 1, j = c == 0 ? 2 : c - 1;
    return pick3(a, i) * pick3(b, j) - pick3(a, j) * pick3(b, i);
}
// Component c of qd_rotate(q, v) and qd_rotate_inv(q, v).
__device__ __forceinline__ double rot_c(bm_qd q, bm_v3d v, int c) {
    const bm_v3d u = v3d(q.x, q.y, q.z);
    const double cc = 2.0 * q.w * q.w - 1.0;
    const double d = 2.0 * v3d_dot(u, v);
    return (pick3(v, c) * cc + pick3(u, c) * d) + cross_c(u, v, c) * (2.0 * q.w);
}
__device__ __forceinline__ double rot_inv_c(bm_qd q, bm_v3d v, int c) {
    const bm_v3d u = v3d(q.x, q.y, q.z);
    const double cc = 2.0 * q.w * q.w - 1.0;
    const double d = 2.0 * v3d_dot(u, v);
    return (pick3(v, c) * cc - cross_c(u, v, c) * (2.0 * q.w)) + pick3(u, c) * d;
}
// Component c (0..3) of qd_mul(a, b): both forms are evaluated, then selected.
__device__ __forceinline__ double qmul_c(bm_qd a, bm_qd b, int c) {
    const int i = c < 3 ? c : 0;
    const double vec = a.w * pick4(b, i) + b.w * pick4(a, i) + cross_c(v3d(a.x, a.y, a.z), v3d(b.x, b.y, b.z), i);
    const double scalar = a.w * b.w - ((a.x * b.x + a.y * b.y) + a.z * b.z);
    return c < 3 ? vec : scalar;
}
// qd_normalize across lanes 0..3.
__device__ __forceinline__ bm_qd normalize_warp(bm_qd q, int c) {
    const double l = sqrt(((q.x * q.x + q.y * q.y) + q.z * q.z) + q.w * q.w);
    if (l > 0.0) return gather4(pick4(q, c) / l);
    return qd(0.0, 0.0, 0.0, 0.0);
}

// tool.inv_inertia (tool.py:141-143): one thread, and across lanes 0..2.
__device__ __forceinline__ bm_v3d inv_inertia(bm_qd q, bm_v3d ii, bm_v3d torque) {
    return qd_rotate(q, v3d_cw(ii, qd_rotate_inv(q, torque)));
}
__device__ __forceinline__ bm_v3d inv_inertia_warp(bm_qd q, bm_v3d ii, bm_v3d torque, int c) {
    const bm_v3d local = gather3(rot_inv_c(q, torque, c));
    const bm_v3d scaled = gather3(pick3(ii, c) * pick3(local, c));
    return gather3(rot_c(q, scaled, c));
}

// True when no vertex of the knife can meet the board during this substep's
// sweeps, shown in float32 with a margin: every vertex lies within R of the
// centre, so its gap is at least x.z - R and its normal speed at least
// -(|v.z| + |w| R); once the clearance exceeds twice dt times that speed,
// desired = -gap/dt stays below the vertex's normal speed and no sweep
// applies an impulse, so v and w pass through unchanged.  NaN never clears.
__device__ __forceinline__ bool board_clear(const bm_params& P, bm_v3d x, bm_v3d v, bm_v3d w) {
    const float reach = blade_radius(P) * 1.001f + 1.0e-6f;
    const float wx = (float)w.x, wy = (float)w.y, wz = (float)w.z;
    const float spin = sqrtf((wx * wx + wy * wy) + wz * wz) * 1.001f;
    const float clearance = (float)x.z - reach;
    const float travel = (float)P.dt_d * (fabsf((float)v.z) + spin * reach);
    return clearance > 0.0f && clearance > 2.0f * travel + 1.0e-30f;
}

// tool.step (tool.py:146-259) for knife k, run by all 32 lanes of one warp;
// lane 0 stores the result.
__device__ void drive_warp(const bm_params& P, const bm_buffers& B, int k, int index) {
    const int lane = threadIdx.x & 31, c = lane % 3, c4 = lane & 3;
    double* t = B.tool + 13 * k;
    const bm_v3d x = dget3(t);
    bm_v3d v = dget3(t + 3), w = dget3(t + 10);
    const bm_qd q = normalize_warp(qd(t[6], t[7], t[8], t[9]), c4);
    bm_fx fr, ft;
    fr.lo = B.acc[BM_ACC_REACTION(k) + 2 * c];
    fr.hi = B.acc[BM_ACC_REACTION(k) + 2 * c + 1];
    ft.lo = B.acc[BM_ACC_TORQUE(k) + 2 * c];
    ft.hi = B.acc[BM_ACC_TORQUE(k) + 2 * c + 1];
    const bm_v3d reaction = gather3(bm_fx_to_double(fr)), torque = gather3(bm_fx_to_double(ft));
    const double mass = P.blade_mass_d, dt = P.dt_d;
    bm_v3d force = v3d(0.0, 0.0, -9.81 * mass), servo_torque = v3d(0.0, 0.0, 0.0);
    if (P.free_blade == 0) {
        const float* tg = B.targets + 3 * index;
        const float* rt = B.rotations + 4 * index;
        const bm_qd target_q = qd(rt[0], rt[1], rt[2], rt[3]);
        const bm_v3d target_center = v3d_add(v3d(tg[0], tg[1], tg[2]), qd_rotate(target_q, v3d(0.0, 0.0, P.half_d[2])));
        force = v3d_sub(v3d_mul(v3d_sub(target_center, x), P.drive_stiffness), v3d_mul(v, P.drive_damping));
        const double norm = v3d_len(force);
        if (norm > P.drive_force_limit) force = v3d_mul(force, P.drive_force_limit / norm);
        bm_qd dq = qd_normalize(qd_mul(target_q, qd_inverse(q)));
        if (dq.w < 0.0) dq = qd(-dq.x, -dq.y, -dq.z, -dq.w);
        const bm_v3d vector = v3d(dq.x, dq.y, dq.z);
        const double s = v3d_len(vector);
        bm_v3d error = v3d_mul(vector, 2.0);
        if (s > 1.0e-8) error = v3d_mul(vector, 2.0 * bm_atan2(s, dq.w) / s);
        servo_torque = v3d_sub(v3d_mul(error, P.rot_stiffness), v3d_mul(w, P.rot_damping));
    }
    v = gather3(pick3(v, c) + (pick3(force, c) * dt + pick3(reaction, c)) / mass);
    bm_v3d ii = v3d(P.inertia_inv_d[0], P.inertia_inv_d[1], P.inertia_inv_d[2]);
    if (P.lock_rotation) {
        ii = v3d(0.0, 0.0, 0.0);
        w = v3d(0.0, 0.0, 0.0);
    } else {
        const bm_v3d local_w = gather3(rot_inv_c(q, w, c));
        const bm_v3d inertia = gather3(1.0 / pick3(ii, c));
        const bm_v3d spun = gather3(pick3(inertia, c) * pick3(local_w, c));
        const bm_v3d gyroscopic = gather3(rot_c(q, gather3(cross_c(local_w, spun, c)), c));
        const bm_v3d drive = gather3(pick3(torque, c) + (pick3(servo_torque, c) - pick3(gyroscopic, c)) * dt);
        w = gather3(pick3(w, c) + pick3(inv_inertia_warp(q, ii, drive, c), c));
    }
    const bm_v3d normal = v3d(0.0, 0.0, 1.0);
    bm_v3d total = v3d(0.0, 0.0, 0.0);
    if (!board_clear(P, x, v, w)) {
        // Sweep invariants of vertex `lane` (lanes 10..31 repeat vertex lane % 10).
        const int me = lane % 10;
        const bm_v3d r = qd_rotate(q, vertex(me, P)), corner = v3d_add(x, r);
        const bool skip = (P.board_half_d[0] > 0.0 && fabs(corner.x) > P.board_half_d[0]) ||
                          (P.board_half_d[1] > 0.0 && fabs(corner.y) > P.board_half_d[1]);
        const double gap = corner.z;
        double desired = -gap / dt;
        if (gap < 0.0) desired *= 0.2;
        const bm_v3d rn = v3d_cross(r, normal);
        const double effective = 1.0 / mass + v3d_dot(rn, inv_inertia(q, ii, rn));
        // Until a vertex acts, v and w stay as they are: when none acts on the
        // first sweep's values, no sweep acts at all.
        const double vn0 = v3d_dot(v3d_add(v, v3d_cross(w, r)), normal);
        const unsigned acting = __ballot_sync(kFull, lane < 10 && !skip && vn0 < desired);
        if (acting != 0u) {
            for (int sweep = 0; sweep < 6; ++sweep)
                for (int i = 0; i < 10; ++i) {
                    if (__shfl_sync(kFull, (int)skip, i)) continue;
                    const bm_v3d ri = v3d(__shfl_sync(kFull, r.x, i), __shfl_sync(kFull, r.y, i),
                                          __shfl_sync(kFull, r.z, i));
                    const double want = __shfl_sync(kFull, desired, i);
                    const double vn = v3d_dot(v3d_add(v, v3d_cross(w, ri)), normal);
                    if (vn < want) {
                        const double jn = (want - vn) / __shfl_sync(kFull, effective, i);
                        bm_v3d impulse = v3d_mul(normal, jn);
                        v = v3d_add(v, v3d_div(impulse, mass));
                        w = v3d_add(w, inv_inertia(q, ii, v3d_cross(ri, impulse)));
                        bm_v3d vt = v3d_add(v, v3d_cross(w, ri));
                        vt = v3d_sub(vt, v3d_mul(normal, v3d_dot(vt, normal)));
                        const double sp = v3d_len(vt);
                        if (sp > 1.0e-10) {
                            const bm_v3d direction = v3d_div(v3d_neg(vt), sp), rtd = v3d_cross(ri, direction);
                            const double wt = 1.0 / mass + v3d_dot(rtd, inv_inertia(q, ii, rtd));
                            const double jt = sp / wt < P.friction_dynamic_d * jn ? sp / wt : P.friction_dynamic_d * jn;
                            const bm_v3d tangent = v3d_mul(direction, jt);
                            impulse = v3d_add(impulse, tangent);
                            v = v3d_add(v, v3d_div(tangent, mass));
                            w = v3d_add(w, inv_inertia(q, ii, v3d_cross(ri, tangent)));
                        }
                        total = v3d_add(total, impulse);
                    }
                }
        }
    }
    const bm_v3d xn = gather3(pick3(x, c) + pick3(v, c) * dt);
    const double speed = v3d_len(w);
    bm_qd qn = q;
    if (speed > 1.0e-10) {
        const bm_v3d axis = gather3(pick3(w, c) / speed);
        double s, co;
        bm_sincos(0.5 * (dt * speed), &s, &co);
        const bm_qd turn = qd(axis.x * s, axis.y * s, axis.z * s, co);
        qn = normalize_warp(gather4(qmul_c(turn, q, c4)), c4);
    }
    if (lane == 0) {
        dput3(t, xn);
        dput3(t + 3, v);
        t[6] = qn.x;
        t[7] = qn.y;
        t[8] = qn.z;
        t[9] = qn.w;
        dput3(t + 10, w);
        dput3(B.table_impulse + 3 * k, total);
        write_mirror(P, B, k);
    }
}

// tool.accumulate_reaction (tool.py:6-16): interval sums about the world origin.
__device__ void accumulate_reaction(const bm_buffers& B) {
    const bm_v3d j = acc_read3(B.acc, BM_ACC_REACTION(0)), tau = acc_read3(B.acc, BM_ACC_TORQUE(0));
    const bm_v3d pos = dget3(B.tool);
    dput3(B.interval, v3d_add(dget3(B.interval), j));
    dput3(B.interval + 3, v3d_add(dget3(B.interval + 3), v3d_add(tau, v3d_cross(pos, j))));
}

// tool.finish_external_step (tool.py:70-115).
__device__ void finish_external(const bm_params& P, const bm_buffers& B) {
    double* t = B.tool;
    const bm_v3d j = acc_read3(B.acc, BM_ACC_REACTION(0)), tau = acc_read3(B.acc, BM_ACC_TORQUE(0));
    accumulate_reaction(B);
    if (P.predict) {
        const double u[6] = {j.x, j.y, j.z, tau.x, tau.y, tau.z};
        double dv[3] = {0.0, 0.0, 0.0}, dw[3] = {0.0, 0.0, 0.0};
        for (int row = 0; row < 3; ++row)
            for (int col = 0; col < 6; ++col) {
                dv[row] = dv[row] + (double)B.mobility[6 * row + col] * u[col];
                dw[row] = dw[row] + (double)B.mobility[6 * (row + 3) + col] * u[col];
            }
        dput3(t + 3, v3d_add(dget3(t + 3), v3d(dv[0], dv[1], dv[2])));
        const bm_v3d w = v3d_add(dget3(t + 10), v3d(dw[0], dw[1], dw[2]));
        dput3(t + 10, w);
        dput3(t, v3d_add(dget3(t), v3d_mul(dget3(t + 3), P.dt_d)));
        const double rate = v3d_len(w);
        if (rate > 1.0e-12) {
            bm_qd q = qd_mul(qd_from_axis_angle(v3d_div(w, rate), P.dt_d * rate), qd(t[6], t[7], t[8], t[9]));
            q = qd_normalize(q);
            t[6] = q.x;
            t[7] = q.y;
            t[8] = q.z;
            t[9] = q.w;
        }
        write_mirror(P, B, 0);
    }
    acc_clear3(B.acc, BM_ACC_REACTION(0));
    acc_clear3(B.acc, BM_ACC_TORQUE(0));
    acc_clear3(B.acc, BM_ACC_BOARD);
    B.speed[0] = 0.0f;
}

__global__ void k_tool(bm_params P, bm_buffers B, int mode) {
    const int k = threadIdx.x;
    if (mode == kToolFinishExternal) {
        if (k == 0) finish_external(P, B);
    } else if (mode == kToolClear) {
        if (k < P.tool_count) {
            acc_clear3(B.acc, BM_ACC_REACTION(k));
            acc_clear3(B.acc, BM_ACC_TORQUE(k));
        }
        if (k == 0) {
            acc_clear3(B.acc, BM_ACC_BOARD);
            B.speed[0] = 0.0f;
        }
    }
}

// One warp per knife (block k = knife k).  With accumulate, knife 0 first adds
// the substep's reaction to the interval sums about its position at the start
// of the substep (a single knife: the configuration refuses several).
__global__ void __launch_bounds__(32) k_tool_drive(bm_params P, bm_buffers B, int accumulate, int index) {
    if (accumulate && blockIdx.x == 0) {
        if (threadIdx.x == 0) accumulate_reaction(B);
        __syncwarp();
    }
    drive_warp(P, B, blockIdx.x, index);
}

// tool.load_external_state (tool.py:19-39).
__global__ void k_load_external(bm_params P, bm_buffers B) {
    const float* p = B.packed;
    double* t = B.tool;
    for (int i = 0; i < 3; ++i) t[i] = p[i];
    for (int i = 0; i < 4; ++i) t[6 + i] = p[3 + i];
    for (int i = 0; i < 3; ++i) t[3 + i] = p[7 + i];
    for (int i = 0; i < 3; ++i) t[10 + i] = p[10 + i];
    for (int i = 0; i < 36; ++i) B.mobility[i] = p[13 + i];
    for (int i = 0; i < 6; ++i) B.interval[i] = 0.0;
    write_mirror(P, B, 0);
}

// tool.store_interval (tool.py:56-67).
__global__ void k_store_interval(bm_buffers B) {
    for (int i = 0; i < 3; ++i) {
        B.result[i] = (float)B.interval[i];
        B.result[3 + i] = (float)B.interval[3 + i];
        B.result[6 + i] = (float)B.errors[i];
    }
}

// tool.record_pose (tool.py:42-53).
__global__ void k_record_pose(bm_buffers B, int index) {
    const int offset = 9 + 7 * index;
    for (int i = 0; i < 3; ++i) B.result[offset + i] = (float)B.tool[i];
    for (int i = 0; i < 4; ++i) B.result[offset + 3 + i] = (float)B.tool[6 + i];
}

__global__ void k_tool_mirror(bm_params P, bm_buffers B) {
    const int k = threadIdx.x;
    if (k < P.tool_count) write_mirror(P, B, k);
}

__global__ void k_read_acc(bm_params P, bm_buffers B, float* reaction, float* torque, float* board, float* work) {
    const int k = threadIdx.x;
    if (k < P.tool_count) {
        const bm_v3d r = acc_read3(B.acc, BM_ACC_REACTION(k)), t = acc_read3(B.acc, BM_ACC_TORQUE(k));
        if (reaction) {
            reaction[3 * k] = (float)r.x;
            reaction[3 * k + 1] = (float)r.y;
            reaction[3 * k + 2] = (float)r.z;
        }
        if (torque) {
            torque[3 * k] = (float)t.x;
            torque[3 * k + 1] = (float)t.y;
            torque[3 * k + 2] = (float)t.z;
        }
    }
    if (k == 0) {
        const bm_v3d b = acc_read3(B.acc, BM_ACC_BOARD);
        if (board) {
            board[0] = (float)b.x;
            board[1] = (float)b.y;
            board[2] = (float)b.z;
        }
        if (work) {
            bm_fx w;
            w.lo = B.acc[BM_ACC_WORK];
            w.hi = B.acc[BM_ACC_WORK + 1];
            work[0] = (float)bm_fx_to_double(w);
        }
    }
}

__device__ __forceinline__ void acc_put_float(uint64_t* acc, int word, float v) {
    const bm_fx f = bm_fx_from_float(v);
    acc[word] = f.lo;
    acc[word + 1] = f.hi;
}

__global__ void k_write_acc(bm_params P, bm_buffers B, const float* reaction, const float* torque, const float* board,
                            const float* work) {
    const int k = threadIdx.x;
    if (k < P.tool_count) {
        for (int i = 0; i < 3; ++i) {
            if (reaction) acc_put_float(B.acc, BM_ACC_REACTION(k) + 2 * i, reaction[3 * k + i]);
            if (torque) acc_put_float(B.acc, BM_ACC_TORQUE(k) + 2 * i, torque[3 * k + i]);
        }
    }
    if (k == 0) {
        for (int i = 0; i < 3; ++i)
            if (board) acc_put_float(B.acc, BM_ACC_BOARD + 2 * i, board[i]);
        if (work) acc_put_float(B.acc, BM_ACC_WORK, work[0]);
    }
}

// material.couple (material.py:155-193) on explicit per-node field runs
// (fields of node i are node_start[i] .. node_start[i+1], ascending code).
__global__ void k_couple_probe(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start,
                               int nodes, float* result) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nodes) return;
    const int begin = node_start[node], end = node_start[node + 1];
    for (int a = begin; a < end; ++a) {
        const float ma = mass[a];
        if (ma <= 0.0f) continue;
        const bm_v3 sa = v3(state[3 * a], state[3 * a + 1], state[3 * a + 2]);
        float total = 0.0f;
        bm_v3 ex = v3_zero();
        for (int b = begin; b < end; ++b) {
            const float mb = mass[b];
            total = total + mb;
            if (b != a && compatible_codes(codes[a], codes[b]))
                ex = v3_add(ex, v3_sub(v3_mul(v3(state[3 * b], state[3 * b + 1], state[3 * b + 2]), ma), v3_mul(sa, mb)));
        }
        const bm_v3 r = v3_add(sa, v3_div(ex, total));
        result[3 * a] = r.x;
        result[3 * a + 1] = r.y;
        result[3 * a + 2] = r.z;
    }
}

// material.g2p (material.py:343-381) on explicit slots and weights.
__global__ void k_g2p_probe(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                            const float* new_v, int n, float dt, float flip) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    bm_v3 pic = v3_zero(), dv = v3_zero();
    for (int a = 0; a < 8; ++a) {
        const int s = slots[8 * p + a];
        const float w = weights[8 * p + a];
        const bm_v3 nv = v3(new_v[3 * s], new_v[3 * s + 1], new_v[3 * s + 2]);
        const bm_v3 ov = v3(old_v[3 * s], old_v[3 * s + 1], old_v[3 * s + 2]);
        pic = v3_add(pic, v3_mul(nv, w));
        dv = v3_add(dv, v3_mul(v3_sub(nv, ov), w));
    }
    const bm_v3 vp = v3(v[3 * p], v[3 * p + 1], v[3 * p + 2]);
    const bm_v3 nvp = v3_add(v3_mul(pic, 1.0f - flip), v3_mul(v3_add(vp, dv), flip));
    v[3 * p] = nvp.x;
    v[3 * p + 1] = nvp.y;
    v[3 * p + 2] = nvp.z;
    x[3 * p] = x[3 * p] + pic.x * dt;
    x[3 * p + 1] = x[3 * p + 1] + pic.y * dt;
    x[3 * p + 2] = x[3 * p + 2] + pic.z * dt;
}

// --------------------------------------------------------------- launches

void launch_tool_step(const bm_solver* s, int mode, int target_index, int advance_step, cudaStream_t st) {
    (void)advance_step;
    if (mode == kToolDrive || mode == kToolAccumulate)
        k_tool_drive<<<s->P.tool_count, 32, 0, st>>>(s->P, s->B, mode == kToolAccumulate, target_index);
    else
        k_tool<<<1, 32, 0, st>>>(s->P, s->B, mode);
}
void launch_load_external(const bm_solver* s, cudaStream_t st) { k_load_external<<<1, 1, 0, st>>>(s->P, s->B); }
void launch_store_interval(const bm_solver* s, cudaStream_t st) { k_store_interval<<<1, 1, 0, st>>>(s->B); }
void launch_record_pose(const bm_solver* s, int index, cudaStream_t st) { k_record_pose<<<1, 1, 0, st>>>(s->B, index); }
void launch_tool_mirror(const bm_solver* s, cudaStream_t st) { k_tool_mirror<<<1, 32, 0, st>>>(s->P, s->B); }
void launch_read_acc(const bm_solver* s, float* reaction, float* torque, float* board, float* work, cudaStream_t st) {
    k_read_acc<<<1, 32, 0, st>>>(s->P, s->B, reaction, torque, board, work);
}
void launch_write_acc(const bm_solver* s, const float* reaction, const float* torque, const float* board,
                      const float* work, cudaStream_t st) {
    k_write_acc<<<1, 32, 0, st>>>(s->P, s->B, reaction, torque, board, work);
}
void launch_couple_probe(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start,
                         int nodes, float* result, cudaStream_t st) {
    k_couple_probe<<<grid_for(nodes), kBlock, 0, st>>>(codes, mass, state, node_start, nodes, result);
}
void launch_g2p_probe(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                      const float* new_v, int n, float dt, float flip, cudaStream_t st) {
    k_g2p_probe<<<grid_for(n), kBlock, 0, st>>>(x, v, slots, weights, old_v, new_v, n, dt, flip);
}

}  // namespace bm
