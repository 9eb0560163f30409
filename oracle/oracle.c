/*
 * CPU ORACLE - test infrastructure, not part of the product.
 *
 * A restatement in plain C of the reference's material substep
 * (Ju6276/BladeMaster-Lab, blademaster_warp/solver.py:920-940 and the Warp
 * kernels it launches), used only by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py to check the CUDA path.  Nothing in the
 * product links or loads it.
 *
 * Deterministic by construction where the reference is not (its float atomics
 * make repeated runs differ, tests/test_maxwell.py:21-32):
 *  - every scatter to the grid sums each slot's contributions in ascending
 *    particle order (particles are in device order: by reference cell);
 *  - the per-node field exchange visits a node's fields in ascending code;
 *  - pair impulses on a particle are added to its rigid impulse in ascending
 *    partner order, each pair evaluated from both sides (the two evaluations
 *    are exact negations);
 *  - reaction, torque, board and work sums use the exact 128-bit fixed-point
 *    accumulator of bm_scalar.h.
 * Arithmetic uses the elementary operations of bm_scalar.h, shared with the
 * kernels, compiled with -ffp-contract=off so no multiply-add is fused.
 *
 * Elastic stress: for yield_stress == 0 the fixed-corotated first Piola stress
 * is evaluated as P = 2 mu (f - R) + lam (J - 1) J f^-T with R the polar
 * rotation (bm_polar3), algebraically the reference's
 * U diag(2 mu (s - 1) + lam (J - 1) J / s) V^T (material.py:78-91).
 *
 * Layout: AoS in device particle order: x[n][3], F[n][9] row-major, ...
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/blademaster_gb300.h"
#ifdef ORC_REAL64
/* The float64 error-reference build of this restatement (liboracle64.so):
 * every float of the restatement and of the shared scalar header becomes
 * double (the parameter struct above keeps its float32 fields, read as
 * float32 values), and the float32 libm calls their double counterparts.
 * It runs the same scenes in double precision so that the float32 results
 * can be given an error against it; it is never compared bit for bit. */
typedef float orc_f32;
#define float double
#define sqrtf sqrt
#define fabsf fabs
#define floorf floor
#define rintf rint
#define ldexpf ldexp
#endif
#include "../blademaster-lab_gb300/csrc/bm_scalar.h"

#define ORC_API __attribute__((visibility("default")))

typedef struct orc_state {
    float* x;          /* [n][3] */
    float* v;          /* [n][3] */
    float* ref;        /* [n][3] */
    float* F;          /* [n][9] */
    float* Fp;         /* [n][9] */
    float* stress;     /* [n][9] */
    double* viscous;   /* [n][9] */
    int64_t* codes;    /* [n] */
    float* damage;     /* [tools][n] */
    float* histories;  /* [1 + tools][n][3] */
    float* impulses;   /* [n][3] */
    int32_t* nodes;    /* [n][8] */
    float* weights;    /* [n][8] */
    float* gradients;  /* [n][8][3] */
    /* registration */
    int64_t* keys;     /* [capacity] */
    int32_t* slots;    /* [n][8] */
    int32_t* node_start;   /* [node_count + 1] CSR of each node's slots, ascending code */
    int32_t* node_slots;   /* [capacity] */
    int32_t* slot_start;   /* [capacity + 1] CSR of each slot's contributions */
    int32_t* contrib;      /* [n * 8] p * 8 + a, ascending p */
    /* grid */
    float* grid_mass;  /* [capacity] */
    float* momentum;   /* [capacity][3] */
    float* grid_impulse;
    float* old_v;
    float* new_v;
    float* remapped;
    float* coupled;
    /* pairs */
    int64_t* pair_keys;    /* [2][pair_capacity] */
    float* pair_history;   /* [2][pair_capacity][3] */
    int32_t* pair_used;    /* [2][pair_capacity] */
    int32_t* pair_count;   /* [2] */
    int32_t* cell_head;    /* [buckets] scratch */
    int32_t* cell_start;   /* [cells + 1] particles of each reference cell (device order) */
    int32_t* cell_next;    /* [n] scratch */
    /* tool */
    double* tool;          /* [tools][13] */
    float* mobility;       /* [36] */
    uint64_t* acc;         /* BM_ACC_WORDS */
    double* interval;      /* [6] */
    double* table_impulse; /* [tools][3] */
    float* speed;          /* [1] */
    int32_t* errors;       /* [3] */
    int32_t* flags;        /* BM_FLAG_WORDS */
    float* result;         /* [10 + 7 * samples] */
    float* hold_side;      /* [n] entry side of each particle at the held knife (-1, 0, +1) */
    int64_t capacity;      /* key table capacity */
    int64_t buckets;       /* pair search buckets (power of two) */
} orc_state;

ORC_API uint32_t orc_state_size(void) { return (uint32_t)sizeof(orc_state); }

/* ------------------------------------------------------------- helpers */

static bm_v3 ld3(const float* a, int64_t i) { return v3(a[3 * i], a[3 * i + 1], a[3 * i + 2]); }
static void st3(float* a, int64_t i, bm_v3 v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
static bm_m33 ld9(const float* a, int64_t i) {
    bm_m33 m; int r, c;
    for (r = 0; r < 3; ++r) for (c = 0; c < 3; ++c) m.m[r][c] = a[9 * i + 3 * r + c];
    return m;
}
static void st9(float* a, int64_t i, bm_m33 m) {
    int r, c;
    for (r = 0; r < 3; ++r) for (c = 0; c < 3; ++c) a[9 * i + 3 * r + c] = m.m[r][c];
}
static bm_fx acc_get(const uint64_t* acc, int word) { bm_fx r; r.lo = acc[word]; r.hi = acc[word + 1]; return r; }
static void acc_put(uint64_t* acc, int word, bm_fx v) { acc[word] = v.lo; acc[word + 1] = v.hi; }
static bm_v3d acc_read3(const uint64_t* acc, int word) {
    return v3d(bm_fx_to_double(acc_get(acc, word)), bm_fx_to_double(acc_get(acc, word + 2)),
               bm_fx_to_double(acc_get(acc, word + 4)));
}
static void acc_clear3(uint64_t* acc, int word) { int i; for (i = 0; i < 6; ++i) acc[word + i] = 0u; }

/* Float32 mirror of the float64 tool state (what the particle kernels read). */
typedef struct { bm_v3 pos, vel, omega; bm_q rot; } tool_f32;
static tool_f32 tool_mirror(const double* t) {
    tool_f32 r;
    r.pos = v3((float)t[0], (float)t[1], (float)t[2]);
    r.vel = v3((float)t[3], (float)t[4], (float)t[5]);
    r.rot.x = (float)t[6]; r.rot.y = (float)t[7]; r.rot.z = (float)t[8]; r.rot.w = (float)t[9];
    r.omega = v3((float)t[10], (float)t[11], (float)t[12]);
    return r;
}

/* material.compatible (material.py:23-34) on int64 codes. */
static int compatible(int64_t a, int64_t b) {
    while (a != 0 || b != 0) {
        int64_t x = a % 3, y = b % 3;
        if (x != 0 && y != 0 && x != y) return 0;
        a /= 3;
        b /= 3;
    }
    return 1;
}

/* material.insert_key / contact.find_key (material.py:37-47, contact.py:569-580). */
static int64_t key_hash(int64_t key, int64_t capacity) {
    return (int64_t)(((uint64_t)key * (uint64_t)2654435761u) % (uint64_t)capacity);
}
static int64_t insert_key(int64_t* keys, int64_t key, int64_t capacity) {
    int64_t slot = key_hash(key, capacity), probe;
    for (probe = 0; probe < capacity; ++probe) {
        if (keys[slot] == -1) { keys[slot] = key; return slot; }
        if (keys[slot] == key) return slot;
        slot = (slot + 1) % capacity;
    }
    return -1;
}
static int64_t find_key(const int64_t* keys, int64_t key, int64_t capacity) {
    int64_t slot = key_hash(key, capacity), probe;
    for (probe = 0; probe < capacity; ++probe) {
        if (keys[slot] == -1) return -1;
        if (keys[slot] == key) return slot;
        slot = (slot + 1) % capacity;
    }
    return -1;
}

/* ------------------------------------------------------------ topology */

/* Solver._register_topology (solver.py:391-429) with material.register
 * (material.py:50-66) and node_lists (68-75).  A node's slots are listed in
 * ascending code; each slot's contributions in ascending particle order. */
ORC_API void orc_register(const bm_params* P, orc_state* S, const int64_t* field_codes) {
    int64_t n = P->n, cap = S->capacity, i, p;
    int a;
    int32_t* count;
    for (i = 0; i < cap; ++i) S->keys[i] = -1;
    for (p = 0; p < n; ++p)
        for (a = 0; a < 8; ++a) {
            int64_t key = field_codes[p] * (int64_t)P->node_count + (int64_t)S->nodes[8 * p + a];
            int64_t s = insert_key(S->keys, key, cap);
            S->slots[8 * p + a] = (int32_t)s;
            if (s < 0) S->errors[0] += 1;
        }
    /* node lists sorted by code */
    for (i = 0; i <= P->node_count; ++i) S->node_start[i] = 0;
    for (i = 0; i < cap; ++i)
        if (S->keys[i] >= 0) S->node_start[S->keys[i] % P->node_count + 1] += 1;
    for (i = 0; i < P->node_count; ++i) S->node_start[i + 1] += S->node_start[i];
    count = (int32_t*)calloc((size_t)(uint32_t)P->node_count, sizeof(int32_t));
    for (i = 0; i < cap; ++i)
        if (S->keys[i] >= 0) {
            int64_t node = S->keys[i] % P->node_count, j;
            int64_t pos = S->node_start[node] + count[node]++;
            /* insertion sort by code */
            int64_t code = S->keys[i] / P->node_count;
            for (j = pos; j > S->node_start[node] && S->keys[S->node_slots[j - 1]] / P->node_count > code; --j)
                S->node_slots[j] = S->node_slots[j - 1];
            S->node_slots[j] = (int32_t)i;
        }
    free(count);
    /* contribution CSR per slot */
    for (i = 0; i <= cap; ++i) S->slot_start[i] = 0;
    for (p = 0; p < n; ++p)
        for (a = 0; a < 8; ++a)
            if (S->slots[8 * p + a] >= 0) S->slot_start[S->slots[8 * p + a] + 1] += 1;
    for (i = 0; i < cap; ++i) S->slot_start[i + 1] += S->slot_start[i];
    count = (int32_t*)calloc((size_t)cap, sizeof(int32_t));
    for (p = 0; p < n; ++p)
        for (a = 0; a < 8; ++a) {
            int32_t s = S->slots[8 * p + a];
            if (s >= 0) S->contrib[S->slot_start[s] + count[s]++] = (int32_t)(8 * p + a);
        }
    free(count);
    S->flags[BM_FLAG_TOPOLOGY_DIRTY] = 0;
}

/* ------------------------------------------------------- constitutive */

/* material.corotated_stress (material.py:78-91). */
static bm_m33 corotated_stress(bm_m33 U, bm_v3 s, bm_m33 V, bm_m33 plastic_inverse, float mu, float lam) {
    float J = (s.x * s.y) * s.z;
    bm_v3 d;
    int i;
    for (i = 0; i < 3; ++i) {
        float si = v3_get(s, i);
        v3_set(&d, i, 2.0f * mu * (si - 1.0f) + lam * (J - 1.0f) * J / si);
    }
    return m33_mul(m33_mul(m33_mul(U, m33_diag(d)), m33_transpose(V)), m33_transpose(plastic_inverse));
}

/* Fixed-corotated stress of f through its polar rotation (see the header). */
static bm_m33 corotated_polar(bm_m33 f, float J, float mu, float lam) {
    bm_m33 R = bm_polar3(f), inv_t = m33_transpose(m33_inverse(f)), P;
    float c = lam * (J - 1.0f) * J, two_mu = 2.0f * mu;
    int i, j;
    for (i = 0; i < 3; ++i)
        for (j = 0; j < 3; ++j) P.m[i][j] = two_mu * (f.m[i][j] - R.m[i][j]) + c * inv_t.m[i][j];
    return P;
}

/* material.stress_at (material.py:94-112). */
static void stress_at(const bm_params* P, orc_state* S, int64_t p, int32_t* err) {
    bm_m33 F = ld9(S->F, p), f, pinv;
    float J;
    if (P->use_fp) {
        pinv = m33_inverse(ld9(S->Fp, p));
        f = m33_mul(F, pinv);
    } else {
        pinv = m33_identity();
        f = F;
    }
    J = m33_det(f);
    if (J <= 0.0f || !bm_isfinitef(J)) {
        *err += 1;
        st9(S->stress, p, m33_zero());
        return;
    }
    if (P->use_fp) st9(S->stress, p, m33_mul(corotated_polar(f, J, P->mu, P->lam), m33_transpose(pinv)));
    else st9(S->stress, p, corotated_polar(f, J, P->mu, P->lam));
}

/* material.plastic_at (material.py:404-431).  Returns 0 if inverted. */
static int plastic_at(const bm_params* P, orc_state* S, int64_t p, float yield_stress, bm_m33* U, bm_v3* s,
                      bm_m33* V, int32_t* err) {
    bm_m33 F = ld9(S->F, p);
    bm_v3 e, dev;
    float norm, limit, mean;
    bm_svd3(m33_mul(F, m33_inverse(ld9(S->Fp, p))), U, s, V);
    if (bm_minf(bm_minf(s->x, s->y), s->z) <= 0.0f) {
        *err += 1;
        return 0;
    }
    e = v3(bm_logf(s->x), bm_logf(s->y), bm_logf(s->z));
    mean = ((e.x + e.y) + e.z) / 3.0f;
    dev = v3_sub(e, v3(mean, mean, mean));
    norm = v3_len(dev);
    limit = yield_stress / (2.0f * P->mu) * sqrtf(2.0f / 3.0f);
    if (norm > limit) {
        bm_v3 ep = v3_sub(e, v3_mul(dev, 1.0f - limit / norm));
        bm_m33 next_f;
        *s = v3(bm_expf(ep.x), bm_expf(ep.y), bm_expf(ep.z));
        next_f = m33_mul(m33_mul(*U, m33_diag(*s)), m33_transpose(*V));
        st9(S->Fp, p, m33_mul(m33_inverse(next_f), F));
    }
    return 1;
}

/* material.maxwell_at (material.py:485-533). */
static void maxwell_at(const bm_params* P, orc_state* S, int64_t p, bm_m33 U, bm_v3 sigma, bm_m33 V, float relax,
                       int32_t* err) {
    bm_m33 f = m33_mul(m33_mul(U, m33_diag(sigma)), m33_transpose(V)), Df, fm, Um, Vm, kirchhoff, equilibrium;
    bm_v3 sm, e, dev;
    float mean, mu_eq, lam_eq;
    double* D = S->viscous + 9 * p;
    int r, c, k;
    for (r = 0; r < 3; ++r) for (c = 0; c < 3; ++c) Df.m[r][c] = (float)D[3 * r + c];
    fm = m33_mul(f, m33_inverse(m33_add(m33_identity(), Df)));
    bm_svd3(fm, &Um, &sm, &Vm);
    if (bm_minf(bm_minf(sm.x, sm.y), sm.z) <= 0.0f) {
        *err += 1;
        st9(S->stress, p, m33_zero());
        return;
    }
    e = v3(bm_logf(sm.x), bm_logf(sm.y), bm_logf(sm.z));
    mean = ((e.x + e.y) + e.z) / 3.0f;
    dev = v3_sub(e, v3(mean, mean, mean));
    if (relax > 0.0f) {
        bm_v3 step = v3_mul(dev, relax), growth;
        bm_m33 delta;
        double dd[9], nd[9];
        dev = v3_sub(dev, step);
        /* f_m <- f_m W with W = Vm diag(exp(-step)) Vm^T, i.e. Fv <- W^-1 Fv (material.py:518-521) */
        growth = v3(bm_expm1f(step.x), bm_expm1f(step.y), bm_expm1f(step.z));
        delta = m33_mul(m33_mul(Vm, m33_diag(growth)), m33_transpose(Vm));
        for (r = 0; r < 3; ++r) for (c = 0; c < 3; ++c) dd[3 * r + c] = (double)delta.m[r][c];
        /* D + delta + delta D in float64 */
        for (r = 0; r < 3; ++r)
            for (c = 0; c < 3; ++c) {
                double prod = 0.0;
                for (k = 0; k < 3; ++k) prod = prod + dd[3 * r + k] * D[3 * k + c];
                nd[3 * r + c] = (D[3 * r + c] + dd[3 * r + c]) + prod;
            }
        for (r = 0; r < 9; ++r) D[r] = nd[r];
    }
    kirchhoff = m33_mul(m33_mul(Um, m33_diag(v3_mul(dev, 2.0f * P->mu_maxwell))), m33_transpose(Um));
    mu_eq = P->mu - P->mu_maxwell;
    lam_eq = P->lam + 2.0f / 3.0f * P->mu_maxwell;
    equilibrium = corotated_stress(U, sigma, V, m33_inverse(ld9(S->Fp, p)), mu_eq, lam_eq);
    st9(S->stress, p, m33_add(equilibrium, m33_mul(kirchhoff, m33_transpose(m33_inverse(ld9(S->F, p))))));
}

/* material.maxwell_stress_at (material.py:536-566); with project == 0 the
 * stress of the current F, Fp and Fv alone (compute_stress_maxwell,
 * material.py:569-589: no return map, relax 0). */
static void maxwell_stress_at(const bm_params* P, orc_state* S, int64_t p, float relax, int project, int32_t* err) {
    bm_m33 U, V, f;
    bm_v3 sigma;
    float J;
    if (project && P->yield_stress > 0.0f) {
        if (!plastic_at(P, S, p, P->yield_stress, &U, &sigma, &V, err)) {
            st9(S->stress, p, m33_zero());
            return;
        }
        maxwell_at(P, S, p, U, sigma, V, relax, err);
        return;
    }
    f = m33_mul(ld9(S->F, p), m33_inverse(ld9(S->Fp, p)));
    J = m33_det(f);
    if (J <= 0.0f || !bm_isfinitef(J)) {
        *err += 1;
        st9(S->stress, p, m33_zero());
        return;
    }
    bm_svd3(f, &U, &sigma, &V);
    maxwell_at(P, S, p, U, sigma, V, relax, err);
}

/* Solver.refresh_stress (solver.py:318-329). */
ORC_API void orc_refresh_stress(const bm_params* P, orc_state* S) {
    int64_t p;
    for (p = 0; p < P->n; ++p) {
        if (P->maxwell) maxwell_stress_at(P, S, p, 0.0f, 0, &S->errors[1]);
        else stress_at(P, S, p, &S->errors[1]);
    }
}

/* update_F_maxwell (material.py:592-618) with a zero velocity gradient, `steps`
 * times: F is held and only the Maxwell branch relaxes (the reference's
 * hold_step, tests/test_maxwell.py:49-69). */
ORC_API void orc_maxwell_hold(const bm_params* P, orc_state* S, int steps) {
    int64_t p;
    int k;
    for (k = 0; k < steps; ++k)
        for (p = 0; p < P->n; ++p) maxwell_stress_at(P, S, p, P->maxwell_relax, 1, &S->errors[1]);
}

/* material.plastic_project (material.py:434-442). */
ORC_API void orc_plastic_project(const bm_params* P, orc_state* S, float yield_stress) {
    int64_t p;
    bm_m33 U, V;
    bm_v3 s;
    for (p = 0; p < P->n; ++p) plastic_at(P, S, p, yield_stress, &U, &s, &V, &S->errors[1]);
}

/* ------------------------------------------------------------ transfers */

/* couple_and_velocity_at (material.py:252-284): fields of the node in ascending code. */
static void couple_and_velocity(const bm_params* P, orc_state* S, int64_t a) {
    int64_t node, code_a, i;
    float total = 0.0f, ma = S->grid_mass[a];
    bm_v3 dm = v3_zero(), di = v3_zero(), pa = ld3(S->momentum, a), ja = ld3(S->grid_impulse, a), pm, jm;
    if (S->keys[a] < 0 || ma <= 0.0f) {
        st3(S->old_v, a, v3_zero());
        st3(S->new_v, a, v3_zero());
        return;
    }
    node = S->keys[a] % P->node_count;
    code_a = S->keys[a] / P->node_count;
    for (i = S->node_start[node]; i < S->node_start[node + 1]; ++i) {
        int64_t b = S->node_slots[i];
        float mb = S->grid_mass[b];
        total = total + mb;
        if (b != a && compatible(code_a, S->keys[b] / P->node_count)) {
            dm = v3_add(dm, v3_sub(v3_mul(ld3(S->momentum, b), ma), v3_mul(pa, mb)));
            di = v3_add(di, v3_sub(v3_mul(ld3(S->grid_impulse, b), ma), v3_mul(ja, mb)));
        }
    }
    pm = v3_add(pa, v3_div(dm, total));
    jm = v3_add(ja, v3_div(di, total));
    st3(S->old_v, a, v3_div(pm, ma));
    st3(S->new_v, a, v3_div(v3_add(pm, jm), ma));
}

/* couple_at (material.py:155-179). */
static void couple(const bm_params* P, orc_state* S, const float* state, float* result, int64_t a) {
    int64_t node, code_a, i;
    float total = 0.0f, ma = S->grid_mass[a];
    bm_v3 ex = v3_zero(), sa = ld3(state, a);
    if (S->keys[a] < 0 || ma <= 0.0f) return;
    node = S->keys[a] % P->node_count;
    code_a = S->keys[a] / P->node_count;
    for (i = S->node_start[node]; i < S->node_start[node + 1]; ++i) {
        int64_t b = S->node_slots[i];
        float mb = S->grid_mass[b];
        total = total + mb;
        if (b != a && compatible(code_a, S->keys[b] / P->node_count))
            ex = v3_add(ex, v3_sub(v3_mul(ld3(state, b), ma), v3_mul(sa, mb)));
    }
    st3(result, a, v3_add(sa, v3_div(ex, total)));
}

/* grid_vel_at (material.py:212-223). */
static void grid_vel(orc_state* S, const float* momentum, const float* impulse, int64_t s) {
    float m = S->grid_mass[s];
    if (m > 0.0f) {
        bm_v3 pm = ld3(momentum, s);
        st3(S->old_v, s, v3_div(pm, m));
        st3(S->new_v, s, v3_div(v3_add(pm, ld3(impulse, s)), m));
    }
}

/* The cell whose corner a is node n, or -1. */
static int64_t cell_at(const bm_params* P, int64_t n, int a) {
    int64_t nyz = (int64_t)P->node_dims[1] * P->node_dims[2];
    int64_t ci = n / nyz - ((a >> 2) & 1), cj = (n / P->node_dims[2]) % P->node_dims[1] - ((a >> 1) & 1),
            ck = n % P->node_dims[2] - (a & 1);
    if (ci < 0 || cj < 0 || ck < 0 || ci >= P->cell_dims[0] || cj >= P->cell_dims[1] || ck >= P->cell_dims[2]) return -1;
    return (ci * P->cell_dims[1] + cj) * P->cell_dims[2] + ck;
}

/* ((v0+v1)+(v2+v3))+((v4+v5)+(v6+v7)) */
static float tree8(const float* v) { return ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7])); }

/* p2g (material.py:127-152) in the canonical order: per slot, over the
 * adjacent cells in ascending cell index, the tree sum over the cell's 8
 * particle slots of the contributions that map to this slot (others +0);
 * cells without such a contribution are skipped. */
static void p2g(const bm_params* P, orc_state* S) {
    int64_t s;
    float dtv = P->dt * P->volume;
#pragma omp parallel for schedule(static)
    for (s = 0; s < S->capacity; ++s) {
        float m = 0.0f;
        bm_v3 mom = v3_zero(), J = v3_zero();
        int64_t n;
        int a, k;
        if (S->keys[s] >= 0) {
            n = S->keys[s] % P->node_count;
            for (a = 7; a >= 0; --a) {
                int64_t c = cell_at(P, n, a), b;
                int count, any = 0;
                float vm[8], v0[8], v1[8], v2[8], j0[8], j1[8], j2[8];
                if (c < 0) continue;
                b = S->cell_start[c];
                count = S->cell_start[c + 1] - S->cell_start[c];
                if (count == 0) continue;
                for (k = 0; k < 8; ++k) {
                    vm[k] = v0[k] = v1[k] = v2[k] = j0[k] = j1[k] = j2[k] = 0.0f;
                    if (k < count && S->slots[8 * (b + k) + a] == s) {
                        int64_t p = b + k;
                        float w = S->weights[8 * p + a], mw = P->mass * w;
                        bm_v3 g = ld3(S->gradients, 8 * p + a), mv = v3_mul(ld3(S->v, p), mw);
                        bm_v3 jv = v3_sub(v3_mul(ld3(S->impulses, p), w), m33_mul_v3(m33_scale(ld9(S->stress, p), dtv), g));
                        vm[k] = mw; v0[k] = mv.x; v1[k] = mv.y; v2[k] = mv.z; j0[k] = jv.x; j1[k] = jv.y; j2[k] = jv.z;
                        any = 1;
                    }
                }
                if (!any) continue;
                m = m + tree8(vm);
                mom = v3_add(mom, v3(tree8(v0), tree8(v1), tree8(v2)));
                J = v3_add(J, v3(tree8(j0), tree8(j1), tree8(j2)));
            }
        }
        S->grid_mass[s] = m;
        st3(S->momentum, s, mom);
        st3(S->grid_impulse, s, J);
    }
}

/* The MUSL re-scatter (material.py:400-401) in the same canonical order. */
static void remap(const bm_params* P, orc_state* S) {
    int64_t s;
#pragma omp parallel for schedule(static)
    for (s = 0; s < S->capacity; ++s) {
        bm_v3 r = v3_zero();
        int64_t n;
        int a, k;
        if (S->keys[s] >= 0) {
            n = S->keys[s] % P->node_count;
            for (a = 7; a >= 0; --a) {
                int64_t c = cell_at(P, n, a), b;
                int count, any = 0;
                float v0[8], v1[8], v2[8];
                if (c < 0) continue;
                b = S->cell_start[c];
                count = S->cell_start[c + 1] - S->cell_start[c];
                if (count == 0) continue;
                for (k = 0; k < 8; ++k) {
                    v0[k] = v1[k] = v2[k] = 0.0f;
                    if (k < count && S->slots[8 * (b + k) + a] == s) {
                        int64_t p = b + k;
                        bm_v3 rv = v3_mul(ld3(S->v, p), P->mass * S->weights[8 * p + a]);
                        v0[k] = rv.x; v1[k] = rv.y; v2[k] = rv.z;
                        any = 1;
                    }
                }
                if (any) r = v3_add(r, v3(tree8(v0), tree8(v1), tree8(v2)));
            }
        }
        st3(S->remapped, s, r);
    }
}

/* viscous_impulse (material.py:321-340), gathered per slot in ascending particle order. */
static void viscous_impulse(const bm_params* P, orc_state* S) {
    int64_t p, s;
    float* viscous_stress = (float*)malloc(sizeof(float) * 9 * (size_t)P->n);
#pragma omp parallel for schedule(static)
    for (p = 0; p < P->n; ++p) {
        bm_m33 rate = m33_zero(), inv, L, F = ld9(S->F, p);
        int a;
        for (a = 0; a < 8; ++a)
            rate = m33_add(rate, m33_outer(ld3(S->old_v, S->slots[8 * p + a]), ld3(S->gradients, 8 * p + a)));
        inv = m33_inverse(F);
        L = m33_mul(rate, inv);
        st9(viscous_stress, p,
            m33_mul(m33_scale(m33_add(L, m33_transpose(L)), P->dynamic_viscosity * m33_det(F)), m33_transpose(inv)));
    }
#pragma omp parallel for schedule(static)
    for (s = 0; s < S->capacity; ++s) {
        bm_v3 J = ld3(S->grid_impulse, s);
        int32_t i;
        for (i = S->slot_start[s]; i < S->slot_start[s + 1]; ++i) {
            int64_t q = S->contrib[i] / 8;
            int a = S->contrib[i] % 8;
            J = v3_add(J, m33_mul_v3(m33_scale(ld9(viscous_stress, q), -P->dt * P->volume), ld3(S->gradients, 8 * q + a)));
        }
        st3(S->grid_impulse, s, J);
    }
    free(viscous_stress);
}

/* g2p_at (material.py:343-367). */
static void g2p_at(const bm_params* P, orc_state* S, int64_t p) {
    bm_v3 pic = v3_zero(), dv = v3_zero(), v = ld3(S->v, p);
    int a;
    for (a = 0; a < 8; ++a) {
        int32_t s = S->slots[8 * p + a];
        float w = S->weights[8 * p + a];
        bm_v3 nv = ld3(S->new_v, s);
        pic = v3_add(pic, v3_mul(nv, w));
        dv = v3_add(dv, v3_mul(v3_sub(nv, ld3(S->old_v, s)), w));
    }
    st3(S->v, p, v3_add(v3_mul(pic, 1.0f - P->flip), v3_mul(v3_add(v, dv), P->flip)));
    st3(S->x, p, v3_add(ld3(S->x, p), v3_mul(pic, P->dt)));
}

/* F update of update_F_plastic / update_F_maxwell (material.py:461-467, 611-617). */
static void update_F(const bm_params* P, orc_state* S, int64_t p) {
    bm_m33 rate = m33_zero();
    int a;
    for (a = 0; a < 8; ++a) {
        int32_t s = S->slots[8 * p + a];
        float m = S->grid_mass[s];
        if (m > 0.0f) rate = m33_add(rate, m33_outer(v3_div(ld3(S->coupled, s), m), ld3(S->gradients, 8 * p + a)));
    }
    st9(S->F, p, m33_add(ld9(S->F, p), m33_scale(rate, P->dt)));
}

/* Solver.material_step (solver.py:334-376) and _material_transfers (431-535). */
/* ------------------------------------------------ held-blade constraint */

/* Per-slot scatter of w * j_p over the particles with `active` set, for the
 * slots of the listed nodes, then couple (couple_at, material.py:155-179)
 * into C; both zeroed first for those slots.  Order of a slot's sum: the
 * adjacent cells in ascending cell index (corner a = 7 ... 0), within a cell
 * ascending particles; one sequential float sum. */
static void hold_scatter_couple(const bm_params* P, orc_state* S, const int64_t* nodes, int64_t node_total,
                                const char* active, const float* j, float* G, float* C) {
    int64_t t;
    for (t = 0; t < node_total; ++t) {
        int64_t X = nodes[t], i;
        int a;
        for (i = S->node_start[X]; i < S->node_start[X + 1]; ++i) {
            int64_t s = S->node_slots[i];
            bm_v3 g = v3_zero();
            for (a = 7; a >= 0; --a) {
                int64_t c = cell_at(P, X, a), p;
                if (c < 0) continue;
                for (p = S->cell_start[c]; p < S->cell_start[c + 1]; ++p)
                    if (active[p] && S->slots[8 * p + a] == s) g = v3_add(g, v3_mul(ld3(j, p), S->weights[8 * p + a]));
            }
            st3(G, s, g);
        }
        for (i = S->node_start[X]; i < S->node_start[X + 1]; ++i) {
            int64_t s = S->node_slots[i];
            st3(C, s, v3_zero());
            couple(P, S, G, C, s);
        }
    }
}

/* response_at (blade_constraint.py:114-127): sum over a of w C / m, mass > 0. */
static bm_v3 hold_response(const orc_state* S, int64_t p, const float* C) {
    bm_v3 r = v3_zero();
    int a;
    for (a = 0; a < 8; ++a) {
        int32_t s = S->slots[8 * p + a];
        if (s >= 0 && S->grid_mass[s] > 0.0f) r = v3_add(r, v3_div(v3_mul(ld3(C, s), S->weights[8 * p + a]), S->grid_mass[s]));
    }
    return r;
}

/* BladeConstraint.solve (blade_constraint.py:254-324) for the externally held
 * knife 0: prepare (13-70), row_bound (73-90), batches of 48 projected
 * gradient iterations (project 130-152) until the largest inward residual
 * (record_residual 155-168) is at most 1e-6 m/s or 8 batches ran
 * (finish_refinement 171-184), then apply_grid (187-194) and apply_reaction
 * (197-205).  The reaction is subtracted in the exact fixed-point sums. */
static void hold_constraint(const bm_params* P, orc_state* S) {
    int64_t n = P->n, cap = S->capacity, p, m = 0, node_total = 0, t;
    tool_f32 T = tool_mirror(S->tool);
    float *normal = (float*)calloc((size_t)(3 * n), sizeof(float)), *lever = (float*)calloc((size_t)(3 * n), sizeof(float));
    float *rhs = (float*)calloc((size_t)n, sizeof(float)), *bound = (float*)calloc((size_t)n, sizeof(float));
    float *imp = (float*)calloc((size_t)n, sizeof(float)), *ext = (float*)calloc((size_t)n, sizeof(float));
    float *j = (float*)calloc((size_t)(3 * n), sizeof(float));
    float *G = (float*)calloc((size_t)(3 * cap), sizeof(float)), *C = (float*)calloc((size_t)(3 * cap), sizeof(float));
    char *active = (char*)calloc((size_t)n, 1), *mark = (char*)calloc((size_t)P->node_count, 1);
    int64_t *list = (int64_t*)malloc(sizeof(int64_t) * (size_t)n), *nodes = NULL;
    int needs = 0, batches = 0, a;
    float residual = 0.0f;
    for (p = 0; p < n; ++p) {
        bm_v3 local = q_rotate_inv(T.rot, v3_sub(ld3(S->x, p), T.pos)), grid_v = v3_zero(), nn;
        float side, gap;
        if (fabsf(local.y) >= P->half[1] || local.z <= -P->half[2] + P->bevel || local.z >= P->half[2]) {
            S->hold_side[p] = 0.0f;
            continue;
        }
        for (a = 0; a < 8; ++a) grid_v = v3_add(grid_v, v3_mul(ld3(S->new_v, S->slots[8 * p + a]), S->weights[8 * p + a]));
        side = S->hold_side[p];
        if (side == 0.0f || fabsf(local.x) > P->half[0] + P->blade_offset) side = local.x < 0.0f ? -1.0f : 1.0f;
        nn = q_rotate(T.rot, v3(side, 0.0f, 0.0f));
        gap = side * local.x - P->half[0];
        if (gap > P->blade_offset && gap + P->dt * v3_dot(grid_v, nn) > 0.0f) {
            S->hold_side[p] = 0.0f;
            continue;
        }
        S->hold_side[p] = side;
        active[p] = 1;
        st3(normal, p, nn);
        st3(lever, p, q_rotate(T.rot, v3(side * P->half[0], local.y, local.z)));
        rhs[p] = -bm_maxf(gap, 0.0f) / P->dt - v3_dot(grid_v, nn);
        if (rhs[p] > 1.0e-7f) needs = 1;
    }
    if (needs) {
        for (p = 0; p < n; ++p)
            if (active[p]) {
                list[m++] = p;
                for (a = 0; a < 8; ++a) mark[S->nodes[8 * p + a]] = 1;
            }
        nodes = (int64_t*)malloc(sizeof(int64_t) * (size_t)P->node_count);
        for (t = 0; t < P->node_count; ++t)
            if (mark[t]) nodes[node_total++] = t;
        /* active weights (w, 0, 0) coupled, then the absolute row-sum bound */
        for (t = 0; t < m; ++t) st3(j, list[t], v3(1.0f, 0.0f, 0.0f));
        hold_scatter_couple(P, S, nodes, node_total, active, j, G, C);
        for (t = 0; t < m; ++t) {
            float total = 0.0f;
            p = list[t];
            for (a = 0; a < 8; ++a) {
                int32_t s = S->slots[8 * p + a];
                if (s >= 0 && S->grid_mass[s] > 0.0f) total = total + S->weights[8 * p + a] * C[3 * s] / S->grid_mass[s];
            }
            bound[p] = total;
        }
        for (;;) {
            int it;
            for (t = 0; t < m; ++t) ext[list[t]] = imp[list[t]];
            for (it = 0; it < 48; ++it) {
                float acc = (float)((double)it / (double)(it + 3));
                for (t = 0; t < m; ++t) st3(j, list[t], v3_mul(ld3(normal, list[t]), ext[list[t]]));
                hold_scatter_couple(P, S, nodes, node_total, active, j, G, C);
                for (t = 0; t < m; ++t) {
                    bm_v3 r;
                    float previous, current;
                    p = list[t];
                    r = hold_response(S, p, C);
                    previous = imp[p];
                    current = bm_maxf(0.0f, ext[p] + (rhs[p] - v3_dot(ld3(normal, p), r)) / bm_maxf(bound[p], 1.0e-12f));
                    imp[p] = current;
                    ext[p] = current + acc * (current - previous);
                }
            }
            for (t = 0; t < m; ++t) st3(j, list[t], v3_mul(ld3(normal, list[t]), imp[list[t]]));
            hold_scatter_couple(P, S, nodes, node_total, active, j, G, C);
            residual = 0.0f;
            for (t = 0; t < m; ++t) {
                p = list[t];
                residual = bm_maxf(residual, bm_maxf(0.0f, rhs[p] - v3_dot(ld3(normal, p), hold_response(S, p, C))));
            }
            batches += 1;
            if (!(residual > 1.0e-6f && batches < 8)) break;
        }
        {
            float previous = bm_u2f((uint32_t)S->flags[BM_FLAG_HOLD_RESIDUAL]);
            S->flags[BM_FLAG_HOLD_RESIDUAL] = (int32_t)bm_f2u(bm_maxf(previous, residual));
        }
        /* apply_grid: every slot with mass (C is zero away from the contacts) */
        for (t = 0; t < cap; ++t)
            if (S->keys[t] >= 0 && S->grid_mass[t] > 0.0f)
                st3(S->new_v, t, v3_add(ld3(S->new_v, t), v3_div(ld3(C, t), S->grid_mass[t])));
        /* apply_reaction: reaction -= sum j, torque -= sum lever x j */
        {
            bm_fx sums[6];
            int k;
            for (k = 0; k < 6; ++k) sums[k] = acc_get(S->acc, k < 3 ? BM_ACC_REACTION(0) + 2 * k : BM_ACC_TORQUE(0) + 2 * (k - 3));
            for (t = 0; t < m; ++t) {
                bm_v3 jj = ld3(j, list[t]), tq = v3_cross(ld3(lever, list[t]), jj);
                sums[0] = bm_fx_add(sums[0], bm_fx_from_float(-jj.x));
                sums[1] = bm_fx_add(sums[1], bm_fx_from_float(-jj.y));
                sums[2] = bm_fx_add(sums[2], bm_fx_from_float(-jj.z));
                sums[3] = bm_fx_add(sums[3], bm_fx_from_float(-tq.x));
                sums[4] = bm_fx_add(sums[4], bm_fx_from_float(-tq.y));
                sums[5] = bm_fx_add(sums[5], bm_fx_from_float(-tq.z));
            }
            for (k = 0; k < 6; ++k) acc_put(S->acc, k < 3 ? BM_ACC_REACTION(0) + 2 * k : BM_ACC_TORQUE(0) + 2 * (k - 3), sums[k]);
        }
        S->flags[BM_FLAG_HOLD_COUNT] = (int32_t)m;
        S->flags[BM_FLAG_HOLD_NODES] = (int32_t)node_total;
    }
    free(normal); free(lever); free(rhs); free(bound); free(imp); free(ext); free(j); free(G); free(C);
    free(active); free(mark); free(list); free(nodes);
}

/* BladeConstraint.solve (blade_constraint.py:254-324) alone, on the current
 * grid velocities and masses, as the reference's tests/test_blade_constraint.py
 * calls it. */
ORC_API void orc_hold_solve(const bm_params* P, orc_state* S) { hold_constraint(P, S); }

ORC_API void orc_material_step(const bm_params* P, orc_state* S, const int64_t* field_codes, int register_now) {
    int64_t s, p;
    if (register_now) orc_register(P, S, field_codes);
    p2g(P, S);
    if (P->viscous) {
#pragma omp parallel for schedule(static)
        for (s = 0; s < S->capacity; ++s) couple(P, S, S->momentum, S->coupled, s);
#pragma omp parallel for schedule(static)
        for (s = 0; s < S->capacity; ++s) grid_vel(S, S->coupled, S->grid_impulse, s);
        viscous_impulse(P, S);
        /* couple the impulse into `remapped` as scratch, then the velocities */
#pragma omp parallel for schedule(static)
        for (s = 0; s < S->capacity; ++s) couple(P, S, S->grid_impulse, S->remapped, s);
#pragma omp parallel for schedule(static)
        for (s = 0; s < S->capacity; ++s) grid_vel(S, S->coupled, S->remapped, s);
    } else {
#pragma omp parallel for schedule(static)
        for (s = 0; s < S->capacity; ++s) couple_and_velocity(P, S, s);
    }
    if (P->external_tool && !P->predict) hold_constraint(P, S);
#pragma omp parallel for schedule(static)
    for (p = 0; p < P->n; ++p) g2p_at(P, S, p);
    remap(P, S);
#pragma omp parallel for schedule(static)
    for (s = 0; s < S->capacity; ++s) couple(P, S, S->remapped, S->coupled, s);
    {
        int32_t errors1 = 0;
#pragma omp parallel for schedule(static) reduction(+ : errors1)
        for (p = 0; p < P->n; ++p) {
            update_F(P, S, p);
            if (P->maxwell) {
                maxwell_stress_at(P, S, p, P->maxwell_relax, 1, &errors1);
            } else if (P->plastic) {
                bm_m33 U, V;
                bm_v3 sg;
                if (plastic_at(P, S, p, P->yield_stress, &U, &sg, &V, &errors1))
                    st9(S->stress, p, corotated_stress(U, sg, V, m33_inverse(ld9(S->Fp, p)), P->mu, P->lam));
                else
                    st9(S->stress, p, m33_zero());
            } else {
                stress_at(P, S, p, &errors1);
            }
        }
        S->errors[1] += errors1;
    }
}

/* ------------------------------------------------------------- contact */

/* contact.friction (contact.py:21-43). */
static void friction(bm_v3 n, bm_v3 relative, float jn, bm_v3 history, float me, float dt, float mus, float mud,
                     float gk, float gc, bm_v3* impulse, bm_v3* new_history) {
    bm_v3 vt = v3_sub(relative, v3_mul(n, v3_dot(relative, n)));
    bm_v3 ht = v3_sub(history, v3_mul(n, v3_dot(history, n)));
    float k = gk * me / (dt * dt);
    float damping = 2.0f * gc * sqrtf(me * k);
    bm_v3 trial = v3_mul(v3_sub(v3_mul(ht, -k), v3_mul(vt, damping)), dt);
    float magnitude = v3_len(trial);
    bm_v3 applied;
    if (magnitude <= mus * jn) {
        *impulse = trial;
        *new_history = v3_add(ht, v3_mul(vt, dt));
        return;
    }
    applied = v3_mul(trial, mud * jn / magnitude);
    *impulse = applied;
    *new_history = v3_div(v3_neg(v3_add(v3_div(applied, dt), v3_mul(vt, damping))), k);
}

ORC_API void orc_friction(const float* n, const float* relative, const float* jn, const float* history, int count,
                          float me, float dt, float mus, float mud, float gk, float gc, float* impulse,
                          float* new_history) {
    int i;
    for (i = 0; i < count; ++i) {
        bm_v3 j, h;
        friction(ld3(n, i), ld3(relative, i), jn[i], ld3(history, i), me, dt, mus, mud, gk, gc, &j, &h);
        st3(impulse, i, j);
        st3(new_history, i, h);
    }
}

/* contact.blade_query (contact.py:46-120). */
static void blade_query(bm_v3 local, const float* half, float bevel, bm_v3* closest_out, bm_v3* normal_out,
                        float* distance_out) {
    bm_v3 closest = v3(bm_clampf(local.x, -half[0], half[0]), bm_clampf(local.y, -half[1], half[1]),
                       bm_clampf(local.z, -half[2], half[2]));
    bm_v3 delta = v3_sub(local, closest), normal = v3_zero();
    float distance = v3_len(delta);
    if (bevel == 0.0f) {
        if (distance > 1.0e-12f) {
            normal = v3_div(delta, distance);
        } else {
            bm_v3 margin = v3(half[0] - fabsf(local.x), half[1] - fabsf(local.y), half[2] - fabsf(local.z));
            int axis = 0;
            if (margin.y < v3_get(margin, axis)) axis = 1;
            if (margin.z < v3_get(margin, axis)) axis = 2;
            v3_set(&normal, axis, 1.0f);
            if (v3_get(local, axis) < 0.0f) v3_set(&normal, axis, -1.0f);
            v3_set(&closest, axis, v3_get(normal, axis) * half[axis]);
            distance = -v3_get(margin, axis);
        }
    } else {
        float qx = fabsf(local.x), qy = local.z, sign = 1.0f;
        float ex = half[0], ey = bevel, len_sq, t, nx, ny, best_sq, ox, oy, cx, cy, dsq, best;
        int inside;
        if (local.x < 0.0f) sign = -1.0f;
        len_sq = ex * ex + ey * ey;
        t = bm_clampf((qx * ex + (qy + half[2]) * ey) / len_sq, 0.0f, 1.0f);
        nx = t * half[0];
        ny = -half[2] + t * bevel;
        best_sq = (qx - nx) * (qx - nx) + (qy - ny) * (qy - ny);
        ox = bevel / sqrtf(len_sq);
        oy = -half[0] / sqrtf(len_sq);
        cx = half[0];
        cy = bm_clampf(qy, -half[2] + bevel, half[2]);
        dsq = (qx - cx) * (qx - cx) + (qy - cy) * (qy - cy);
        if (dsq < best_sq) { best_sq = dsq; nx = cx; ny = cy; ox = 1.0f; oy = 0.0f; }
        cx = bm_clampf(qx, 0.0f, half[0]);
        cy = half[2];
        dsq = (qx - cx) * (qx - cx) + (qy - cy) * (qy - cy);
        if (dsq < best_sq) { best_sq = dsq; nx = cx; ny = cy; ox = 0.0f; oy = 1.0f; }
        inside = qx <= half[0] && qy <= half[2] && half[0] * (qy + half[2]) >= bevel * qx;
        best = sqrtf(best_sq);
        nx = sign * nx;
        ox = sign * ox;
        closest = v3(nx, bm_clampf(local.y, -half[1], half[1]), ny);
        if (inside && fabsf(local.y) <= half[1]) {
            normal = v3(ox, 0.0f, oy);
            distance = -best;
            if (half[1] - fabsf(local.y) < best) {
                float s2 = 1.0f;
                if (local.y < 0.0f) s2 = -1.0f;
                closest = local;
                closest.y = s2 * half[1];
                normal = v3(0.0f, s2, 0.0f);
                distance = -(half[1] - fabsf(local.y));
            }
        } else {
            if (inside) { closest.x = local.x; closest.z = local.z; }
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

ORC_API void orc_blade_query(const float* local, int count, const float* half, float bevel, float* closest,
                             float* normal, float* distance) {
    int i;
    for (i = 0; i < count; ++i) {
        bm_v3 c, nn;
        float d;
        blade_query(ld3(local, i), half, bevel, &c, &nn, &d);
        st3(closest, i, c);
        st3(normal, i, nn);
        distance[i] = d;
    }
}

/* contact.penalty_impulse (contact.py:123-147).  Returns 0 when separated. */
static int penalty_impulse(float gap, bm_v3 relative, bm_v3 n, float me, bm_v3 history, float dt, float sn, float mus,
                           float mud, float gk, float gc, bm_v3* impulse, bm_v3* new_history) {
    float predicted = gap + dt * bm_minf(v3_dot(relative, n), 0.0f), jn;
    bm_v3 jt, ht;
    if (predicted >= 0.0f) {
        *impulse = v3_zero();
        *new_history = v3_zero();
        return 0;
    }
    jn = sn * me / dt * (-predicted);
    friction(n, relative, jn, history, me, dt, mus, mud, gk, gc, &jt, &ht);
    *impulse = v3_add(v3_mul(n, jn), jt);
    *new_history = ht;
    return 1;
}

/* contact.blade_effective_mass (contact.py:150-178). */
static float blade_effective_mass(const bm_params* P, const float* mobility, bm_v3 lever, bm_v3 n, bm_q q) {
    float inverse = 1.0f / P->blade_mass;
    if (P->tool_model < 0) {
        bm_v3 rn = v3_cross(lever, n);
        float u[6];
        int row, col;
        u[0] = n.x; u[1] = n.y; u[2] = n.z; u[3] = rn.x; u[4] = rn.y; u[5] = rn.z;
        inverse = 0.0f;
        for (row = 0; row < 6; ++row)
            for (col = 0; col < 6; ++col) inverse = inverse + u[row] * mobility[6 * row + col] * u[col];
    } else if (P->tool_model > 0) {
        bm_v3 rn = q_rotate_inv(q, v3_cross(lever, n));
        inverse = inverse + v3_dot(rn, v3_cw(v3(P->inertia_inv[0], P->inertia_inv[1], P->inertia_inv[2]), rn));
    }
    return 1.0f / (1.0f / P->mass + inverse);
}

/* contact.resist_cut (contact.py:181-232).  Work is added to `work`. */
static bm_v3 resist_cut(bm_v3 j, bm_v3 xp, bm_v3 vp, bm_v3 origin, bm_v3 tool_velocity, bm_q q, bm_v3 tool_angular,
                        const float* half, float radius, float spacing, float* damage, float threshold, int cutting,
                        bm_fx* work) {
    bm_v3 edge = v3_add(origin, q_rotate(q, v3(0.0f, 0.0f, -half[2])));
    bm_v3 down = q_rotate(q, v3(0.0f, 0.0f, -1.0f));
    bm_v3 edge_velocity = v3_add(tool_velocity, v3_cross(tool_angular, v3_sub(edge, origin)));
    float front = v3_dot(v3_sub(xp, edge), down);
    float advance = v3_dot(v3_sub(edge_velocity, vp), down), push;
    bm_v3 local_edge;
    int ahead;
    if ((cutting & BM_CUT_ADVANCE) != 0) advance = v3_dot(edge_velocity, down);
    local_edge = q_rotate_inv(q, v3_sub(xp, edge));
    ahead = front >= 0.0f && front <= 2.0f * radius && fabsf(local_edge.x) <= 6.0f * spacing &&
            fabsf(local_edge.y) <= half[1];
    if (!ahead) return j;
    push = bm_maxf(v3_dot(j, down), 0.0f);
    if (*damage >= 1.0f) return v3_sub(j, v3_mul(down, push));
    if (advance > 0.0f) {
        float delta = push * advance;
        *work = bm_fx_add(*work, bm_fx_from_float(delta));
        *damage = bm_minf(1.0f, *damage + delta / threshold);
    }
    return j;
}

ORC_API void orc_resist_cut(const float* j, const float* x, const float* v, const float* origin,
                            const float* tool_velocity, const float* q, const float* tool_angular, const float* half,
                            float radius, float spacing, float* damage, float threshold, int cutting, uint64_t* work,
                            float* result, int count) {
    int i;
    bm_fx w;
    w.lo = work[0]; w.hi = work[1];
    for (i = 0; i < count; ++i) {
        bm_q qq;
        qq.x = q[0]; qq.y = q[1]; qq.z = q[2]; qq.w = q[3];
        st3(result, i, resist_cut(ld3(j, i), ld3(x, i), ld3(v, i), ld3(origin, 0), ld3(tool_velocity, i), qq,
                                  ld3(tool_angular, 0), half, radius, spacing, &damage[i], threshold, cutting, &w));
    }
    work[0] = w.lo; work[1] = w.hi;
}

/* Per-thread partial sums of the rigid contact reactions. */
typedef struct { bm_fx reaction[BM_MAX_TOOLS][3], torque[BM_MAX_TOOLS][3], board[3], work; } rigid_sums;

static void sums_add3(bm_fx* dst, bm_v3 v) {
    dst[0] = bm_fx_add(dst[0], bm_fx_from_float(v.x));
    dst[1] = bm_fx_add(dst[1], bm_fx_from_float(v.y));
    dst[2] = bm_fx_add(dst[2], bm_fx_from_float(v.z));
}

/* contact.blade_at (contact.py:235-329) for knife k. */
static bm_v3 blade_at(const bm_params* P, orc_state* S, int64_t p, int k, tool_f32 T, int cutting, rigid_sums* sums) {
    bm_v3 xp = ld3(S->x, p), vp = ld3(S->v, p), result = v3_zero();
    float* hist = S->histories + 3 * ((int64_t)(1 + k) * P->n + p);
    float* damage = S->damage + (int64_t)k * P->n + p;
    float blade_radius = sqrtf((P->half[0] * P->half[0] + P->half[1] * P->half[1]) + P->half[2] * P->half[2]);
    float max_closing = v3_len(vp) + v3_len(T.vel) + v3_len(T.omega) * blade_radius;
    if (v3_len(v3_sub(xp, T.pos)) - blade_radius - P->blade_offset > P->dt * max_closing) {
        hist[0] = hist[1] = hist[2] = 0.0f;
    } else {
        bm_v3 local = q_rotate_inv(T.rot, v3_sub(xp, T.pos)), closest_local, normal_local, lever, n, relative;
        float distance, front;
        const float half[3] = {P->half[0], P->half[1], P->half[2]};  /* the working type's copy */
        blade_query(local, half, P->bevel, &closest_local, &normal_local, &distance);
        front = -P->half[2] - local.z;
        if ((cutting & BM_CUT_HOLD) != 0 && *damage < 1.0f && fabsf(local.x) <= P->half[0] + P->blade_offset &&
            fabsf(local.y) <= P->half[1] && front >= 0.0f) {
            closest_local = v3(local.x, local.y, -P->half[2]);
            normal_local = v3(0.0f, 0.0f, -1.0f);
            distance = front;
        }
        lever = q_rotate(T.rot, closest_local);
        n = q_rotate(T.rot, normal_local);
        relative = v3_sub(v3_sub(vp, T.vel), v3_cross(T.omega, lever));
        if (distance - P->blade_offset + P->dt * bm_minf(v3_dot(relative, n), 0.0f) >= 0.0f) {
            hist[0] = hist[1] = hist[2] = 0.0f;
        } else {
            float me = blade_effective_mass(P, S->mobility, lever, n, T.rot);
            bm_v3 j, h;
            penalty_impulse(distance - P->blade_offset, relative, n, me, v3(hist[0], hist[1], hist[2]), P->dt,
                            P->normal_scale, P->friction_static, P->friction_dynamic, P->tangent_stiffness,
                            P->tangent_damping, &j, &h);
            hist[0] = h.x; hist[1] = h.y; hist[2] = h.z;
            if (v3_len_sq(j) > 0.0f) {
                if (cutting != 0)
                    j = resist_cut(j, xp, vp, T.pos, T.vel, T.rot, T.omega, half, P->blade_offset, P->spacing,
                                   damage, P->threshold, cutting, &sums->work);
                result = j;
                sums_add3(sums->reaction[k], v3_neg(j));
                sums_add3(sums->torque[k], v3_neg(v3_cross(lever, j)));
            }
        }
    }
    return result;
}

/* contact.rigid_and_speed + extra_blade (contact.py:332-566), every knife. */
ORC_API void orc_rigid_contacts(const bm_params* P, orc_state* S, int cutting) {
    int64_t p;
    int k, i;
    tool_f32 T[BM_MAX_TOOLS];
    rigid_sums total;
    float speed = S->speed[0];
    memset(&total, 0, sizeof(total));
    for (k = 0; k < P->tool_count; ++k) T[k] = tool_mirror(S->tool + 13 * k);
#pragma omp parallel
    {
        rigid_sums local;
        float local_speed = 0.0f;
        memset(&local, 0, sizeof(local));
#pragma omp for schedule(static)
        for (p = 0; p < P->n; ++p) {
            bm_v3 xp = ld3(S->x, p), vp = ld3(S->v, p), tot, jb, hb;
            float board_gap = xp.z - P->radius;
            float* hist = S->histories + 3 * p;
            local_speed = bm_maxf(local_speed, v3_len(vp));
            tot = v3(0.0f, 0.0f, -9.81f * P->mass * P->dt);
            if (P->board_half[0] > 0.0f && fabsf(xp.x) > P->board_half[0]) board_gap = 1.0e30f;
            if (P->board_half[1] > 0.0f && fabsf(xp.y) > P->board_half[1]) board_gap = 1.0e30f;
            penalty_impulse(board_gap, vp, v3(0.0f, 0.0f, 1.0f), P->mass, v3(hist[0], hist[1], hist[2]), P->dt,
                            P->board_scale, P->friction_static, P->friction_dynamic, P->tangent_stiffness,
                            P->tangent_damping, &jb, &hb);
            hist[0] = hb.x; hist[1] = hb.y; hist[2] = hb.z;
            if (v3_len_sq(jb) > 0.0f) {
                tot = v3_add(tot, jb);
                sums_add3(local.board, jb);
            }
            tot = v3_add(tot, blade_at(P, S, p, 0, T[0], cutting, &local));
            for (k = 1; k < P->tool_count; ++k) tot = v3_add(tot, blade_at(P, S, p, k, T[k], cutting, &local));
            st3(S->impulses, p, tot);
        }
#pragma omp critical
        {
            for (k = 0; k < P->tool_count; ++k)
                for (i = 0; i < 3; ++i) {
                    total.reaction[k][i] = bm_fx_add(total.reaction[k][i], local.reaction[k][i]);
                    total.torque[k][i] = bm_fx_add(total.torque[k][i], local.torque[k][i]);
                }
            for (i = 0; i < 3; ++i) total.board[i] = bm_fx_add(total.board[i], local.board[i]);
            total.work = bm_fx_add(total.work, local.work);
            speed = bm_maxf(speed, local_speed);
        }
    }
    for (k = 0; k < P->tool_count; ++k)
        for (i = 0; i < 3; ++i) {
            acc_put(S->acc, BM_ACC_REACTION(k) + 2 * i,
                    bm_fx_add(acc_get(S->acc, BM_ACC_REACTION(k) + 2 * i), total.reaction[k][i]));
            acc_put(S->acc, BM_ACC_TORQUE(k) + 2 * i,
                    bm_fx_add(acc_get(S->acc, BM_ACC_TORQUE(k) + 2 * i), total.torque[k][i]));
        }
    for (i = 0; i < 3; ++i)
        acc_put(S->acc, BM_ACC_BOARD + 2 * i, bm_fx_add(acc_get(S->acc, BM_ACC_BOARD + 2 * i), total.board[i]));
    acc_put(S->acc, BM_ACC_WORK, bm_fx_add(acc_get(S->acc, BM_ACC_WORK), total.work));
    S->speed[0] = speed;
}

/* pair_at (contact.py:583-640) from the side of p.  Returns 1 and the impulse on p
 * when the pair is in contact; the owner p < q records the friction history. */
static int pair_impulse(const bm_params* P, orc_state* S, int64_t p, int64_t q, int old, int nw, bm_v3* out,
                        int32_t* err0, int32_t* err2) {
    bm_v3 delta = v3_sub(ld3(S->x, p), ld3(S->x, q)), normal, relative, history = v3_zero(), jt, ht;
    float dist = v3_len(delta), predicted, jn, half_mass;
    int64_t lo = p < q ? p : q, hi = p < q ? q : p, key, oslot, nslot = -1;
    int owner = p < q;
    if (dist >= 2.0f * P->radius + P->dt * v3_len(v3_sub(ld3(S->v, p), ld3(S->v, q)))) return 0;
    if (compatible(S->codes[p], S->codes[q]) && v3_len(v3_sub(ld3(S->ref, p), ld3(S->ref, q))) < 2.0f * P->spacing)
        return 0;
    if (dist < 1.0e-12f) {
        if (owner) *err2 += 1;
        return 0;
    }
    normal = v3_div(delta, dist);
    relative = v3_sub(ld3(S->v, p), ld3(S->v, q));
    predicted = 2.0f * P->radius - dist - P->dt * bm_minf(v3_dot(relative, normal), 0.0f);
    if (predicted <= 0.0f) return 0;
    key = lo * (int64_t)P->n + hi;
    oslot = find_key(S->pair_keys + (int64_t)old * P->pair_capacity, key, P->pair_capacity);
    if (oslot >= 0) history = ld3(S->pair_history + 3 * (int64_t)old * P->pair_capacity, oslot);
    if (!owner) history = v3_neg(history);
    half_mass = P->mass / 2.0f;
    jn = P->normal_scale * half_mass / P->dt * predicted;
    friction(normal, relative, jn, history, half_mass, P->dt, P->friction_static, P->friction_dynamic,
             P->tangent_stiffness, P->tangent_damping, &jt, &ht);
    if (owner) {
        int failed = 0;
#pragma omp critical(orc_pair_table)
        {
            nslot = insert_key(S->pair_keys + (int64_t)nw * P->pair_capacity, key, P->pair_capacity);
            if (nslot < 0) {
                failed = 1;
            } else {
                st3(S->pair_history + 3 * (int64_t)nw * P->pair_capacity, nslot, ht);
                S->pair_used[(int64_t)nw * P->pair_capacity + S->pair_count[nw]] = (int32_t)nslot;
                S->pair_count[nw] += 1;
            }
        }
        if (failed) {
            *err0 += 1;
            return 0;
        }
    }
    *out = v3_add(v3_mul(normal, jn), jt);
    return 1;
}

static int64_t cell_coord(float x, float size) { return (int64_t)floorf(x / size); }
static int64_t list_bucket(int64_t cx, int64_t cy, int64_t cz, int64_t mask) {
    return (int64_t)((((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u)) &
                     (uint32_t)mask);
}

/* Solver.particle_contacts (solver.py:670-751): clear_pair_slots, then every
 * pair within 2 radius + 2 dt speed (the hash search reach, contact.py:684)
 * through pair_at.  Partners of a particle are visited in ascending order. */
ORC_API void orc_particle_contacts(const bm_params* P, orc_state* S) {
    int64_t n = P->n, p, i;
    int step = S->flags[BM_FLAG_STEP];
    int old = step % 2, nw = (step + 1) % 2;
    float reach = 2.0f * P->radius + 2.0f * P->dt * S->speed[0];
    int64_t mask = S->buckets - 1;
    int32_t err0 = 0, err2 = 0;
    for (i = 0; i < S->pair_count[nw]; ++i)
        S->pair_keys[(int64_t)nw * P->pair_capacity + S->pair_used[(int64_t)nw * P->pair_capacity + i]] = -1;
    S->pair_count[nw] = 0;
    /* each particle's cell, once (the candidate test below compares cells) */
    int64_t* cell = (int64_t*)malloc(sizeof(int64_t) * 3 * (size_t)(n > 0 ? n : 1));
    for (p = 0; p < n; ++p) {
        bm_v3 xp = ld3(S->x, p);
        cell[3 * p] = cell_coord(xp.x, reach);
        cell[3 * p + 1] = cell_coord(xp.y, reach);
        cell[3 * p + 2] = cell_coord(xp.z, reach);
    }
    for (i = 0; i < S->buckets; ++i) S->cell_head[i] = -1;
    for (p = n - 1; p >= 0; --p) {
        int64_t b = list_bucket(cell[3 * p], cell[3 * p + 1], cell[3 * p + 2], mask);
        S->cell_next[p] = S->cell_head[b];
        S->cell_head[b] = (int32_t)p;
    }
#pragma omp parallel
    {
    int64_t* list = (int64_t*)malloc(sizeof(int64_t) * 4096);
#pragma omp for schedule(dynamic, 64) reduction(+ : err0, err2)
    for (p = 0; p < n; ++p) {
        bm_v3 total = ld3(S->impulses, p);
        int64_t cx = cell[3 * p], cy = cell[3 * p + 1], cz = cell[3 * p + 2], count = 0, u, w;
        int c, touched = 0;
        for (c = 0; c < 27; ++c) {
            int64_t nx = cx + c % 3 - 1, ny = cy + (c / 3) % 3 - 1, nz = cz + c / 9 - 1;
            int32_t q = S->cell_head[list_bucket(nx, ny, nz, mask)];
            for (; q >= 0; q = S->cell_next[q]) {
                if (q == p) continue;
                if (cell[3 * q] != nx || cell[3 * q + 1] != ny || cell[3 * q + 2] != nz) continue;
                if (count < 4096) list[count++] = q;
            }
        }
        /* ascending partner order (insertion sort: the lists are short) */
        for (u = 1; u < count; ++u) {
            int64_t v = list[u];
            for (w = u; w > 0 && list[w - 1] > v; --w) list[w] = list[w - 1];
            list[w] = v;
        }
        for (int64_t li = 0; li < count; ++li) {
            bm_v3 j;
            if (pair_impulse(P, S, p, list[li], old, nw, &j, &err0, &err2)) {
                total = v3_add(total, j);
                touched = 1;
            }
        }
        if (touched) st3(S->impulses, p, total);
    }
    free(list);
    }
    free(cell);
    S->errors[0] += err0;
    S->errors[2] += err2;
}

/* contact.assign (contact.py:996-1039) for every knife k with digit 3^(cut_index + k). */
ORC_API void orc_assign(const bm_params* P, orc_state* S, int cut_index, int cutting) {
    int64_t p;
    int k, dirty = 0;
    for (k = 0; k < P->tool_count; ++k) {
        tool_f32 T = tool_mirror(S->tool + 13 * k);
        int64_t digit = 1;
        int e;
        for (e = 0; e < cut_index + k; ++e) digit *= 3;
        if (cutting == 0) continue;
#pragma omp parallel for schedule(static) reduction(| : dirty)
        for (p = 0; p < P->n; ++p) {
            bm_v3 xp = ld3(S->x, p), edge, local, edge_v, d, edge_here;
            float front, advance, back;
            int behind, on_board, pinched;
            if ((S->codes[p] / digit) % 3 != 0) continue;
            edge = v3_add(T.pos, q_rotate(T.rot, v3(0.0f, 0.0f, -P->half[2])));
            local = q_rotate_inv(T.rot, v3_sub(xp, edge));
            front = -local.z;
            edge_v = v3_add(T.vel, v3_cross(T.omega, v3_sub(edge, T.pos)));
            d = q_rotate(T.rot, v3(0.0f, 0.0f, -1.0f));
            advance = v3_dot(v3_sub(edge_v, ld3(S->v, p)), d);
            back = 2.0f * P->spacing + bm_maxf(advance * P->dt, 0.0f);
            behind = front >= -back && front <= 0.0f;
            on_board = (P->board_half[0] == 0.0f || fabsf(xp.x) <= P->board_half[0]) &&
                       (P->board_half[1] == 0.0f || fabsf(xp.y) <= P->board_half[1]);
            edge_here = v3_add(edge, q_rotate(T.rot, v3(0.0f, local.y, 0.0f)));
            pinched = on_board && edge_here.z <= P->radius && xp.z <= edge_here.z + P->radius;
            if (fabsf(local.x) <= 6.0f * P->spacing && fabsf(local.y) <= P->half[1] && (behind || pinched)) {
                int side = 2;
                if (local.x < 0.0f) side = 1;
                S->codes[p] += digit * (int64_t)side;
                dirty = 1;
            }
        }
    }
    if (dirty) S->flags[BM_FLAG_TOPOLOGY_DIRTY] = 1;
}

/* contact.count_embedded (contact.py:1042-1055). */
ORC_API int64_t orc_count_embedded(const bm_params* P, orc_state* S) {
    tool_f32 T = tool_mirror(S->tool);
    int64_t p, count = 0;
    for (p = 0; p < P->n; ++p) {
        bm_v3 local = q_rotate_inv(T.rot, v3_sub(ld3(S->x, p), T.pos));
        if (fabsf(local.x) <= 6.0f * P->spacing && fabsf(local.y) <= P->half[1] && fabsf(local.z) <= P->half[2])
            count += 1;
    }
    return count;
}

/* ---------------------------------------------------------------- tool */

static bm_v3d dget3(const double* t) { return v3d(t[0], t[1], t[2]); }
static void dput3(double* t, bm_v3d v) { t[0] = v.x; t[1] = v.y; t[2] = v.z; }

/* tool.vertex (tool.py:118-138). */
static bm_v3d vertex(int i, const bm_params* P) {
    int j = i % 5;
    double x = 0.0, z = -P->half_d[2], y;
    if (j == 1) { x = P->half_d[0]; z += P->bevel_d; }
    else if (j == 2) { x = P->half_d[0]; z = P->half_d[2]; }
    else if (j == 3) { x = -P->half_d[0]; z = P->half_d[2]; }
    else if (j == 4) { x = -P->half_d[0]; z += P->bevel_d; }
    y = -P->half_d[1];
    if (i >= 5) y = P->half_d[1];
    return v3d(x, y, z);
}

/* tool.inv_inertia (tool.py:141-143). */
static bm_v3d inv_inertia(bm_qd q, bm_v3d ii, bm_v3d torque) { return qd_rotate(q, v3d_cw(ii, qd_rotate_inv(q, torque))); }

/* tool.step (tool.py:146-259) for knife k in float64, reaction/torque from the accumulators. */
ORC_API void orc_drive_one(const bm_params* P, orc_state* S, int k, const float* target, const float* rotation) {
    double* t = S->tool + 13 * k;
    bm_v3d x = dget3(t), v = dget3(t + 3), w = dget3(t + 10), force, servo_torque = v3d(0, 0, 0), ii, total, normal;
    bm_qd q = qd_normalize(qd(t[6], t[7], t[8], t[9]));
    bm_v3d reaction = acc_read3(S->acc, BM_ACC_REACTION(k)), torque = acc_read3(S->acc, BM_ACC_TORQUE(k));
    double mass = P->blade_mass_d, dt = P->dt_d, speed;
    int sweep, i;
    force = v3d(0.0, 0.0, -9.81 * mass);
    if (P->free_blade == 0) {
        bm_qd target_q = qd(rotation[0], rotation[1], rotation[2], rotation[3]), dq;
        bm_v3d target_center = v3d_add(v3d(target[0], target[1], target[2]),
                                       qd_rotate(target_q, v3d(0.0, 0.0, P->half_d[2])));
        bm_v3d vector, error;
        double norm, s;
        force = v3d_sub(v3d_mul(v3d_sub(target_center, x), P->drive_stiffness), v3d_mul(v, P->drive_damping));
        norm = v3d_len(force);
        if (norm > P->drive_force_limit) force = v3d_mul(force, P->drive_force_limit / norm);
        dq = qd_normalize(qd_mul(target_q, qd_inverse(q)));
        if (dq.w < 0.0) dq = qd(-dq.x, -dq.y, -dq.z, -dq.w);
        vector = v3d(dq.x, dq.y, dq.z);
        s = v3d_len(vector);
        error = v3d_mul(vector, 2.0);
        if (s > 1.0e-8) error = v3d_mul(vector, 2.0 * bm_atan2(s, dq.w) / s);
        servo_torque = v3d_sub(v3d_mul(error, P->rot_stiffness), v3d_mul(w, P->rot_damping));
    }
    v = v3d_add(v, v3d_div(v3d_add(v3d_mul(force, dt), reaction), mass));
    ii = v3d(P->inertia_inv_d[0], P->inertia_inv_d[1], P->inertia_inv_d[2]);
    if (P->lock_rotation) {
        ii = v3d(0.0, 0.0, 0.0);
        w = v3d(0.0, 0.0, 0.0);
    } else {
        bm_v3d local_w = qd_rotate_inv(q, w);
        bm_v3d inertia = v3d(1.0 / ii.x, 1.0 / ii.y, 1.0 / ii.z);
        bm_v3d gyroscopic = qd_rotate(q, v3d_cross(local_w, v3d_cw(inertia, local_w)));
        w = v3d_add(w, inv_inertia(q, ii, v3d_add(torque, v3d_mul(v3d_sub(servo_torque, gyroscopic), dt))));
    }
    normal = v3d(0.0, 0.0, 1.0);
    total = v3d(0.0, 0.0, 0.0);
    for (sweep = 0; sweep < 6; ++sweep)
        for (i = 0; i < 10; ++i) {
            bm_v3d r = qd_rotate(q, vertex(i, P)), corner = v3d_add(x, r);
            double gap, vn, desired;
            if ((P->board_half_d[0] > 0.0 && fabs(corner.x) > P->board_half_d[0]) ||
                (P->board_half_d[1] > 0.0 && fabs(corner.y) > P->board_half_d[1]))
                continue;
            gap = corner.z;
            vn = v3d_dot(v3d_add(v, v3d_cross(w, r)), normal);
            desired = -gap / dt;
            if (gap < 0.0) desired *= 0.2;
            if (vn < desired) {
                bm_v3d rn = v3d_cross(r, normal), impulse, vt;
                double effective = 1.0 / mass + v3d_dot(rn, inv_inertia(q, ii, rn));
                double jn = (desired - vn) / effective, sp;
                impulse = v3d_mul(normal, jn);
                v = v3d_add(v, v3d_div(impulse, mass));
                w = v3d_add(w, inv_inertia(q, ii, v3d_cross(r, impulse)));
                vt = v3d_add(v, v3d_cross(w, r));
                vt = v3d_sub(vt, v3d_mul(normal, v3d_dot(vt, normal)));
                sp = v3d_len(vt);
                if (sp > 1.0e-10) {
                    bm_v3d direction = v3d_div(v3d_neg(vt), sp), rt = v3d_cross(r, direction), tangent;
                    double wt = 1.0 / mass + v3d_dot(rt, inv_inertia(q, ii, rt));
                    double jt = sp / wt < P->friction_dynamic_d * jn ? sp / wt : P->friction_dynamic_d * jn;
                    tangent = v3d_mul(direction, jt);
                    impulse = v3d_add(impulse, tangent);
                    v = v3d_add(v, v3d_div(tangent, mass));
                    w = v3d_add(w, inv_inertia(q, ii, v3d_cross(r, tangent)));
                }
                total = v3d_add(total, impulse);
            }
        }
    x = v3d_add(x, v3d_mul(v, dt));
    speed = v3d_len(w);
    if (speed > 1.0e-10) q = qd_normalize(qd_mul(qd_from_axis_angle(v3d_div(w, speed), dt * speed), q));
    dput3(t, x);
    dput3(t + 3, v);
    t[6] = q.x; t[7] = q.y; t[8] = q.z; t[9] = q.w;
    dput3(t + 10, w);
    dput3(S->table_impulse + 3 * k, total);
}

/* tool.accumulate_reaction (tool.py:6-16), knife 0. */
ORC_API void orc_accumulate_tool_impulses(const bm_params* P, orc_state* S) {
    bm_v3d j = acc_read3(S->acc, BM_ACC_REACTION(0)), tau = acc_read3(S->acc, BM_ACC_TORQUE(0));
    bm_v3d pos = dget3(S->tool);
    (void)P;
    dput3(S->interval, v3d_add(dget3(S->interval), j));
    dput3(S->interval + 3, v3d_add(dget3(S->interval + 3), v3d_add(tau, v3d_cross(pos, j))));
}

/* tool.finish_external_step (tool.py:70-115). */
ORC_API void orc_finish_external(const bm_params* P, orc_state* S) {
    double* t = S->tool;
    bm_v3d j = acc_read3(S->acc, BM_ACC_REACTION(0)), tau = acc_read3(S->acc, BM_ACC_TORQUE(0));
    bm_v3d pos = dget3(t);
    dput3(S->interval, v3d_add(dget3(S->interval), j));
    dput3(S->interval + 3, v3d_add(dget3(S->interval + 3), v3d_add(tau, v3d_cross(pos, j))));
    if (P->predict) {
        double u[6] = {j.x, j.y, j.z, tau.x, tau.y, tau.z}, dv[3] = {0, 0, 0}, dw[3] = {0, 0, 0}, rate;
        int row, col;
        bm_v3d w;
        for (row = 0; row < 3; ++row)
            for (col = 0; col < 6; ++col) {
                dv[row] = dv[row] + (double)S->mobility[6 * row + col] * u[col];
                dw[row] = dw[row] + (double)S->mobility[6 * (row + 3) + col] * u[col];
            }
        dput3(t + 3, v3d_add(dget3(t + 3), v3d(dv[0], dv[1], dv[2])));
        w = v3d_add(dget3(t + 10), v3d(dw[0], dw[1], dw[2]));
        dput3(t + 10, w);
        dput3(t, v3d_add(dget3(t), v3d_mul(dget3(t + 3), P->dt_d)));
        rate = v3d_len(w);
        if (rate > 1.0e-12) {
            bm_qd q = qd_mul(qd_from_axis_angle(v3d_div(w, rate), P->dt_d * rate), qd(t[6], t[7], t[8], t[9]));
            q = qd_normalize(q);
            t[6] = q.x; t[7] = q.y; t[8] = q.z; t[9] = q.w;
        }
    }
    acc_clear3(S->acc, BM_ACC_REACTION(0));
    acc_clear3(S->acc, BM_ACC_TORQUE(0));
    acc_clear3(S->acc, BM_ACC_BOARD);
    S->speed[0] = 0.0f;
}

/* contact.clear_step (contact.py:1058-1068) for every knife. */
ORC_API void orc_clear_step(const bm_params* P, orc_state* S) {
    int k;
    for (k = 0; k < P->tool_count; ++k) {
        acc_clear3(S->acc, BM_ACC_REACTION(k));
        acc_clear3(S->acc, BM_ACC_TORQUE(k));
    }
    acc_clear3(S->acc, BM_ACC_BOARD);
    S->speed[0] = 0.0f;
}

/* tool.load_external_state (tool.py:19-39). */
ORC_API void orc_load_external(const bm_params* P, orc_state* S, const float* packed) {
    double* t = S->tool;
    int i;
    (void)P;
    for (i = 0; i < 3; ++i) t[i] = packed[i];
    for (i = 0; i < 4; ++i) t[6 + i] = packed[3 + i];
    for (i = 0; i < 3; ++i) t[3 + i] = packed[7 + i];
    for (i = 0; i < 3; ++i) t[10 + i] = packed[10 + i];
    for (i = 0; i < 36; ++i) S->mobility[i] = packed[13 + i];
    for (i = 0; i < 6; ++i) S->interval[i] = 0.0;
}

/* material.validate_interval (material.py:6-20). */
ORC_API void orc_validate_interval(const bm_params* P, orc_state* S) {
    int64_t p;
    for (p = 0; p < P->n; ++p) {
        float d = m33_det(ld9(S->F, p));
        int i;
        if (d <= 0.0f || !bm_isfinitef(d)) S->errors[1] += 1;
        for (i = 0; i < 3; ++i)
            if (!bm_isfinitef(S->x[3 * p + i]) || !bm_isfinitef(S->v[3 * p + i])) S->errors[1] += 1;
    }
}

/* One substep, Solver._step_kernels (solver.py:920-940).  target/rotation: the
 * driven knives' target edge and orientation of this substep. */
ORC_API void orc_substep(const bm_params* P, orc_state* S, int cut_bits, int cut_index, const int64_t* field_codes,
                         int cache_topology, const float* target, const float* rotation) {
    int k;
    if (!P->external_tool) orc_clear_step(P, S);
    orc_rigid_contacts(P, S, cut_bits);
    orc_particle_contacts(P, S);
    orc_material_step(P, S, field_codes, !cache_topology || S->flags[BM_FLAG_TOPOLOGY_DIRTY]);
    if (P->external_tool) {
        orc_finish_external(P, S);
    } else {
        if (P->accumulate_tool_impulses) orc_accumulate_tool_impulses(P, S);
        for (k = 0; k < P->tool_count; ++k) orc_drive_one(P, S, k, target, rotation);
    }
    orc_assign(P, S, cut_index, cut_bits != 0);
    S->flags[BM_FLAG_STEP] += 1;
}

/* --------------------------------------------------------------- MLS-MPM */

/* MlsSolver state (mlsmpm.py:232-291), particle arrays AoS in reference order. */
typedef struct {
    float* x;                /* [n][3] (shared with the contact state) */
    float* v;                /* [n][3] */
    float* C;                /* [n][9] */
    float* F;                /* [n][9] */
    float* yield_stress;     /* [n] */
    float* damage;           /* [n] */
    float* damage_reference; /* [n] */
    int64_t* grid_mass;      /* [nodes] fixed point */
    int64_t* grid_momentum;  /* [nodes][3] fixed point */
    float* grid_v;           /* [nodes][3] */
    int32_t* inversions;     /* [1] */
} orc_mls_state;

ORC_API uint32_t orc_mls_state_size(void) { return (uint32_t)sizeof(orc_mls_state); }

/* spline_weights (mlsmpm.py:41-51). */
static void mls_weights(bm_v3 fx, float w[3][3]) {
    int axis;
    for (axis = 0; axis < 3; ++axis) {
        float f = v3_get(fx, axis);
        w[0][axis] = 0.5f * (1.5f - f) * (1.5f - f);
        w[1][axis] = 0.75f - (f - 1.0f) * (f - 1.0f);
        w[2][axis] = 0.5f * (f - 0.5f) * (f - 0.5f);
    }
}

/* cell_base + inside_domain (mlsmpm.py:54-72). */
static int mls_locate(const bm_mls_params* M, bm_v3 x, int base[3], bm_v3* fx) {
    bm_v3 local;
    float f[3];
    int i;
    if (!bm_isfinitef(x.x) || !bm_isfinitef(x.y) || !bm_isfinitef(x.z)) return 0;
    local = v3_div(v3_sub(x, v3(M->origin[0], M->origin[1], M->origin[2])), M->dx);
    for (i = 0; i < 3; ++i) {
        float b = floorf(v3_get(local, i) - 0.5f);
        if (!(b >= 0.0f && b < (float)(M->dims[i] - 2))) return 0;
        base[i] = (int)b;
        f[i] = v3_get(local, i) - b;
    }
    *fx = v3(f[0], f[1], f[2]);
    return 1;
}

/* MlsSolver._substep (mlsmpm.py:293-393): rigid_and_speed for the held knife
 * (cutting off), accumulate_reaction, p2g (exact fixed-point grid sums),
 * grid_update, g2p. */
ORC_API void orc_mls_substep(const bm_mls_params* M, orc_mls_state* T, const bm_params* P, orc_state* S) {
    int64_t n = M->n, nodes = (int64_t)M->dims[0] * M->dims[1] * M->dims[2], p, node;
    int32_t inversions = 0;
    orc_rigid_contacts(P, S, 0);
    {
        bm_v3d j = acc_read3(S->acc, BM_ACC_REACTION(0)), tau = acc_read3(S->acc, BM_ACC_TORQUE(0));
        S->interval[0] += j.x; S->interval[1] += j.y; S->interval[2] += j.z;
        S->interval[3] += tau.x; S->interval[4] += tau.y; S->interval[5] += tau.z;
        acc_clear3(S->acc, BM_ACC_REACTION(0));
        acc_clear3(S->acc, BM_ACC_TORQUE(0));
        acc_clear3(S->acc, BM_ACC_BOARD);
        S->speed[0] = 0.0f;
    }
    memset(T->grid_mass, 0, sizeof(int64_t) * (size_t)nodes);
    memset(T->grid_momentum, 0, sizeof(int64_t) * 3 * (size_t)nodes);
#pragma omp parallel for schedule(static)
    for (p = 0; p < n; ++p) {
        int base[3], i, j, k;
        bm_v3 fx, sigma, momentum;
        float w[3][3], shear;
        bm_m33 F, U, V, Ps, stress, affine;
        if (!mls_locate(M, ld3(T->x, p), base, &fx)) continue;
        mls_weights(fx, w);
        shear = T->damage[p] > 0.0f ? M->mu * M->damaged_shear : M->mu;
        F = ld9(T->F, p);
        bm_svd3(F, &U, &sigma, &V);
        Ps = corotated_stress(U, sigma, V, m33_identity(), shear, M->lam);
        stress = m33_mul(m33_scale(Ps, (-M->dt * M->volume * 4.0f) / (M->dx * M->dx)), m33_transpose(F));
        affine = m33_add(stress, m33_scale(ld9(T->C, p), M->mass));
        momentum = v3_add(v3_mul(ld3(T->v, p), M->mass), ld3(S->impulses, p));
        for (i = 0; i < 3; ++i)
            for (j = 0; j < 3; ++j)
                for (k = 0; k < 3; ++k) {
                    float weight = (w[i][0] * w[j][1]) * w[k][2];
                    bm_v3 dpos = v3_mul(v3_sub(v3((float)i, (float)j, (float)k), fx), M->dx);
                    bm_v3 c = v3_mul(v3_add(momentum, m33_mul_v3(affine, dpos)), weight);
                    int64_t at = ((int64_t)(base[0] + i) * M->dims[1] + (base[1] + j)) * M->dims[2] + (base[2] + k);
                    int64_t cx = bm_fixed64(c.x, M->momentum_shift), cy = bm_fixed64(c.y, M->momentum_shift);
                    int64_t cz = bm_fixed64(c.z, M->momentum_shift), cm = bm_fixed64(weight * M->mass, M->mass_shift);
#pragma omp atomic
                    T->grid_momentum[3 * at] += cx;
#pragma omp atomic
                    T->grid_momentum[3 * at + 1] += cy;
#pragma omp atomic
                    T->grid_momentum[3 * at + 2] += cz;
#pragma omp atomic
                    T->grid_mass[at] += cm;
                }
    }
#pragma omp parallel for schedule(static)
    for (node = 0; node < nodes; ++node) {
        int kk = (int)(node % M->dims[2]), jj = (int)((node / M->dims[2]) % M->dims[1]);
        int ii = (int)(node / ((int64_t)M->dims[1] * M->dims[2]));
        float m = bm_unfixed64(T->grid_mass[node], M->mass_shift);
        bm_v3 v = v3_zero();
        if (m > 0.0f)
            v = v3_div(v3(bm_unfixed64(T->grid_momentum[3 * node], M->momentum_shift),
                          bm_unfixed64(T->grid_momentum[3 * node + 1], M->momentum_shift),
                          bm_unfixed64(T->grid_momentum[3 * node + 2], M->momentum_shift)), m);
        if (ii < 1 || jj < 1 || kk < 1 || ii >= M->dims[0] - 1 || jj >= M->dims[1] - 1 || kk >= M->dims[2] - 1) v = v3_zero();
        st3(T->grid_v, node, v);
    }
#pragma omp parallel for schedule(static) reduction(+ : inversions)
    for (p = 0; p < n; ++p) {
        int base[3], i, j, k;
        bm_v3 fx, new_v = v3_zero(), s, x = ld3(T->x, p);
        bm_m33 new_C = m33_zero(), f, U, V;
        float w[3][3], smallest, reference_J;
        if (!mls_locate(M, x, base, &fx)) continue;
        mls_weights(fx, w);
        for (i = 0; i < 3; ++i)
            for (j = 0; j < 3; ++j)
                for (k = 0; k < 3; ++k) {
                    float weight = (w[i][0] * w[j][1]) * w[k][2];
                    bm_v3 dpos = v3_mul(v3_sub(v3((float)i, (float)j, (float)k), fx), M->dx);
                    int64_t at = ((int64_t)(base[0] + i) * M->dims[1] + (base[1] + j)) * M->dims[2] + (base[2] + k);
                    bm_v3 gv = ld3(T->grid_v, at);
                    new_v = v3_add(new_v, v3_mul(gv, weight));
                    new_C = m33_add(new_C, m33_scale(m33_outer(gv, dpos), (4.0f * weight) / (M->dx * M->dx)));
                }
        st3(T->v, p, new_v);
        st9(T->C, p, new_C);
        st3(T->x, p, v3_add(x, v3_mul(new_v, M->dt)));
        f = m33_mul(m33_add(m33_identity(), m33_scale(new_C, M->dt)), ld9(T->F, p));
        bm_svd3(f, &U, &s, &V);
        smallest = bm_minf(bm_minf(s.x, s.y), s.z);
        if (smallest <= 0.0f) inversions += 1;
        if (smallest < 0.05f) {
            s = v3(bm_maxf(s.x, 0.05f), bm_maxf(s.y, 0.05f), bm_maxf(s.z, 0.05f));
            f = m33_mul(m33_mul(U, m33_diag(s)), m33_transpose(V));
        }
        reference_J = T->damage_reference[p];
        if (M->plastic) {
            bm_v3 e = v3(bm_logf(s.x), bm_logf(s.y), bm_logf(s.z)), dev;
            float mean = ((e.x + e.y) + e.z) / 3.0f, norm, yield = T->yield_stress[p], limit;
            dev = v3_sub(e, v3(mean, mean, mean));
            norm = v3_len(dev);
            limit = yield / (2.0f * M->mu) * sqrtf(2.0f / 3.0f);
            if (norm > limit) {
                e = v3_sub(e, v3_mul(dev, 1.0f - limit / norm));
                s = v3(bm_expf(e.x), bm_expf(e.y), bm_expf(e.z));
                f = m33_mul(m33_mul(U, m33_diag(s)), m33_transpose(V));
                if (M->softening > 0.0f && reference_J > 0.0f) {
                    float softened = bm_maxf(0.0f, yield - M->softening * (norm - limit));
                    T->yield_stress[p] = softened;
                    if (softened <= 0.0f) T->damage[p] = 1.0f;
                }
            }
        }
        st9(T->F, p, f);
        if (reference_J > 0.0f) {
            float J = ((s.x * s.y) * s.z) / reference_J;
            if (J <= M->compressed || J >= M->stretched) T->damage[p] = 1.0f;
        }
    }
    T->inversions[0] += inversions;
}

ORC_API int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------- probes */

/* material.couple (material.py:155-193) on explicit per-node field runs. */
ORC_API void orc_couple_fields(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start,
                               int nodes, float* result) {
    int node, a, b;
    for (node = 0; node < nodes; ++node)
        for (a = node_start[node]; a < node_start[node + 1]; ++a) {
            float total = 0.0f, ma = mass[a];
            bm_v3 ex = v3_zero(), sa = ld3(state, a);
            if (ma <= 0.0f) continue;
            for (b = node_start[node]; b < node_start[node + 1]; ++b) {
                total = total + mass[b];
                if (b != a && compatible(codes[a], codes[b]))
                    ex = v3_add(ex, v3_sub(v3_mul(ld3(state, b), ma), v3_mul(sa, mass[b])));
            }
            st3(result, a, v3_add(sa, v3_div(ex, total)));
        }
}

/* material.g2p (material.py:343-381) on explicit slots/weights. */
ORC_API void orc_g2p(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                     const float* new_v, int n, float dt, float flip) {
    int p, a;
    for (p = 0; p < n; ++p) {
        bm_v3 pic = v3_zero(), dv = v3_zero();
        for (a = 0; a < 8; ++a) {
            int s = slots[8 * p + a];
            float w = weights[8 * p + a];
            bm_v3 nv = ld3(new_v, s);
            pic = v3_add(pic, v3_mul(nv, w));
            dv = v3_add(dv, v3_mul(v3_sub(nv, ld3(old_v, s)), w));
        }
        st3(v, p, v3_add(v3_mul(pic, 1.0f - flip), v3_mul(v3_add(ld3(v, p), dv), flip)));
        st3(x, p, v3_add(ld3(x, p), v3_mul(pic, dt)));
    }
}

/* Elementary functions of bm_scalar.h, for their own tests. */
ORC_API void orc_math_f(const float* x, int n, float* logf_out, float* expf_out) {
    int i;
    for (i = 0; i < n; ++i) { logf_out[i] = bm_logf(x[i]); expf_out[i] = bm_expf(x[i]); }
}
ORC_API void orc_math_d(const double* x, const double* y, int n, double* s, double* c, double* a) {
    int i;
    for (i = 0; i < n; ++i) { bm_sincos(x[i], &s[i], &c[i]); a[i] = bm_atan2(y[i], x[i]); }
}
ORC_API void orc_svd(const float* A, int n, float* U, float* sigma, float* V, float* R) {
    int i;
    for (i = 0; i < n; ++i) {
        bm_m33 u, v, r;
        bm_v3 s;
        bm_svd3(ld9(A, i), &u, &s, &v);
        r = bm_polar3(ld9(A, i));
        st9(U, i, u); st9(V, i, v); st3(sigma, i, s); st9(R, i, r);
    }
}
ORC_API void orc_fx_roundtrip(const float* x, int n, double* out) {
    int i;
    for (i = 0; i < n; ++i) out[i] = bm_fx_to_double(bm_fx_from_float(x[i]));
}

/* diagnostics.metrics (diagnostics.py:7-32) of n particles (AoS): out[0..2]
 * the exact 128-bit fixed-point sums of the kinetic, gravitational and
 * elastic energies (one rounding to double), out[3] max |v| (from 0),
 * out[4] max z (from -1e20), out[5] min det F (from 1e20).  The per-particle
 * terms use the kernel's operation order, so the sums are bit-exact with the
 * device's whatever the order of its atomic additions. */
ORC_API void orc_metrics(const float* x, const float* v, const float* F, const float* Fp, int n, float mass,
                         float volume, float mu, float lam, double* out) {
    bm_fx sum[3];
    float speed = 0.0f, top = -1.0e20f, low = 1.0e20f;
    int i, a, b, k;
    for (k = 0; k < 3; ++k) { sum[k].lo = 0u; sum[k].hi = 0u; }
    for (i = 0; i < n; ++i) {
        bm_v3 xp = ld3(x, i), vp = ld3(v, i), s;
        bm_m33 f = ld9(F, i), fe = m33_mul(f, m33_inverse(ld9(Fp, i))), u, w, strain;
        float energy = 0.0f, J, len, det;
        bm_svd3(fe, &u, &s, &w);
        strain = m33_sub(fe, m33_mul(u, m33_transpose(w)));
        for (a = 0; a < 3; ++a)
            for (b = 0; b < 3; ++b) energy = energy + mu * strain.m[a][b] * strain.m[a][b];
        J = m33_det(fe);
        energy = energy + 0.5f * lam * (J - 1.0f) * (J - 1.0f);
        sum[0] = bm_fx_add(sum[0], bm_fx_from_float(0.5f * mass * v3_dot(vp, vp)));
        sum[1] = bm_fx_add(sum[1], bm_fx_from_float(mass * 9.81f * xp.z));
        sum[2] = bm_fx_add(sum[2], bm_fx_from_float(volume * energy));
        len = v3_len(vp);
        det = m33_det(f);
        if (len > speed) speed = len;
        if (xp.z > top) top = xp.z;
        if (det < low) low = det;
    }
    for (k = 0; k < 3; ++k) out[k] = bm_fx_to_double(sum[k]);
    out[3] = speed;
    out[4] = top;
    out[5] = low;
}
