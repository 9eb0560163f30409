/*
 * Elementary vector, matrix, quaternion and transcendental operations with a
 * fixed IEEE operation sequence.
 *
 * Compiled as C11 (the CPU oracle, gcc -ffp-contract=off) and as CUDA C++
 * (the kernels, nvcc --fmad=false), so both evaluate the same sequence of
 * correctly rounded +, -, *, / and sqrt, and the material state they produce
 * is bit-identical.  No function here calls a vendor math routine other than
 * sqrt/sqrtf, fabs, floor, rint and ldexp, which are exact or correctly
 * rounded on both sides.
 *
 * Transcendentals are written from textbook series:
 *   bm_logf  - atanh series log(m) = 2 atanh((m-1)/(m+1)), m in [1/sqrt2, sqrt2]
 *   bm_expf  - Cody-Waite reduction x = k ln2 + r, Taylor series of exp(r)
 *   bm_sin/bm_cos (double) - reduction by pi/2 in three parts, Taylor series
 *   bm_atan2 (double) - octant reduction plus atan(z) Taylor series, |z| <= tan(pi/8)
 * Matrix decompositions:
 *   bm_svd3  - cyclic Jacobi eigen-decomposition of A^T A (Golub & Van Loan,
 *              Matrix Computations, Alg. 8.4.2 "sym.schur2") followed by a
 *              Givens QR of A V (the structure of McAdams et al. 2011, with
 *              exact rotations in place of their approximate ones)
 *   bm_polar3 - rotation factor of the polar decomposition by Newton's
 *              iteration X <- (X + X^-T) / 2 (Higham, Functions of Matrices,
 *              section 8.3)
 */
#ifndef BM_SCALAR_H
#define BM_SCALAR_H

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define BM_HD __host__ __device__ __forceinline__
#else
#define BM_HD static inline
#endif

typedef struct { float x, y, z; } bm_v3;
typedef struct { float m[3][3]; } bm_m33;
typedef struct { float x, y, z, w; } bm_q;
typedef struct { double x, y, z; } bm_v3d;
typedef struct { double x, y, z, w; } bm_qd;

/* ------------------------------------------------------------------ bits */

#ifdef ORC_REAL64
/* The oracle's float64 error-reference build (host C only): `float` is
 * defined as double there, orc_f32 is the real float32 type, and float bit
 * patterns (kept in int flag words) are those of the value rounded to float32. */
BM_HD uint32_t bm_f2u(double f) { union { orc_f32 f; uint32_t u; } c; c.f = (orc_f32)f; return c.u; }
BM_HD double bm_u2f(uint32_t u) { union { orc_f32 f; uint32_t u; } c; c.u = u; return (double)c.f; }
#else
BM_HD uint32_t bm_f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    union { float f; uint32_t u; } c; c.f = f; return c.u;
#endif
}
BM_HD float bm_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    union { float f; uint32_t u; } c; c.u = u; return c.f;
#endif
}
#endif
BM_HD uint64_t bm_d2u(double f) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(f);
#else
    union { double f; uint64_t u; } c; c.f = f; return c.u;
#endif
}
#ifdef ORC_REAL64
BM_HD int bm_isfinitef(double f) { return isfinite(f) != 0; }
#else
BM_HD int bm_isfinitef(float f) { return (bm_f2u(f) & 0x7f800000u) != 0x7f800000u; }
#endif
BM_HD int bm_isfinite(double f) { return (bm_d2u(f) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull; }
BM_HD float bm_minf(float a, float b) { return a < b ? a : b; }
BM_HD float bm_maxf(float a, float b) { return a > b ? a : b; }
BM_HD float bm_clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* ------------------------------------------------------------- float vec3 */

BM_HD bm_v3 v3(float x, float y, float z) { bm_v3 r; r.x = x; r.y = y; r.z = z; return r; }
BM_HD bm_v3 v3_zero(void) { return v3(0.0f, 0.0f, 0.0f); }
BM_HD bm_v3 v3_add(bm_v3 a, bm_v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
BM_HD bm_v3 v3_sub(bm_v3 a, bm_v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
BM_HD bm_v3 v3_neg(bm_v3 a) { return v3(-a.x, -a.y, -a.z); }
BM_HD bm_v3 v3_mul(bm_v3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
BM_HD bm_v3 v3_div(bm_v3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
BM_HD bm_v3 v3_cw(bm_v3 a, bm_v3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
BM_HD float v3_dot(bm_v3 a, bm_v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
BM_HD float v3_len_sq(bm_v3 a) { return v3_dot(a, a); }
BM_HD float v3_len(bm_v3 a) { return sqrtf(v3_dot(a, a)); }
BM_HD bm_v3 v3_cross(bm_v3 a, bm_v3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
BM_HD float v3_get(bm_v3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
BM_HD void v3_set(bm_v3* a, int i, float v) { if (i == 0) a->x = v; else if (i == 1) a->y = v; else a->z = v; }

/* ----------------------------------------------------------- float mat33 */

BM_HD bm_m33 m33_zero(void) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) r.m[i][j] = 0.0f;
    return r;
}
BM_HD bm_m33 m33_identity(void) { bm_m33 r = m33_zero(); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0f; return r; }
BM_HD bm_m33 m33_diag(bm_v3 d) { bm_m33 r = m33_zero(); r.m[0][0] = d.x; r.m[1][1] = d.y; r.m[2][2] = d.z; return r; }
BM_HD bm_m33 m33_add(bm_m33 a, bm_m33 b) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}
BM_HD bm_m33 m33_sub(bm_m33 a, bm_m33 b) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
    return r;
}
BM_HD bm_m33 m33_scale(bm_m33 a, float s) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s;
    return r;
}
BM_HD bm_m33 m33_transpose(bm_m33 a) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
BM_HD bm_m33 m33_mul(bm_m33 a, bm_m33 b) {
    bm_m33 r; int i, j;
    for (i = 0; i < 3; ++i)
        for (j = 0; j < 3; ++j) r.m[i][j] = (a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j]) + a.m[i][2] * b.m[2][j];
    return r;
}
BM_HD bm_v3 m33_mul_v3(bm_m33 a, bm_v3 v) {
    return v3((a.m[0][0] * v.x + a.m[0][1] * v.y) + a.m[0][2] * v.z,
              (a.m[1][0] * v.x + a.m[1][1] * v.y) + a.m[1][2] * v.z,
              (a.m[2][0] * v.x + a.m[2][1] * v.y) + a.m[2][2] * v.z);
}
BM_HD bm_m33 m33_outer(bm_v3 a, bm_v3 b) {
    bm_m33 r;
    r.m[0][0] = a.x * b.x; r.m[0][1] = a.x * b.y; r.m[0][2] = a.x * b.z;
    r.m[1][0] = a.y * b.x; r.m[1][1] = a.y * b.y; r.m[1][2] = a.y * b.z;
    r.m[2][0] = a.z * b.x; r.m[2][1] = a.z * b.y; r.m[2][2] = a.z * b.z;
    return r;
}
BM_HD float m33_det(bm_m33 a) {
    return (a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1])
            - a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]))
           + a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
/* Adjugate times 1/det; the zero matrix when det == 0. */
BM_HD bm_m33 m33_inverse(bm_m33 a) {
    float d = m33_det(a);
    bm_m33 b;
    float s;
    if (d == 0.0f) return m33_zero();
    s = 1.0f / d;
    b.m[0][0] = (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) * s;
    b.m[0][1] = (a.m[0][2] * a.m[2][1] - a.m[0][1] * a.m[2][2]) * s;
    b.m[0][2] = (a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]) * s;
    b.m[1][0] = (a.m[1][2] * a.m[2][0] - a.m[1][0] * a.m[2][2]) * s;
    b.m[1][1] = (a.m[0][0] * a.m[2][2] - a.m[0][2] * a.m[2][0]) * s;
    b.m[1][2] = (a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]) * s;
    b.m[2][0] = (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]) * s;
    b.m[2][1] = (a.m[0][1] * a.m[2][0] - a.m[0][0] * a.m[2][1]) * s;
    b.m[2][2] = (a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]) * s;
    return b;
}
BM_HD int m33_isfinite(bm_m33 a) {
    int i, j, ok = 1;
    for (i = 0; i < 3; ++i) for (j = 0; j < 3; ++j) ok &= bm_isfinitef(a.m[i][j]);
    return ok;
}

/* ------------------------------------------------------ float quaternion */

/* q v q^-1 for a unit quaternion (x, y, z, w). */
BM_HD bm_v3 q_rotate(bm_q q, bm_v3 v) {
    bm_v3 u = v3(q.x, q.y, q.z);
    float c = 2.0f * q.w * q.w - 1.0f;
    float d = 2.0f * v3_dot(u, v);
    return v3_add(v3_add(v3_mul(v, c), v3_mul(u, d)), v3_mul(v3_cross(u, v), 2.0f * q.w));
}
BM_HD bm_v3 q_rotate_inv(bm_q q, bm_v3 v) {
    bm_v3 u = v3(q.x, q.y, q.z);
    float c = 2.0f * q.w * q.w - 1.0f;
    float d = 2.0f * v3_dot(u, v);
    return v3_add(v3_sub(v3_mul(v, c), v3_mul(v3_cross(u, v), 2.0f * q.w)), v3_mul(u, d));
}

/* ---------------------------------------------------------- double vec3 */

BM_HD bm_v3d v3d(double x, double y, double z) { bm_v3d r; r.x = x; r.y = y; r.z = z; return r; }
BM_HD bm_v3d v3d_add(bm_v3d a, bm_v3d b) { return v3d(a.x + b.x, a.y + b.y, a.z + b.z); }
BM_HD bm_v3d v3d_sub(bm_v3d a, bm_v3d b) { return v3d(a.x - b.x, a.y - b.y, a.z - b.z); }
BM_HD bm_v3d v3d_neg(bm_v3d a) { return v3d(-a.x, -a.y, -a.z); }
BM_HD bm_v3d v3d_mul(bm_v3d a, double s) { return v3d(a.x * s, a.y * s, a.z * s); }
BM_HD bm_v3d v3d_div(bm_v3d a, double s) { return v3d(a.x / s, a.y / s, a.z / s); }
BM_HD bm_v3d v3d_cw(bm_v3d a, bm_v3d b) { return v3d(a.x * b.x, a.y * b.y, a.z * b.z); }
BM_HD double v3d_dot(bm_v3d a, bm_v3d b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
BM_HD double v3d_len(bm_v3d a) { return sqrt(v3d_dot(a, a)); }
BM_HD bm_v3d v3d_cross(bm_v3d a, bm_v3d b) {
    return v3d(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
BM_HD bm_v3d v3_to_d(bm_v3 a) { return v3d((double)a.x, (double)a.y, (double)a.z); }
BM_HD bm_v3 v3d_to_f(bm_v3d a) { return v3((float)a.x, (float)a.y, (float)a.z); }
BM_HD double v3d_get(bm_v3d a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

/* ---------------------------------------------------- double quaternion */

BM_HD bm_qd qd(double x, double y, double z, double w) { bm_qd r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
BM_HD bm_qd qd_mul(bm_qd a, bm_qd b) {
    return qd(a.w * b.x + b.w * a.x + (a.y * b.z - a.z * b.y),
              a.w * b.y + b.w * a.y + (a.z * b.x - a.x * b.z),
              a.w * b.z + b.w * a.z + (a.x * b.y - a.y * b.x),
              a.w * b.w - ((a.x * b.x + a.y * b.y) + a.z * b.z));
}
BM_HD bm_qd qd_normalize(bm_qd q) {
    double l = sqrt(((q.x * q.x + q.y * q.y) + q.z * q.z) + q.w * q.w);
    if (l > 0.0) return qd(q.x / l, q.y / l, q.z / l, q.w / l);
    return qd(0.0, 0.0, 0.0, 0.0);
}
BM_HD bm_qd qd_inverse(bm_qd q) { return qd(-q.x, -q.y, -q.z, q.w); }
BM_HD bm_v3d qd_rotate(bm_qd q, bm_v3d v) {
    bm_v3d u = v3d(q.x, q.y, q.z);
    double c = 2.0 * q.w * q.w - 1.0;
    double d = 2.0 * v3d_dot(u, v);
    return v3d_add(v3d_add(v3d_mul(v, c), v3d_mul(u, d)), v3d_mul(v3d_cross(u, v), 2.0 * q.w));
}
BM_HD bm_v3d qd_rotate_inv(bm_qd q, bm_v3d v) {
    bm_v3d u = v3d(q.x, q.y, q.z);
    double c = 2.0 * q.w * q.w - 1.0;
    double d = 2.0 * v3d_dot(u, v);
    return v3d_add(v3d_sub(v3d_mul(v, c), v3d_mul(v3d_cross(u, v), 2.0 * q.w)), v3d_mul(u, d));
}

/* ------------------------------------------------- float transcendentals */

#define BM_LN2_HI_F 0.693145751953125f
#define BM_LN2_LO_F 1.428606765330187e-06f

#ifdef ORC_REAL64
/* float64 error-reference build: the C library's double functions */
BM_HD double bm_logf(double x) { return log(x); }
BM_HD double bm_expf(double x) { return exp(x); }
BM_HD double bm_expm1f(double x) { return expm1(x); }
#else
BM_HD float bm_logf(float x) {
    uint32_t bits;
    int e;
    float m, u, u2, p, fe;
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (!bm_isfinitef(x)) return x;
    e = 0;
    if (x < 1.17549435e-38f) { x = x * 8388608.0f; e = -23; }
    bits = bm_f2u(x);
    e += (int)((bits >> 23) & 0xffu) - 127;
    m = bm_u2f((bits & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    u = (m - 1.0f) / (m + 1.0f);
    u2 = u * u;
    p = 0.0909090909f;                      /* 1/11 */
    p = 0.111111111f + u2 * p;              /* 1/9 */
    p = 0.142857143f + u2 * p;              /* 1/7 */
    p = 0.2f + u2 * p;                      /* 1/5 */
    p = 0.333333333f + u2 * p;              /* 1/3 */
    p = 1.0f + u2 * p;
    p = (2.0f * u) * p;
    fe = (float)e;
    return fe * BM_LN2_HI_F + (fe * BM_LN2_LO_F + p);
}

BM_HD float bm_expf(float x) {
    float k, r, p;
    if (x != x) return x;
    if (x > 88.72f) return INFINITY;
    if (x < -103.98f) return 0.0f;
    k = rintf(x * 1.44269504f);
    r = (x - k * BM_LN2_HI_F) - k * BM_LN2_LO_F;
    p = 1.98412698e-4f;                     /* 1/5040 */
    p = 1.38888889e-3f + r * p;             /* 1/720 */
    p = 8.33333333e-3f + r * p;             /* 1/120 */
    p = 4.16666667e-2f + r * p;             /* 1/24 */
    p = 0.166666667f + r * p;               /* 1/6 */
    p = 0.5f + r * p;
    p = 1.0f + r * p;
    p = 1.0f + r * p;
    return ldexpf(p, (int)k);
}

/* expm1 as the reference's material.expm1 (material.py:478-482), with bm_expf. */
BM_HD float bm_expm1f(float x) {
    if (fabsf(x) < 1.0e-3f) return x * (1.0f + 0.5f * x * (1.0f + x / 3.0f));
    return bm_expf(x) - 1.0f;
}
#endif

/* ------------------------------------------------ double transcendentals */

#define BM_PI 3.141592653589793
#define BM_PIO2_1 1.5707963267341256e+00   /* first 33 bits of pi/2 */
#define BM_PIO2_2 6.0771005065061922e-11   /* next 33 bits */
#define BM_PIO2_3 2.0222662487959506e-21   /* remainder */

BM_HD double bm_sin_poly(double r) {   /* Taylor series to r^19, |r| <= pi/4 */
    double r2 = r * r, p;
    p = -1.0 / 121645100408832000.0;                         /* -1/19! */
    p = 1.0 / 355687428096000.0 + r2 * p;                    /* 1/17! */
    p = -1.0 / 1307674368000.0 + r2 * p;                     /* -1/15! */
    p = 1.0 / 6227020800.0 + r2 * p;                         /* 1/13! */
    p = -1.0 / 39916800.0 + r2 * p;                          /* -1/11! */
    p = 1.0 / 362880.0 + r2 * p;                             /* 1/9! */
    p = -1.0 / 5040.0 + r2 * p;                              /* -1/7! */
    p = 1.0 / 120.0 + r2 * p;                                /* 1/5! */
    p = -1.0 / 6.0 + r2 * p;                                 /* -1/3! */
    return r + (r * r2) * p;
}
BM_HD double bm_cos_poly(double r) {   /* Taylor series to r^18, |r| <= pi/4 */
    double r2 = r * r, p;
    p = 1.0 / 6402373705728000.0;                            /* 1/18! */
    p = -1.0 / 20922789888000.0 + r2 * p;                    /* -1/16! */
    p = 1.0 / 87178291200.0 + r2 * p;                        /* 1/14! */
    p = -1.0 / 479001600.0 + r2 * p;                         /* -1/12! */
    p = 1.0 / 3628800.0 + r2 * p;                            /* 1/10! */
    p = -1.0 / 40320.0 + r2 * p;                             /* -1/8! */
    p = 1.0 / 720.0 + r2 * p;                                /* 1/6! */
    p = -1.0 / 24.0 + r2 * p;                                /* -1/4! */
    p = 0.5 + r2 * p;                                        /* 1/2! */
    return 1.0 - r2 * p;
}
/* sin and cos of x by reduction modulo pi/2 (accurate for |x| < 1e5). */
BM_HD void bm_sincos(double x, double* s, double* c) {
    double k = rint(x * (2.0 / BM_PI));
    double r = ((x - k * BM_PIO2_1) - k * BM_PIO2_2) - k * BM_PIO2_3;
    double sr = bm_sin_poly(r), cr = bm_cos_poly(r);
    long q = (long)k & 3;
    if (q == 0) { *s = sr; *c = cr; }
    else if (q == 1) { *s = cr; *c = -sr; }
    else if (q == 2) { *s = -sr; *c = -cr; }
    else { *s = -cr; *c = sr; }
}
BM_HD double bm_atan_small(double z) {   /* Taylor series to z^55, |z| <= tan(pi/8) */
    double z2 = z * z, p = 0.0;
    int k;
    for (k = 27; k >= 1; --k) p = ((k & 1) ? -1.0 : 1.0) / (double)(2 * k + 1) + z2 * p;
    return z + (z * z2) * p;
}
BM_HD double bm_atan2(double y, double x) {
    double ax = fabs(x), ay = fabs(y), t, a;
    if (ax == 0.0 && ay == 0.0) return (bm_d2u(x) >> 63) ? ((bm_d2u(y) >> 63) ? -BM_PI : BM_PI) : y;
    if (!bm_isfinite(ax) || !bm_isfinite(ay)) {
        if (ax != ax || ay != ay) return x + y;
        if (!bm_isfinite(ay) && !bm_isfinite(ax)) a = 0.25 * BM_PI;
        else if (!bm_isfinite(ay)) a = 0.5 * BM_PI;
        else a = 0.0;
    } else {
        t = ay <= ax ? ay / ax : ax / ay;
        if (t > 0.41421356237309503) a = 0.25 * BM_PI + bm_atan_small((t - 1.0) / (t + 1.0));
        else a = bm_atan_small(t);
        if (ay > ax) a = 0.5 * BM_PI - a;
    }
    if (x < 0.0) a = BM_PI - a;
    return (bm_d2u(y) >> 63) ? -a : a;
}
/* Rotation of angle about a unit axis (w last). */
BM_HD bm_qd qd_from_axis_angle(bm_v3d axis, double angle) {
    double s, c;
    bm_sincos(0.5 * angle, &s, &c);
    return qd(axis.x * s, axis.y * s, axis.z * s, c);
}

/* --------------------------------------------------------- 3x3 polar / SVD */

/* Rotation factor of the polar decomposition of a (det a > 0 assumed).
 * Newton's iteration X <- (X + X^-T)/2 from X = a converges quadratically:
 * an update of size d leaves an error of about d^2 / 2, so the iteration
 * stops after an update below 1e-4 (remaining error < 1e-8, below float
 * resolution), or after 16 iterations. */
BM_HD bm_m33 bm_polar3_inv(bm_m33 a, bm_m33* first_inv_t);
BM_HD bm_m33 bm_polar3(bm_m33 a) {
    bm_m33 unused;
    return bm_polar3_inv(a, &unused);
}
/* bm_polar3, also returning a^-T (the first iteration's inverse transpose). */
BM_HD bm_m33 bm_polar3_inv(bm_m33 a, bm_m33* first_inv_t) {
    bm_m33 x = a, y;
    int it, i, j;
    for (it = 0; it < 16; ++it) {
        bm_m33 inv_t = m33_transpose(m33_inverse(x));
        if (it == 0) *first_inv_t = inv_t;
        float change = 0.0f;
        for (i = 0; i < 3; ++i)
            for (j = 0; j < 3; ++j) {
                y.m[i][j] = 0.5f * (x.m[i][j] + inv_t.m[i][j]);
                change = bm_maxf(change, fabsf(y.m[i][j] - x.m[i][j]));
            }
        x = y;
        if (!(change > 1.0e-4f)) break;
    }
    return x;
}

/* One Jacobi rotation zeroing s[p][q] of the symmetric s, accumulated in v. */
BM_HD void bm_jacobi_rotate(bm_m33* s, bm_m33* v, int p, int q) {
    float apq = s->m[p][q], app, aqq, tau, t, c, sn, arp, arq;
    int r;
    if (apq == 0.0f) return;
    app = s->m[p][p];
    aqq = s->m[q][q];
    tau = (aqq - app) / (2.0f * apq);
    if (tau >= 0.0f) t = 1.0f / (tau + sqrtf(1.0f + tau * tau));
    else t = -1.0f / (-tau + sqrtf(1.0f + tau * tau));
    c = 1.0f / sqrtf(1.0f + t * t);
    sn = t * c;
    s->m[p][p] = app - t * apq;
    s->m[q][q] = aqq + t * apq;
    s->m[p][q] = s->m[q][p] = 0.0f;
    for (r = 0; r < 3; ++r) {
        if (r == p || r == q) continue;
        arp = s->m[r][p];
        arq = s->m[r][q];
        s->m[r][p] = s->m[p][r] = c * arp - sn * arq;
        s->m[r][q] = s->m[q][r] = sn * arp + c * arq;
    }
    for (r = 0; r < 3; ++r) {
        arp = v->m[r][p];
        arq = v->m[r][q];
        v->m[r][p] = c * arp - sn * arq;
        v->m[r][q] = sn * arp + c * arq;
    }
}

/* Givens rotation of rows p, q of b zeroing b[q][col]; accumulated into the columns of u. */
BM_HD void bm_givens_rows(bm_m33* b, bm_m33* u, int p, int q, int col) {
    float x = b->m[p][col], y = b->m[q][col], r, c, s, bp, bq;
    int j;
    r = sqrtf(x * x + y * y);
    if (r == 0.0f) return;
    c = x / r;
    s = y / r;
    for (j = 0; j < 3; ++j) {
        bp = b->m[p][j];
        bq = b->m[q][j];
        b->m[p][j] = c * bp + s * bq;
        b->m[q][j] = -s * bp + c * bq;
    }
    b->m[q][col] = 0.0f;
    for (j = 0; j < 3; ++j) {
        bp = u->m[j][p];
        bq = u->m[j][q];
        u->m[j][p] = c * bp + s * bq;
        u->m[j][q] = -s * bp + c * bq;
    }
}

BM_HD void bm_swap_cols(bm_m33* a, int i, int j, int negate) {
    int r;
    for (r = 0; r < 3; ++r) {
        float t = a->m[r][i];
        a->m[r][i] = negate ? -a->m[r][j] : a->m[r][j];
        a->m[r][j] = t;
    }
}

/* a = u diag(sigma) v^T with u, v rotations, sigma[0] >= sigma[1] >= |sigma[2]|;
 * sigma[2] < 0 when det a < 0. */
BM_HD void bm_svd3(bm_m33 a, bm_m33* u_out, bm_v3* sigma, bm_m33* v_out) {
    bm_m33 s = m33_mul(m33_transpose(a), a);
    bm_m33 v = m33_identity(), b, u = m33_identity();
    float n0, n1, n2;
    int sweep;
    for (sweep = 0; sweep < 5; ++sweep) {
        bm_jacobi_rotate(&s, &v, 0, 1);
        bm_jacobi_rotate(&s, &v, 0, 2);
        bm_jacobi_rotate(&s, &v, 1, 2);
    }
    b = m33_mul(a, v);
    /* Order the columns by decreasing norm; a swap negates one column so det v stays +1. */
    n0 = (b.m[0][0] * b.m[0][0] + b.m[1][0] * b.m[1][0]) + b.m[2][0] * b.m[2][0];
    n1 = (b.m[0][1] * b.m[0][1] + b.m[1][1] * b.m[1][1]) + b.m[2][1] * b.m[2][1];
    n2 = (b.m[0][2] * b.m[0][2] + b.m[1][2] * b.m[1][2]) + b.m[2][2] * b.m[2][2];
    if (n0 < n1) { float t = n0; n0 = n1; n1 = t; bm_swap_cols(&b, 0, 1, 1); bm_swap_cols(&v, 0, 1, 1); }
    if (n0 < n2) { float t = n0; n0 = n2; n2 = t; bm_swap_cols(&b, 0, 2, 1); bm_swap_cols(&v, 0, 2, 1); }
    if (n1 < n2) { float t = n1; n1 = n2; n2 = t; bm_swap_cols(&b, 1, 2, 1); bm_swap_cols(&v, 1, 2, 1); }
    /* QR of b by Givens rotations: b = u r, r upper triangular (diagonal up to rounding). */
    bm_givens_rows(&b, &u, 0, 1, 0);
    bm_givens_rows(&b, &u, 0, 2, 0);
    bm_givens_rows(&b, &u, 1, 2, 1);
    *u_out = u;
    *v_out = v;
    *sigma = v3(b.m[0][0], b.m[1][1], b.m[2][2]);
}

/* ------------------------------------------------- exact 128-bit accumulator */

/* Fixed point with 2^-96 resolution in two 64-bit words (two's complement).
 * Sums of these are exact and independent of the order of addition, which
 * makes impulse, torque and work accumulation deterministic on the device. */
typedef struct { uint64_t lo; uint64_t hi; } bm_fx;
#define BM_FX_SHIFT 96

BM_HD bm_fx bm_fx_neg(bm_fx a) {
    bm_fx r;
    r.lo = ~a.lo + 1u;
    r.hi = ~a.hi + (r.lo == 0u ? 1u : 0u);
    return r;
}
BM_HD bm_fx bm_fx_add(bm_fx a, bm_fx b) {
    bm_fx r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1u : 0u);
    return r;
}
/* Exact for |f| >= 2^-73; smaller magnitudes round half away from zero; |f| < 2^31 required. */
/* f * 2^k rounded to the nearest integer (halves away from zero) as int64,
 * from the float's bits so that CPU and GPU agree; |result| saturates at
 * 2^62 and non-finite f gives 0.  Sums of such values are exact and do not
 * depend on their order. */
#ifdef ORC_REAL64
/* float64 error-reference build: f * 2^k rounded to the nearest integer,
 * f * 2^-96 split exactly into the two 64-bit words (truncated below 2^-96). */
BM_HD int64_t bm_fixed64(double f, int k) {
    if (!isfinite(f)) return 0;
    return (int64_t)llround(ldexp(f, k));
}
BM_HD double bm_unfixed64(int64_t v, int k) { return ldexp((double)v, -k); }
BM_HD bm_fx bm_fx_from_float(double f) {
    bm_fx r;
    double top, rest;
    r.lo = 0u; r.hi = 0u;
    if (!isfinite(f) || fabs(f) >= 2147483648.0) return r;
    top = floor(ldexp(f, 32));           /* the integer part of f * 2^32 */
    rest = ldexp(f, 32) - top;           /* in [0, 1), exact */
    r.hi = (uint64_t)(int64_t)top;
    r.lo = (uint64_t)ldexp(rest, 64);
    return r;
}
#else
BM_HD int64_t bm_fixed64(float f, int k) {
    uint32_t bits = bm_f2u(f);
    int exponent = (int)((bits >> 23) & 0xffu), shift;
    uint64_t mant = bits & 0x007fffffu, mag;
    if (exponent == 0xff) return 0;
    if (exponent == 0) exponent = 1; else mant |= 0x00800000u;
    if (mant == 0u) return 0;
    /* |f| = mant * 2^(exponent - 150) */
    shift = exponent - 150 + k;
    if (shift >= 0) {
        mag = shift > 38 ? ((uint64_t)1 << 62) : (mant << shift);
    } else {
        int down = -shift;
        if (down > 25) return 0;
        mag = (mant + ((uint64_t)1 << (down - 1))) >> down;
    }
    return (bits >> 31) ? -(int64_t)mag : (int64_t)mag;
}
/* The float nearest to v * 2^-k (one rounding; 2^-k is applied exactly). */
BM_HD float bm_unfixed64(int64_t v, int k) { return (float)v * bm_u2f((uint32_t)(127 - k) << 23); }

BM_HD bm_fx bm_fx_from_float(float f) {
    uint32_t bits = bm_f2u(f);
    int exponent = (int)((bits >> 23) & 0xffu);
    uint64_t mant = bits & 0x007fffffu;
    int shift;
    bm_fx r;
    r.lo = 0u; r.hi = 0u;
    if (exponent == 0xff) return r;
    if (exponent == 0) exponent = 1; else mant |= 0x00800000u;
    /* f = mant * 2^(exponent - 150); fixed = mant * 2^(exponent - 150 + 96) */
    shift = exponent - 54;
    if (mant == 0u) return r;
    if (shift >= 0) {
        if (shift >= 104) return r;  /* out of range: treated as zero */
        if (shift >= 64) { r.hi = mant << (shift - 64); r.lo = 0u; }
        else if (shift == 0) { r.lo = mant; r.hi = 0u; }
        else { r.lo = mant << shift; r.hi = mant >> (64 - shift); }
    } else {
        int down = -shift;
        if (down > 25) return r;
        r.lo = (mant + ((uint64_t)1 << (down - 1))) >> down;
        r.hi = 0u;
    }
    if (bits >> 31) r = bm_fx_neg(r);
    return r;
}
#endif
BM_HD double bm_fx_to_double(bm_fx a) {
    int negative = (a.hi >> 63) != 0u;
    double v;
    if (negative) a = bm_fx_neg(a);
    v = (double)a.hi * 2.3283064365386963e-10 + (double)a.lo * 1.2621774483536189e-29; /* 2^-32, 2^-96 */
    return negative ? -v : v;
}

#endif /* BM_SCALAR_H */
