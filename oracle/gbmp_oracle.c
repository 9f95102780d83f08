/*
 * gbmp_oracle.c -- CPU restatement of the reference hot path.
 *
 * TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py, never by the product library.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp (see oracle/build.py).  Contraction
 * is off so that every fused multiply-add below is the explicit fmaf() written
 * here; the CUDA kernels use the same explicit __fmaf_rn chain, so the FP32
 * results differ only where cosf/sinf differ in the last bit.
 */
#include "gbmp_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int32_t or_num_threads(void)
{
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Forward kinematics.                                                       */
/* Follows the generated kernel cudampl/CUDAMPLib/include/spaces/            */
/* KernelGenerator.h:222-406 (multiply4x4 :257-280, make_rotation_axis_angle */
/* :293-325, revolute :328-340, prismatic :343-361, unrolled chain :369-400) */
/* and the table-driven twin cudampl/CUDAMPLib/src/states/                   */
/* SingleArmStates.cu:178-221.  Poses are 3x4 affine blocks of a row-major   */
/* 4x4; the last row is always (0,0,0,1) (KernelGenerator.h:275).           */
/* ------------------------------------------------------------------------- */

/* C = A * B for row-major 4x4 with implicit last row (0 0 0 1). */
static void mul_f32(const float *A, const float *B, float *C)
{
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 4; ++c) {
            float acc = A[r * 4 + 0] * B[0 * 4 + c];
            acc = fmaf(A[r * 4 + 1], B[1 * 4 + c], acc);
            acc = fmaf(A[r * 4 + 2], B[2 * 4 + c], acc);
            if (c == 3) acc = acc + A[r * 4 + 3];
            C[r * 4 + c] = acc;
        }
    }
    C[12] = 0.f; C[13] = 0.f; C[14] = 0.f; C[15] = 1.f;
}

static void mul_f64(const double *A, const double *B, double *C)
{
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) {
            double acc = A[r * 4 + 0] * B[c] + A[r * 4 + 1] * B[4 + c] + A[r * 4 + 2] * B[8 + c];
            if (c == 3) acc += A[r * 4 + 3];
            C[r * 4 + c] = acc;
        }
    C[12] = 0.; C[13] = 0.; C[14] = 0.; C[15] = 1.;
}

/* Normalised axis, KernelGenerator.h:295-304 (length threshold 1e-12). */
static void unit_axis_f32(const float *a, float *n)
{
    float len = sqrtf(fmaf(a[2], a[2], fmaf(a[1], a[1], a[0] * a[0])));
    float valid = (len >= 1e-12f) ? 1.f : 0.f;
    float inv = 1.f / fmaxf(len, 1e-12f);
    n[0] = a[0] * inv * valid;
    n[1] = a[1] * inv * valid;
    n[2] = a[2] * inv * valid;
    n[3] = valid;
}

/* Rodrigues rotation, KernelGenerator.h:305-325. */
static void rot_f32(const float *n, float angle, float *R)
{
    float nx = n[0], ny = n[1], nz = n[2], valid = n[3];
    float c = cosf(angle), s = sinf(angle), oc = 1.f - c;
    float r0 = fmaf(nx * nx, oc, c);
    float r1 = fmaf(nx * ny, oc, -(nz * s));
    float r2 = fmaf(nx * nz, oc, ny * s);
    float r4 = fmaf(ny * nx, oc, nz * s);
    float r5 = fmaf(ny * ny, oc, c);
    float r6 = fmaf(ny * nz, oc, -(nx * s));
    float r8 = fmaf(nz * nx, oc, -(ny * s));
    float r9 = fmaf(nz * ny, oc, nx * s);
    float r10 = fmaf(nz * nz, oc, c);
    float iv = 1.f - valid;
    R[0] = r0 * valid + iv; R[1] = r1 * valid; R[2] = r2 * valid; R[3] = 0.f;
    R[4] = r4 * valid; R[5] = r5 * valid + iv; R[6] = r6 * valid; R[7] = 0.f;
    R[8] = r8 * valid; R[9] = r9 * valid; R[10] = r10 * valid + iv; R[11] = 0.f;
    R[12] = 0.f; R[13] = 0.f; R[14] = 0.f; R[15] = 1.f;
}

static void rot_f64(const float *a, double angle, double *R)
{
    double x = a[0], y = a[1], z = a[2];
    double len = sqrt(x * x + y * y + z * z);
    double valid = len >= 1e-12 ? 1. : 0.;
    double inv = 1. / fmax(len, 1e-12);
    double nx = x * inv * valid, ny = y * inv * valid, nz = z * inv * valid;
    double c = cos(angle), s = sin(angle), oc = 1. - c, iv = 1. - valid;
    R[0] = (c + nx * nx * oc) * valid + iv; R[1] = (nx * ny * oc - nz * s) * valid;
    R[2] = (nx * nz * oc + ny * s) * valid; R[3] = 0.;
    R[4] = (ny * nx * oc + nz * s) * valid; R[5] = (c + ny * ny * oc) * valid + iv;
    R[6] = (ny * nz * oc - nx * s) * valid; R[7] = 0.;
    R[8] = (nz * nx * oc - ny * s) * valid; R[9] = (nz * ny * oc + nx * s) * valid;
    R[10] = (c + nz * nz * oc) * valid + iv; R[11] = 0.;
    R[12] = 0.; R[13] = 0.; R[14] = 0.; R[15] = 1.;
}

static void fk_one_f32(const or_robot *r, const float *q, float *P)
{
    static const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    memcpy(P, I, sizeof I);                       /* link 0 = identity (:365-368) */
    float tmp[16], M[16], n[4];
    for (int i = 1; i < r->L; ++i) {
        const float *par = P + 16 * r->parent[i];
        const float *jp = r->pose + 16 * i;
        float *out = P + 16 * i;
        switch (r->type[i]) {
        case OR_REVOLUTE:                         /* parent * (pose * R(axis, q)): same product as
                                                     (parent * pose) * R up to rounding */
            unit_axis_f32(r->axis + 3 * i, n);
            rot_f32(n, q[i], M);
            mul_f32(jp, M, tmp);
            mul_f32(par, tmp, out);
            break;
        case OR_PRISMATIC: {                      /* parent * (pose * T(axis q)) */
            const float *a = r->axis + 3 * i;
            float T[16] = {1, 0, 0, a[0] * q[i], 0, 1, 0, a[1] * q[i], 0, 0, 1, a[2] * q[i], 0, 0, 0, 1};
            mul_f32(jp, T, tmp);
            mul_f32(par, tmp, out);
            break;
        }
        case OR_FIXED:
            mul_f32(par, jp, out);
            break;
        default:                                  /* unsupported type: pose left unwritten in the
                                                     reference (:397); identity here */
            memcpy(out, I, sizeof I);
            break;
        }
    }
}

static void fk_one_f64(const or_robot *r, const double *q, double *P)
{
    for (int k = 0; k < 16; ++k) P[k] = (k % 5 == 0) ? 1. : 0.;
    double tmp[16], M[16], jp[16];
    for (int i = 1; i < r->L; ++i) {
        const double *par = P + 16 * r->parent[i];
        double *out = P + 16 * i;
        for (int k = 0; k < 16; ++k) jp[k] = r->pose[16 * i + k];
        if (r->type[i] == OR_REVOLUTE) {
            rot_f64(r->axis + 3 * i, q[i], M);
            mul_f64(par, jp, tmp);
            mul_f64(tmp, M, out);
        } else if (r->type[i] == OR_PRISMATIC) {
            const float *a = r->axis + 3 * i;
            double T[16] = {1, 0, 0, a[0] * q[i], 0, 1, 0, a[1] * q[i], 0, 0, 1, a[2] * q[i], 0, 0, 0, 1};
            mul_f64(jp, T, tmp);
            mul_f64(par, tmp, out);
        } else if (r->type[i] == OR_FIXED) {
            mul_f64(par, jp, out);
        } else {
            for (int k = 0; k < 16; ++k) out[k] = (k % 5 == 0) ? 1. : 0.;
        }
    }
}

void or_fk_f32(const or_robot *r, const float *q, int64_t n, float *poses)
{
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) fk_one_f32(r, q + s * r->L, poses + s * r->L * 16);
}

void or_fk_f64(const or_robot *r, const double *q, int64_t n, double *poses)
{
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) fk_one_f64(r, q + s * r->L, poses + s * r->L * 16);
}

/* Sphere centres in the base frame, cudampl/CUDAMPLib/src/states/SingleArmStates.cu:340-393. */
static void centers_one_f32(const or_robot *r, const float *P, float *C)
{
    for (int i = 0; i < r->S; ++i) {
        const float *T = P + 16 * r->sph_link[i];
        float sx = r->sph_pos[3 * i], sy = r->sph_pos[3 * i + 1], sz = r->sph_pos[3 * i + 2];
        for (int row = 0; row < 3; ++row)
            C[3 * i + row] = fmaf(T[4 * row + 2], sz, fmaf(T[4 * row + 1], sy, T[4 * row] * sx)) + T[4 * row + 3];
    }
}

void or_sphere_centers_f32(const or_robot *r, const float *poses, int64_t n, float *centers)
{
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) centers_one_f32(r, poses + s * r->L * 16, centers + s * r->S * 3);
}

void or_sphere_centers_f64(const or_robot *r, const double *poses, int64_t n, double *centers)
{
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < n; ++s) {
        const double *P = poses + s * r->L * 16;
        double *C = centers + s * r->S * 3;
        for (int i = 0; i < r->S; ++i) {
            const double *T = P + 16 * r->sph_link[i];
            double sx = r->sph_pos[3 * i], sy = r->sph_pos[3 * i + 1], sz = r->sph_pos[3 * i + 2];
            for (int row = 0; row < 3; ++row)
                C[3 * i + row] = T[4 * row] * sx + T[4 * row + 1] * sy + T[4 * row + 2] * sz + T[4 * row + 3];
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Collision model.                                                          */
/* ------------------------------------------------------------------------- */

/* Self-collision pair list, cudampl/CUDAMPLib/src/constraints/
 * SelfCollisionConstraint.cu:28-38: i < j, different links, link pair enabled;
 * threshold stored squared.  enables == NULL means every link pair enabled. */
int32_t or_self_pairs(const or_robot *r, const uint8_t *enables, int32_t *pairs, float *thr_sq, int32_t cap)
{
    int32_t k = 0;
    for (int i = 0; i < r->S; ++i)
        for (int j = i + 1; j < r->S; ++j) {
            int li = r->sph_link[i], lj = r->sph_link[j];
            if (li == lj) continue;
            if (enables && !enables[li * r->L + lj]) continue;
            if (k < cap) {
                pairs[2 * k] = i;
                pairs[2 * k + 1] = j;
                float s = r->sph_r[i] + r->sph_r[j];
                thr_sq[k] = s * s;
            }
            ++k;
        }
    return k;
}

/* Inverse pose [R^T | -R^T t] of an obstacle, cudampl/CUDAMPLib/src/constraints/
 * EnvConstraintCuboid.cu:13-34 and EnvConstraintCylinder.cu:17-45. */
void or_inverse_pose(const float *pos, const float *rot, float *inv)
{
    float t00 = rot[0], t01 = rot[3], t02 = rot[6];
    float t10 = rot[1], t11 = rot[4], t12 = rot[7];
    float t20 = rot[2], t21 = rot[5], t22 = rot[8];
    inv[0] = t00; inv[1] = t01; inv[2] = t02;
    inv[4] = t10; inv[5] = t11; inv[6] = t12;
    inv[8] = t20; inv[9] = t21; inv[10] = t22;
    inv[3] = -(t00 * pos[0] + t01 * pos[1] + t02 * pos[2]);
    inv[7] = -(t10 * pos[0] + t11 * pos[1] + t12 * pos[2]);
    inv[11] = -(t20 * pos[0] + t21 * pos[1] + t22 * pos[2]);
}

static inline void xform34(const float *M, float x, float y, float z, float *o)
{
    o[0] = fmaf(M[2], z, fmaf(M[1], y, M[0] * x)) + M[3];
    o[1] = fmaf(M[6], z, fmaf(M[5], y, M[4] * x)) + M[7];
    o[2] = fmaf(M[10], z, fmaf(M[9], y, M[8] * x)) + M[11];
}

/* Self cost, SelfCollisionConstraint.cu:80-112. */
static float self_cost(const float *C, int32_t np, const int32_t *pairs, const float *thr_sq)
{
    float sum = 0.f;
    for (int k = 0; k < np; ++k) {
        const float *a = C + 3 * pairs[2 * k], *b = C + 3 * pairs[2 * k + 1];
        float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        if (d2 < thr_sq[k]) sum += sqrtf(thr_sq[k]) - sqrtf(d2);
    }
    return sum;
}

/* Environment spheres, cudampl/CUDAMPLib/src/constraints/EnvConstraintSphere.cu:57-96. */
static float env_sphere_cost(const or_robot *r, const or_env *e, const float *C)
{
    float sum = 0.f;
    for (int i = 0; i < r->S; ++i) {
        float rs = r->sph_r[i];
        for (int o = 0; o < e->ns; ++o) {
            const float *b = e->sph + 4 * o;
            float dx = C[3 * i] - b[0], dy = C[3 * i + 1] - b[1], dz = C[3 * i + 2] - b[2];
            float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            float rr = rs + b[3];
            if (d2 < rr * rr) sum += fmaxf(0.f, rr - sqrtf(d2));
        }
    }
    return sum;
}

/* Cuboids, cudampl/CUDAMPLib/src/constraints/EnvConstraintCuboid.cu:105-159. */
static float env_cuboid_cost(const or_robot *r, const or_env *e, const float *C)
{
    float sum = 0.f;
    for (int i = 0; i < r->S; ++i) {
        float rs = r->sph_r[i];
        for (int o = 0; o < e->nb; ++o) {
            float l[3];
            xform34(e->box_inv + 12 * o, C[3 * i], C[3 * i + 1], C[3 * i + 2], l);
            const float *mn = e->box_min + 3 * o, *mx = e->box_max + 3 * o;
            float dx = l[0] - fminf(fmaxf(l[0], mn[0]), mx[0]);
            float dy = l[1] - fminf(fmaxf(l[1], mn[1]), mx[1]);
            float dz = l[2] - fminf(fmaxf(l[2], mn[2]), mx[2]);
            float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            if (d2 < rs * rs) sum += rs - sqrtf(d2);
        }
    }
    return sum;
}

/* Cylinders along local z, cudampl/CUDAMPLib/src/constraints/EnvConstraintCylinder.cu:130-180. */
static float env_cylinder_cost(const or_robot *r, const or_env *e, const float *C)
{
    float sum = 0.f;
    for (int i = 0; i < r->S; ++i) {
        float rs = r->sph_r[i];
        for (int o = 0; o < e->nc; ++o) {
            float l[3];
            xform34(e->cyl_inv + 12 * o, C[3 * i], C[3 * i + 1], C[3 * i + 2], l);
            float dxy = sqrtf(fmaf(l[1], l[1], l[0] * l[0]));
            float dx = dxy - e->cyl_r[o];
            float dz = fabsf(l[2]) - e->cyl_h[o] * 0.5f;
            float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
            float outside = sqrtf(fmaf(oz, oz, ox * ox));
            float inside = fminf(fmaxf(dx, dz), 0.f);
            float pen = rs - (outside + inside);
            sum += pen > 0.f ? pen : 0.f;
        }
    }
    return sum;
}

/* checkStates: per-constraint cost in SoA slots, total = sum of slots
 * (cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu:1572-1602,
 *  cudampl/CUDAMPLib/src/base/States.cu:5-21).  Feasible <=> total == 0. */
void or_check_states(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                     const float *thr_sq, const float *q, int64_t n, float *costs, float *total,
                     int32_t nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
    {
        float *P = (float *)malloc(sizeof(float) * 16 * r->L);
        float *C = (float *)malloc(sizeof(float) * 3 * (r->S + 1));
#pragma omp for schedule(dynamic, 16)
        for (int64_t s = 0; s < n; ++s) {
            fk_one_f32(r, q + s * r->L, P);
            centers_one_f32(r, P, C);
            float c0 = self_cost(C, npairs, pairs, thr_sq);
            float c1 = env_sphere_cost(r, e, C);
            float c2 = env_cuboid_cost(r, e, C);
            float c3 = env_cylinder_cost(r, e, C);
            if (costs) {
                costs[0 * n + s] = c0; costs[1 * n + s] = c1;
                costs[2 * n + s] = c2; costs[3 * n + s] = c3;
            }
            if (total) total[s] = ((c0 + c1) + c2) + c3;
        }
        free(P);
        free(C);
    }
}

/* Signed clearance (FP64): min over every checked pair of distance minus radii;
 * negative = penetration.  Used to exclude states within a band of the contact
 * surface from verdict comparisons. */
void or_clearance_f64(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                      const double *q, int64_t n, double *clearance, int32_t nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
    {
        double *P = (double *)malloc(sizeof(double) * 16 * r->L);
        double *C = (double *)malloc(sizeof(double) * 3 * (r->S + 1));
#pragma omp for schedule(dynamic, 16)
        for (int64_t s = 0; s < n; ++s) {
            fk_one_f64(r, q + s * r->L, P);
            for (int i = 0; i < r->S; ++i) {
                const double *T = P + 16 * r->sph_link[i];
                double sx = r->sph_pos[3 * i], sy = r->sph_pos[3 * i + 1], sz = r->sph_pos[3 * i + 2];
                for (int row = 0; row < 3; ++row)
                    C[3 * i + row] = T[4 * row] * sx + T[4 * row + 1] * sy + T[4 * row + 2] * sz + T[4 * row + 3];
            }
            double best = DBL_MAX;
            for (int k = 0; k < npairs; ++k) {
                const double *a = C + 3 * pairs[2 * k], *b = C + 3 * pairs[2 * k + 1];
                double d = sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
                double c = d - ((double)r->sph_r[pairs[2 * k]] + (double)r->sph_r[pairs[2 * k + 1]]);
                if (c < best) best = c;
            }
            for (int i = 0; i < r->S; ++i) {
                double x = C[3 * i], y = C[3 * i + 1], z = C[3 * i + 2], rs = r->sph_r[i];
                for (int o = 0; o < e->ns; ++o) {
                    const float *b = e->sph + 4 * o;
                    double d = sqrt((x - b[0]) * (x - b[0]) + (y - b[1]) * (y - b[1]) + (z - b[2]) * (z - b[2]));
                    double c = d - (rs + (double)b[3]);
                    if (c < best) best = c;
                }
                for (int o = 0; o < e->nb; ++o) {
                    const float *M = e->box_inv + 12 * o;
                    double l[3];
                    for (int row = 0; row < 3; ++row)
                        l[row] = M[4 * row] * x + M[4 * row + 1] * y + M[4 * row + 2] * z + M[4 * row + 3];
                    const float *mn = e->box_min + 3 * o, *mx = e->box_max + 3 * o;
                    double out2 = 0., depth = DBL_MAX;
                    int inside = 1;
                    for (int a = 0; a < 3; ++a) {
                        double lo = mn[a], hi = mx[a];
                        if (l[a] < lo) { out2 += (lo - l[a]) * (lo - l[a]); inside = 0; }
                        else if (l[a] > hi) { out2 += (l[a] - hi) * (l[a] - hi); inside = 0; }
                        else { double dd = fmin(l[a] - lo, hi - l[a]); if (dd < depth) depth = dd; }
                    }
                    double sd = inside ? -depth : sqrt(out2);
                    double c = sd - rs;
                    if (c < best) best = c;
                }
                for (int o = 0; o < e->nc; ++o) {
                    const float *M = e->cyl_inv + 12 * o;
                    double l[3];
                    for (int row = 0; row < 3; ++row)
                        l[row] = M[4 * row] * x + M[4 * row + 1] * y + M[4 * row + 2] * z + M[4 * row + 3];
                    double dx = sqrt(l[0] * l[0] + l[1] * l[1]) - e->cyl_r[o];
                    double dz = fabs(l[2]) - 0.5 * e->cyl_h[o];
                    double ox = dx > 0 ? dx : 0, oz = dz > 0 ? dz : 0;
                    double sdf = sqrt(ox * ox + oz * oz) + fmin(fmax(dx, dz), 0.);
                    double c = sdf - rs;
                    if (c < best) best = c;
                }
            }
            clearance[s] = best;
        }
        free(P);
        free(C);
    }
}

/* ------------------------------------------------------------------------- */
/* Edges.                                                                    */
/* Step rule of the generated get_step kernel, KernelGenerator.h:408-465:    */
/*   d = ||to - from||_2 over all J entries, n = (int)(d / res) + 1,         */
/*   dir = (to - from) / n.                                                  */
/* Interpolation, KernelGenerator.h:467-522: state k = from + dir * k for    */
/* k < n, then state n-1 := to.  The generated code is compiled by NVRTC     */
/* with FMA contraction on (cudampl/CUDAMPLib/include/NvrtcUtil.h:85-94), so */
/* the sum of squares and the interpolation are fused multiply-adds.         */
/* The L-infinity rule (max |to - from| <= res per step) keeps the same n/dir */
/* structure with d = max_j |to_j - from_j|.                                 */
/* ------------------------------------------------------------------------- */

int32_t or_edge_steps(const float *from, const float *to, int32_t J, float res, int32_t rule,
                      float *dir, float *length)
{
    float d2 = 0.f, dinf = 0.f;
    for (int j = 0; j < J; ++j) {
        float d = from[j] - to[j];
        d2 = fmaf(d, d, d2);
        float a = fabsf(d);
        dinf = a > dinf ? a : dinf;
    }
    float d = sqrtf(d2);
    if (length) *length = d;
    if (rule == OR_STEP_COUNT) {   /* pRRTC.cu:430-440: granularity equal steps */
        int32_t g = (int32_t)res;
        if (dir)
            for (int j = 0; j < J; ++j) dir[j] = (to[j] - from[j]) / (float)g;
        return g + 1;
    }
    float metric = (rule == OR_STEP_LINF) ? dinf : d;
    int32_t n = (int32_t)(metric / res) + 1;
    if (dir)
        for (int j = 0; j < J; ++j) dir[j] = (to[j] - from[j]) / (float)n;
    return n;
}

void or_edge_state(const float *from, const float *to, const float *dir, int32_t J, int32_t n,
                   int32_t k, float *out)
{
    if (k == n - 1) {
        memcpy(out, to, sizeof(float) * J);
        return;
    }
    for (int j = 0; j < J; ++j) out[j] = fmaf(dir[j], (float)k, from[j]);
}

/* checkMotions (SingleArmSpace.cu:628-848): every interpolated state is checked;
 * an edge is feasible iff the sum of its states' total costs is 0 (:603-626);
 * its cost is d (:831).  first_hit (not produced by the reference) is the lowest
 * state index with non-zero total cost, -1 if none.  early_exit=0 evaluates every
 * state of every edge like the reference; early_exit=1 stops an edge at its first
 * hit (same outputs). */
void or_check_motions(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                      const float *thr_sq, const float *from, const float *to, int64_t E,
                      float res, int32_t rule, int32_t early_exit, uint8_t *ok, int32_t *first_hit,
                      int32_t *num_steps, float *length, int32_t nthreads)
{
    const int J = r->L;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel num_threads(nthreads)
    {
        float *P = (float *)malloc(sizeof(float) * 16 * J);
        float *C = (float *)malloc(sizeof(float) * 3 * (r->S + 1));
        float *dir = (float *)malloc(sizeof(float) * J);
        float *st = (float *)malloc(sizeof(float) * J);
#pragma omp for schedule(dynamic, 1)
        for (int64_t k = 0; k < E; ++k) {
            const float *f = from + k * J, *t = to + k * J;
            float len;
            int32_t n = or_edge_steps(f, t, J, res, rule, dir, &len);
            int32_t hit = -1;
            float sum = 0.f;
            for (int32_t s = 0; s < n; ++s) {
                or_edge_state(f, t, dir, J, n, s, st);
                fk_one_f32(r, st, P);
                centers_one_f32(r, P, C);
                float tot = self_cost(C, npairs, pairs, thr_sq);
                tot += env_sphere_cost(r, e, C);
                tot += env_cuboid_cost(r, e, C);
                tot += env_cylinder_cost(r, e, C);
                sum += tot;
                if (tot != 0.f && hit < 0) {
                    hit = s;
                    if (early_exit) break;
                }
            }
            if (ok) ok[k] = (sum == 0.f);
            if (first_hit) first_hit[k] = hit;
            if (num_steps) num_steps[k] = n;
            if (length) length[k] = len;
        }
        free(P);
        free(C);
        free(dir);
        free(st);
    }
}

/* ------------------------------------------------------------------------- */
/* State-manager kernels.                                                    */
/* ------------------------------------------------------------------------- */

/* Nearest neighbour among candidate indices, distance over active joints only,
 * cudampl/CUDAMPLib/src/states/SingleArmStates.cu:1265-1336.  The squared
 * distance is accumulated in joint order with fused multiply-adds (the reference's
 * contracted loop, :1285-1300) and compared without the monotone sqrt.  Exact ties
 * resolve to the lowest candidate position. */
void or_nearest(const float *tree, int64_t M, int32_t J, const uint8_t *active,
                const int32_t *cand, int64_t ncand, const float *queries, int64_t Q,
                int32_t *out, int32_t nthreads)
{
    (void)M;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t q = 0; q < Q; ++q) {
        const float *x = queries + q * J;
        float best = INFINITY;
        int32_t bi = -1;
        for (int64_t c = 0; c < ncand; ++c) {
            int64_t idx = cand ? cand[c] : c;
            const float *y = tree + idx * J;
            float s = 0.f;
            for (int j = 0; j < J; ++j)
                if (!active || active[j]) {
                    float d = x[j] - y[j];
                    s = fmaf(d, d, s);
                }
            if (s < best) {
                best = s;
                bi = (int32_t)idx;
            }
        }
        out[q] = bi;
    }
}

/* Philox4x32-10 (Salmon et al., SC'11), the counter-based generator behind the
 * product's sampler: sample k, joint j uses counter (offset + k, j), key seed, and
 * the 24 high bits of output word 0.  Value = fma(u, upper - lower, lower). */
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

void or_sample(const float *lower, const float *upper, const uint8_t *active, const float *defv,
               int32_t J, uint64_t seed, uint64_t offset, int64_t n, float *q)
{
    for (int64_t k = 0; k < n; ++k)
        for (int j = 0; j < J; ++j) {
            if (!active[j]) { q[k * J + j] = defv[j]; continue; }
            uint64_t ctr = offset + (uint64_t)k;
            uint32_t c[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)j, 0u};
            philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
            float u = (float)(c[0] >> 8) * (1.0f / 16777216.0f);
            q[k * J + j] = fmaf(u, upper[j] - lower[j], lower[j]);
        }
}

/* Steer towards a sample, limiting the step to max_distance
 * (SingleArmStates.cu:1488-1522, SingleArmSpace.cu:219-249). */
void or_steer(const float *from, float *to, int64_t n, int32_t J, float max_distance)
{
    for (int64_t k = 0; k < n; ++k) {
        const float *f = from + k * J;
        float *t = to + k * J;
        float s = 0.f;
        for (int j = 0; j < J; ++j) {
            float d = f[j] - t[j];
            s = fmaf(d, d, s);
        }
        float d = sqrtf(s);
        if (d > max_distance) {
            float sc = max_distance / d;
            for (int j = 0; j < J; ++j) t[j] = fmaf(sc, t[j] - f[j], f[j]);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Sequential RRT-Connect with the planner's primitives (the loop of          */
/* cudampl/CPRRTC/src/RobotSolver.cu:562-796 and pRRTC/src/planning/          */
/* pRRTC.cu:340-601 run by one thread): Philox sample (counter iteration,      */
/* lane 0), nearest node by squared active-joint distance, steer to `range`,   */
/* edge validation with the checkMotions step rule (state 0 skipped unless     */
/* n == 1), append, greedy connect in ceil(d / range) steps.  The smaller tree */
/* grows.  Returns 1 when solved; the path runs from start to goal.            */
/* ------------------------------------------------------------------------- */
static int state_collides(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs,
                          const float *thr, const float *q, float *P, float *C)
{
    fk_one_f32(r, q, P);
    centers_one_f32(r, P, C);
    if (self_cost(C, np, pairs, thr) != 0.f) return 1;
    if (env_sphere_cost(r, e, C) != 0.f) return 1;
    if (env_cuboid_cost(r, e, C) != 0.f) return 1;
    return env_cylinder_cost(r, e, C) != 0.f;
}

static int edge_free(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                     const float *a, const float *b, float res, int32_t rule, float *P, float *C, float *dir,
                     float *st)
{
    const int J = r->L;
    int32_t n = or_edge_steps(a, b, J, res, rule, dir, NULL);
    for (int32_t k = (n == 1 ? 0 : 1); k < n; ++k) {
        or_edge_state(a, b, dir, J, n, k, st);
        if (state_collides(r, e, np, pairs, thr, st, P, C)) return 0;
    }
    return 1;
}

/* A tree edge old -> new checked in the direction it takes in a returned path (which runs
 * from the start root to the goal root), so that a path check meets exactly these states:
 * start tree (tr 0) edges from the old node, state 0 skipped (edge_free); goal tree edges
 * from the new node towards the old one, the last state (the old node) skipped, and with
 * one state the new node itself.  Mirrors block_edge_free's old_first rule. */
static int edge_free_tree(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                          const float *old, const float *nw, int tr, float res, int32_t rule, float *P, float *C,
                          float *dir, float *st)
{
    if (tr == 0) return edge_free(r, e, np, pairs, thr, old, nw, res, rule, P, C, dir, st);
    const int J = r->L;
    int32_t n = or_edge_steps(nw, old, J, res, rule, dir, NULL);
    if (n == 1) return !state_collides(r, e, np, pairs, thr, nw, P, C);
    for (int32_t k = 0; k < n - 1; ++k) {
        or_edge_state(nw, old, dir, J, n, k, st);
        if (state_collides(r, e, np, pairs, thr, st, P, C)) return 0;
    }
    return 1;
}

static int32_t tree_nearest(const float *nodes, int32_t size, int32_t J, const uint8_t *active, const float *q)
{
    float best = INFINITY;
    int32_t bi = -1;
    for (int32_t i = 0; i < size; ++i) {
        float s = 0.f;
        for (int j = 0; j < J; ++j)
            if (active[j]) {
                float d = q[j] - nodes[(int64_t)i * J + j];
                s = fmaf(d, d, s);
            }
        if (s < best) { best = s; bi = i; }
    }
    return bi;
}

static float active_dist(const float *a, const float *b, int32_t J, const uint8_t *active)
{
    float s = 0.f;
    for (int j = 0; j < J; ++j)
        if (active[j]) { float d = b[j] - a[j]; s = fmaf(d, d, s); }
    return sqrtf(s);
}

int32_t or_rrtc(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                const float *start, const float *goal, const uint8_t *active, const float *lower,
                const float *upper, const float *defv, float range, float res, int32_t rule, uint64_t seed,
                int32_t max_nodes, int32_t max_iters, float *path, int32_t path_cap, int32_t *path_len,
                float *cost, int32_t *iters, int32_t *tree_sizes)
{
    const int J = r->L;
    float *nodes[2];
    int32_t *par[2], size[2] = {1, 1};
    for (int t = 0; t < 2; ++t) {
        nodes[t] = (float *)malloc(sizeof(float) * (size_t)max_nodes * J);
        par[t] = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_nodes);
    }
    memcpy(nodes[0], start, sizeof(float) * J);
    memcpy(nodes[1], goal, sizeof(float) * J);
    par[0][0] = 0; par[1][0] = 0;
    float *P = (float *)malloc(sizeof(float) * 16 * J), *C = (float *)malloc(sizeof(float) * 3 * (r->S + 1));
    float *dir = (float *)malloc(sizeof(float) * J), *st = (float *)malloc(sizeof(float) * J);
    float *qs = (float *)malloc(sizeof(float) * J), *qn = (float *)malloc(sizeof(float) * J);
    float *qa = (float *)malloc(sizeof(float) * J), *qb = (float *)malloc(sizeof(float) * J);
    float *qc = (float *)malloc(sizeof(float) * J);
    int32_t solved = 0, ca = -1, cb = -1, tr_win = 0, it;
    for (it = 0; it < max_iters && !solved; ++it) {
        int tr = size[0] <= size[1] ? 0 : 1, ot = 1 - tr;
        for (int j = 0; j < J; ++j) {
            if (!active[j]) { qs[j] = defv[j]; continue; }
            uint64_t ctr = (uint64_t)it;
            uint32_t c4[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)j, 0u};
            philox(c4, (uint32_t)seed, (uint32_t)(seed >> 32));
            float u = (float)(c4[0] >> 8) * (1.0f / 16777216.0f);
            qs[j] = fmaf(u, upper[j] - lower[j], lower[j]);
        }
        int32_t nn = tree_nearest(nodes[tr], size[tr], J, active, qs);
        memcpy(qn, nodes[tr] + (int64_t)nn * J, sizeof(float) * J);
        float d = active_dist(qn, qs, J, active);
        if (d > range) {
            float sc = range / d;
            for (int j = 0; j < J; ++j) if (active[j]) qs[j] = fmaf(sc, qs[j] - qn[j], qn[j]);
        }
        if (!edge_free_tree(r, e, np, pairs, thr, qn, qs, tr, res, rule, P, C, dir, st)) continue;
        if (size[tr] >= max_nodes) break;
        int32_t cur = size[tr]++;
        memcpy(nodes[tr] + (int64_t)cur * J, qs, sizeof(float) * J);
        par[tr][cur] = nn;
        int32_t tgt = tree_nearest(nodes[ot], size[ot], J, active, qs);
        memcpy(qb, nodes[ot] + (int64_t)tgt * J, sizeof(float) * J);
        memcpy(qa, qs, sizeof(float) * J);
        float dd = active_dist(qs, qb, J, active);
        int32_t n_ext = (int32_t)ceilf(dd / range);
        if (n_ext < 1) n_ext = 1;
        int ok = 1;
        for (int32_t k = 1; k <= n_ext && ok; ++k) {
            for (int j = 0; j < J; ++j) qc[j] = (k == n_ext) ? qb[j] : fmaf((qb[j] - qs[j]) / (float)n_ext, (float)k, qs[j]);
            if (!edge_free_tree(r, e, np, pairs, thr, qa, qc, tr, res, rule, P, C, dir, st)) { ok = 0; break; }
            if (k < n_ext) {
                if (size[tr] >= max_nodes) { ok = 0; break; }
                int32_t nx = size[tr]++;
                memcpy(nodes[tr] + (int64_t)nx * J, qc, sizeof(float) * J);
                par[tr][nx] = cur;
                cur = nx;
                memcpy(qa, qc, sizeof(float) * J);
            }
        }
        if (ok) { solved = 1; ca = cur; cb = tgt; tr_win = tr; }
    }
    *iters = it;
    tree_sizes[0] = size[0];
    tree_sizes[1] = size[1];
    *path_len = 0;
    *cost = 0.f;
    if (solved) {
        int32_t n0 = tr_win == 0 ? ca : cb, n1 = tr_win == 0 ? cb : ca;
        int32_t l0 = 0, l1 = 0;
        for (int32_t i = n0;; i = par[0][i]) { ++l0; if (i == 0) break; }
        for (int32_t i = n1;; i = par[1][i]) { ++l1; if (i == 0) break; }
        if (l0 + l1 <= path_cap) {
            int32_t k = l0 - 1;
            for (int32_t i = n0;; i = par[0][i], --k) { memcpy(path + (int64_t)k * J, nodes[0] + (int64_t)i * J, sizeof(float) * J); if (i == 0) break; }
            k = l0;
            for (int32_t i = n1;; i = par[1][i], ++k) { memcpy(path + (int64_t)k * J, nodes[1] + (int64_t)i * J, sizeof(float) * J); if (i == 0) break; }
            *path_len = l0 + l1;
            double c = 0.0;
            for (int32_t q = 1; q < l0 + l1; ++q) c += active_dist(path + (int64_t)(q - 1) * J, path + (int64_t)q * J, J, active);
            *cost = (float)c;
        }
    }
    for (int t = 0; t < 2; ++t) { free(nodes[t]); free(par[t]); }
    free(P); free(C); free(dir); free(st); free(qs); free(qn); free(qa); free(qb); free(qc);
    return solved;
}

/* ------------------------------------------------------------------------------------
 * Lane-parallel RRT-Connect in synchronous rounds.
 *
 * The device planner runs `lanes` extension lanes at once (one CUDA block each, as the
 * reference's CPRRTC kernel runs one block per sampled motion, RobotSolver.cu:562-796,
 * and pRRTC one block per new configuration, pRRTC.cu:340-601).  This restatement runs
 * the same per-lane rule in rounds: in round `it` every lane
 *   1. picks its tree by the balance rule from the tree sizes at the start of the round
 *      (pRRTC.cu:348-371; see or_balance_tree),
 *   2. draws its sample with Philox counter (lane << 32 | it), key seed,
 *   3. extends from the nearest node of that tree (as the round began) by at most
 *      `range`, checking the edge with the planner's step rule (state 0 skipped);
 * the new nodes are appended in lane order; then every lane that extended
 *   4. connects: finds the nearest node of the other tree (as it stands after the
 *      round's extensions) and walks towards it in ceil(d / range) checked steps
 *      (RobotSolver.cu:686-794, pRRTC.cu:478-551), keeping every checked step;
 * the connection steps are appended in lane order.  Of the lanes that reach the other
 * tree in a round, the one that needed the fewest steps wins (ties: lowest lane),
 * standing for the device's first connection to finish.  Lanes within a round are
 * independent, so they run in parallel (OpenMP); the commits keep lane order, so the
 * result does not depend on the thread count.
 * ---------------------------------------------------------------------------------- */

/* Lane hash in [0, 1) (Fibonacci hashing of the lane index): the share of lanes below h
 * stands for the reference's block index over the block count. */
static float lane_hash(int32_t lane)
{
    return (float)(((uint32_t)lane * 2654435769u) >> 8) * (1.0f / 16777216.0f);
}

/* Tree grown by a lane (pRRTC.cu:348-371).  balance: 0 none (half the lanes each), 1
 * proportional while the trees are within 1.5 x lanes nodes of each other and the
 * smaller one (by tree_ratio) otherwise, 2 VAMP (swap trees while the size difference
 * relative to the grown tree is below tree_ratio), 3 proportional at every size (the
 * device planner's default).  cur: the lane's tree in its previous round, -1 in its
 * first. */
int32_t or_balance_tree(int32_t balance, float tree_ratio, int32_t lanes, int32_t n0, int32_t n1, float h,
                        int32_t cur)
{
    if (cur < 0 || balance == 0) return h < 0.5f ? 0 : 1;
    if (balance == 3) return h < 1.f - (float)n0 / (float)(n0 + n1 > 1 ? n0 + n1 : 1) ? 0 : 1;
    if (balance == 2) {
        int32_t nt = cur == 0 ? n0 : n1, no = cur == 0 ? n1 : n0;
        float ratio = (float)abs(nt - no) / (float)(nt > 1 ? nt : 1);
        return ratio < tree_ratio ? 1 - cur : cur;
    }
    float ratio = (float)n0 / (float)(n0 + n1 > 1 ? n0 + n1 : 1);
    if ((float)abs(n0 - n1) < 1.5f * (float)lanes) return h < 1.f - ratio ? 0 : 1;
    return ratio < tree_ratio ? 0 : 1;
}

typedef struct lane_out {
    int32_t tr, nn, ext;          /* tree, nearest node, 1 if the extension is free */
    int32_t tgt, n_ext, n_chain;  /* connect target, steps needed, steps kept       */
    int32_t connected;
    int32_t chain_cap;
    float *qs;                    /* [J] new node                                   */
    float *chain;                 /* [chain_cap * J] connection steps               */
} lane_out;

int32_t or_rrtc_lanes(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                      const float *start, const float *goal, const uint8_t *active, const float *lower,
                      const float *upper, const float *defv, float range, float res, int32_t rule, uint64_t seed,
                      int32_t lanes, int32_t balance, float tree_ratio, int32_t max_nodes, int32_t max_iters,
                      float *path, int32_t path_cap, int32_t *path_len, float *cost, int32_t *iters,
                      int32_t *tree_sizes, int32_t nthreads)
{
    const int J = r->L;
    float *nodes[2];
    int32_t *par[2], size[2] = {1, 1};
    for (int t = 0; t < 2; ++t) {
        nodes[t] = (float *)malloc(sizeof(float) * (size_t)max_nodes * J);
        par[t] = (int32_t *)malloc(sizeof(int32_t) * (size_t)max_nodes);
    }
    memcpy(nodes[0], start, sizeof(float) * J);
    memcpy(nodes[1], goal, sizeof(float) * J);
    par[0][0] = 0; par[1][0] = 0;
    lane_out *lo = (lane_out *)calloc((size_t)lanes, sizeof(lane_out));
    int32_t *cur_tree = (int32_t *)malloc(sizeof(int32_t) * (size_t)lanes);
    int32_t *ext_idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)lanes);
    for (int32_t l = 0; l < lanes; ++l) {
        cur_tree[l] = -1;
        lo[l].qs = (float *)malloc(sizeof(float) * J);
        lo[l].chain_cap = 16;
        lo[l].chain = (float *)malloc(sizeof(float) * 16 * J);
    }
    int nth = nthreads > 0 ? nthreads : or_num_threads();
    int32_t solved = 0, ca = -1, cb = -1, tr_win = 0, it, full = 0;
    for (it = 0; it < max_iters && !solved && !full; ++it) {
        const int32_t n0 = size[0], n1 = size[1];
        /* 1-3: extensions against the trees as the round began */
        #pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
        for (int32_t l = 0; l < lanes; ++l) {
            lane_out *o = &lo[l];
            float P[16 * 64], C[3 * 257], dir[64], st[64], qn[64];
            float *P_ = J <= 64 && r->S <= 256 ? P : (float *)malloc(sizeof(float) * 16 * J);
            float *C_ = J <= 64 && r->S <= 256 ? C : (float *)malloc(sizeof(float) * 3 * (r->S + 1));
            o->tr = or_balance_tree(balance, tree_ratio, lanes, n0, n1, lane_hash(l), cur_tree[l]);
            cur_tree[l] = o->tr;
            o->ext = 0;
            o->connected = 0;
            o->n_chain = 0;
            const int32_t tr = o->tr, sz = tr == 0 ? n0 : n1;
            const uint64_t ctr = ((uint64_t)(uint32_t)l << 32) | (uint32_t)it;
            for (int j = 0; j < J; ++j) {
                if (!active[j]) { o->qs[j] = defv[j]; continue; }
                uint32_t c4[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)j, 0u};
                philox(c4, (uint32_t)seed, (uint32_t)(seed >> 32));
                float u = (float)(c4[0] >> 8) * (1.0f / 16777216.0f);
                o->qs[j] = fmaf(u, upper[j] - lower[j], lower[j]);
            }
            o->nn = tree_nearest(nodes[tr], sz, J, active, o->qs);
            memcpy(qn, nodes[tr] + (int64_t)o->nn * J, sizeof(float) * J);
            float d = active_dist(qn, o->qs, J, active);
            if (d > range) {
                float sc = range / d;
                for (int j = 0; j < J; ++j) if (active[j]) o->qs[j] = fmaf(sc, o->qs[j] - qn[j], qn[j]);
            }
            o->ext = edge_free_tree(r, e, np, pairs, thr, qn, o->qs, tr, res, rule, P_, C_, dir, st);
            if (P_ != P) free(P_);
            if (C_ != C) free(C_);
        }
        for (int32_t l = 0; l < lanes; ++l) {
            ext_idx[l] = -1;
            if (!lo[l].ext) continue;
            const int32_t tr = lo[l].tr;
            if (size[tr] >= max_nodes) { full = 1; lo[l].ext = 0; continue; }
            ext_idx[l] = size[tr]++;
            memcpy(nodes[tr] + (int64_t)ext_idx[l] * J, lo[l].qs, sizeof(float) * J);
            par[tr][ext_idx[l]] = lo[l].nn;
        }
        const int32_t s0 = size[0], s1 = size[1];
        /* 4: connections against the trees after the round's extensions */
        #pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
        for (int32_t l = 0; l < lanes; ++l) {
            lane_out *o = &lo[l];
            if (!o->ext) continue;
            float P[16 * 64], C[3 * 257], dir[64], st[64], qa[64], qb[64], qc[64];
            float *P_ = J <= 64 && r->S <= 256 ? P : (float *)malloc(sizeof(float) * 16 * J);
            float *C_ = J <= 64 && r->S <= 256 ? C : (float *)malloc(sizeof(float) * 3 * (r->S + 1));
            const int32_t ot = 1 - o->tr, szo = ot == 0 ? s0 : s1;
            o->tgt = tree_nearest(nodes[ot], szo, J, active, o->qs);
            memcpy(qb, nodes[ot] + (int64_t)o->tgt * J, sizeof(float) * J);
            memcpy(qa, o->qs, sizeof(float) * J);
            float dd = active_dist(o->qs, qb, J, active);
            int32_t n_ext = (int32_t)ceilf(dd / range);
            if (n_ext < 1) n_ext = 1;
            o->n_ext = n_ext;
            int ok = 1;
            for (int32_t k = 1; k <= n_ext && ok; ++k) {
                for (int j = 0; j < J; ++j)
                    qc[j] = (k == n_ext) ? qb[j] : fmaf((qb[j] - o->qs[j]) / (float)n_ext, (float)k, o->qs[j]);
                if (!edge_free_tree(r, e, np, pairs, thr, qa, qc, o->tr, res, rule, P_, C_, dir, st)) { ok = 0; break; }
                if (k < n_ext) {
                    if (o->n_chain == o->chain_cap) {
                        o->chain_cap *= 2;
                        o->chain = (float *)realloc(o->chain, sizeof(float) * (size_t)o->chain_cap * J);
                    }
                    memcpy(o->chain + (int64_t)o->n_chain * J, qc, sizeof(float) * J);
                    ++o->n_chain;
                    memcpy(qa, qc, sizeof(float) * J);
                }
            }
            o->connected = ok;
            if (P_ != P) free(P_);
            if (C_ != C) free(C_);
        }
        int32_t win = -1;
        for (int32_t l = 0; l < lanes; ++l) {
            lane_out *o = &lo[l];
            if (!o->ext) continue;
            const int32_t tr = o->tr;
            int32_t cur = ext_idx[l], kept = 1;
            for (int32_t k = 0; k < o->n_chain; ++k) {
                if (size[tr] >= max_nodes) { full = 1; kept = 0; break; }
                int32_t nx = size[tr]++;
                memcpy(nodes[tr] + (int64_t)nx * J, o->chain + (int64_t)k * J, sizeof(float) * J);
                par[tr][nx] = cur;
                cur = nx;
            }
            if (o->connected && kept && (win < 0 || o->n_ext < lo[win].n_ext)) {
                win = l;
                ca = cur;
            }
        }
        if (win >= 0) {
            solved = 1;
            tr_win = lo[win].tr;
            cb = lo[win].tgt;
        }
    }
    *iters = it;
    tree_sizes[0] = size[0];
    tree_sizes[1] = size[1];
    *path_len = 0;
    *cost = 0.f;
    if (solved) {
        int32_t na = tr_win == 0 ? ca : cb, nb = tr_win == 0 ? cb : ca;
        int32_t l0 = 0, l1 = 0;
        for (int32_t i = na;; i = par[0][i]) { ++l0; if (par[0][i] == i) break; }
        for (int32_t i = nb;; i = par[1][i]) { ++l1; if (par[1][i] == i) break; }
        if (l0 + l1 <= path_cap) {
            int32_t k = l0 - 1;
            for (int32_t i = na;; i = par[0][i], --k) {
                memcpy(path + (int64_t)k * J, nodes[0] + (int64_t)i * J, sizeof(float) * J);
                if (par[0][i] == i) break;
            }
            k = l0;
            for (int32_t i = nb;; i = par[1][i], ++k) {
                memcpy(path + (int64_t)k * J, nodes[1] + (int64_t)i * J, sizeof(float) * J);
                if (par[1][i] == i) break;
            }
            *path_len = l0 + l1;
            double c = 0.0;
            for (int32_t q = 1; q < l0 + l1; ++q) c += active_dist(path + (int64_t)(q - 1) * J, path + (int64_t)q * J, J, active);
            *cost = (float)c;
        }
    }
    for (int32_t l = 0; l < lanes; ++l) { free(lo[l].qs); free(lo[l].chain); }
    free(lo); free(cur_tree); free(ext_idx);
    for (int t = 0; t < 2; ++t) { free(nodes[t]); free(par[t]); }
    return solved;
}

/* ------------------------------------------------------------------------------------
 * Constraint projection.
 * ---------------------------------------------------------------------------------- */

/* 4x4 product with an implicit last row (0 0 0 1), TaskSpaceConstraint.cu:47-63. */
static void pr_mul44(const float *A, const float *B, float *C)
{
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c)
            C[4 * r + c] = A[4 * r] * B[c] + A[4 * r + 1] * B[4 + c] + A[4 * r + 2] * B[8 + c] + A[4 * r + 3] * B[12 + c];
    C[12] = 0.f; C[13] = 0.f; C[14] = 0.f; C[15] = 1.f;
}

/* Task-frame pose and its x, y, z, roll, pitch, yaw (TaskSpaceConstraint.cu:185-206). */
static void pr_task_frame(const float *poses, int task_link, const float *offset, float *P, float v[6])
{
    pr_mul44(poses + 16 * task_link, offset, P);
    v[0] = P[3]; v[1] = P[7]; v[2] = P[11];
    v[4] = asinf(-P[8]);
    v[3] = atan2f(P[9], P[10]);
    v[5] = atan2f(P[4], P[0]);
}

static float pr_dead(float diff, float tol)
{
    return copysignf(fmaxf(fabsf(diff) - tol, 0.0f), diff);
}

/* Gradient of the task-space constraint for one state (TaskSpaceConstraint.cu:167-396). */
static void pr_task_grad(const or_robot *r, const uint8_t *active, const or_projection *p, const float *poses,
                         float *grad)
{
    const int L = r->L;
    float P[16], v[6], err[6];
    pr_task_frame(poses, p->task_link, p->offset, P, v);
    /* reference - current, dead-banded; order roll pitch yaw x y z (angular rows first) */
    err[0] = pr_dead(p->reference[3] - v[3], p->tolerance[3]);
    err[1] = pr_dead(p->reference[4] - v[4], p->tolerance[4]);
    err[2] = pr_dead(p->reference[5] - v[5], p->tolerance[5]);
    err[3] = pr_dead(p->reference[0] - v[0], p->tolerance[0]);
    err[4] = pr_dead(p->reference[1] - v[1], p->tolerance[1]);
    err[5] = pr_dead(p->reference[2] - v[2], p->tolerance[2]);
    float J[64 * 6];
    for (int j = 0; j < L; ++j) {
        float *c = J + 6 * j;
        for (int k = 0; k < 6; ++k) c[k] = 0.f;
        if (j > p->task_link) continue;
        const float *T = poses + 16 * j;
        const float *a = r->axis + 3 * j;
        const float w0 = T[0] * a[0] + T[1] * a[1] + T[2] * a[2];
        const float w1 = T[4] * a[0] + T[5] * a[1] + T[6] * a[2];
        const float w2 = T[8] * a[0] + T[9] * a[1] + T[10] * a[2];
        if (r->type[j] == OR_REVOLUTE) {
            const float d0 = v[0] - T[3], d1 = v[1] - T[7], d2 = v[2] - T[11];
            c[0] = w0; c[1] = w1; c[2] = w2;
            c[3] = w1 * d2 - w2 * d1;
            c[4] = w2 * d0 - w0 * d2;
            c[5] = w0 * d1 - w1 * d0;
        } else if (r->type[j] == OR_PRISMATIC) {
            c[3] = w0; c[4] = w1; c[5] = w2;
        }
    }
    /* A = J_a J_a^T + 1e-4 I, Gauss-Jordan without pivoting (TaskSpaceConstraint.cu:290-350) */
    float aug[6][12];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            float sum = 0.0f;
            for (int k = 0; k < L; ++k)
                if (active[k]) sum += J[6 * k + i] * J[6 * k + j];
            aug[i][j] = (i == j) ? sum + 1e-4f : sum;
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 6; j < 12; ++j) aug[i][j] = (j - 6 == i) ? 1.0f : 0.0f;
    int invertible = 1;
    for (int i = 0; i < 6 && invertible; ++i) {
        const float pivot = aug[i][i];
        if (fabsf(pivot) < 1e-8f) { invertible = 0; break; }
        for (int j = 0; j < 12; ++j) aug[i][j] /= pivot;
        for (int k = 0; k < 6; ++k)
            if (k != i) {
                const float f = aug[k][i];
                for (int j = 0; j < 12; ++j) aug[k][j] -= f * aug[i][j];
            }
    }
    for (int j = 0; j < L; ++j) {
        grad[j] = 0.f;
        if (!active[j] || !invertible) continue;
        float g = 0.0f;
        for (int i = 0; i < 6; ++i) {
            float s = 0.0f;
            for (int m = 0; m < 6; ++m) s += J[6 * j + m] * aug[m][6 + i];
            g += s * err[i];
        }
        grad[j] = g;
    }
}

static float pr_task_cost(const or_projection *p, const float *poses)
{
    float P[16], v[6], c = 0.f;
    pr_task_frame(poses, p->task_link, p->offset, P, v);
    for (int k = 0; k < 6; ++k) {
        const float d = v[k] - p->reference[k], t = p->tolerance[k];
        c += fmaxf(d * d - t * t, 0.f);
    }
    c = sqrtf(c);
    return c < 1e-4f ? 0.0f : c;
}

static float pr_bound_cost(int L, const uint8_t *active, const float *lower, const float *upper, const float *q)
{
    float c = 0.0f;
    for (int j = 0; j < L; ++j) {
        if (!active[j]) continue;
        if (q[j] < lower[j]) c += (lower[j] - q[j]) * (lower[j] - q[j]);
        else if (q[j] > upper[j]) c += (q[j] - upper[j]) * (q[j] - upper[j]);
    }
    return c < 1e-4f ? 0.0f : sqrtf(c);
}

void or_project(const or_robot *r, const uint8_t *active, const float *lower, const float *upper,
                const or_projection *p, float *q, int64_t n, float *task_cost, float *bound_cost,
                int32_t nthreads)
{
    const int L = r->L;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int64_t s = 0; s < n; ++s) {
        float *qs = q + s * L;
        float poses[64 * 16], gt[64], gb[64];
        for (int it = 0; it < p->iterations; ++it) {
            or_fk_f32(r, qs, 1, poses);
            for (int j = 0; j < L; ++j) gt[j] = gb[j] = 0.f;
            if (p->task_link >= 0) pr_task_grad(r, active, p, poses, gt);
            if (p->use_boundary)
                for (int j = 0; j < L; ++j) {
                    if (!active[j]) continue;
                    if (qs[j] < lower[j]) gb[j] = lower[j] - qs[j];
                    else if (qs[j] > upper[j]) gb[j] = upper[j] - qs[j];
                }
            for (int j = 0; j < L; ++j)
                if (active[j]) qs[j] = qs[j] + (gt[j] + gb[j]);
        }
        or_fk_f32(r, qs, 1, poses);
        if (task_cost) task_cost[s] = p->task_link >= 0 ? pr_task_cost(p, poses) : 0.f;
        if (bound_cost) bound_cost[s] = p->use_boundary ? pr_bound_cost(L, active, lower, upper, qs) : 0.f;
    }
}

/* ------------------------------------------------------------------------------------
 * Constrained motions (SingleArmSpace::computeConstrainedMotions,
 * cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu:1049-1366, with approachKernel
 * :855-886, update_with_grad_and_flag :951-975, checkIfCostIsZero :1031-1045,
 * checkValidOfApproaching :888-949, updateMotionStep :980-993 and checkAchieveGoal
 * :998-1029).  Motion k walks from `from` towards `to`: every iteration moves all joints
 * by `res` along the unit direction to the goal, then runs two projection passes (FK,
 * task-space gradient and the joint-limit pull, added with step 1 to the active
 * joints; each pass records the total error: the norm of the dead-banded task error
 * plus the norm of the limit violations, at the state before its update).  The motion
 * stops approaching when the second pass's error exceeds 1e-3, when the new state is
 * farther from the goal than the previous one, or when it moved more than 5 res; each
 * state reached while still approaching is recorded; reaching the goal within `res`
 * ends it as achieved.  A motion is feasible when it achieved the goal and every
 * recorded state passes checkStates (collision costs, task-space cost and limit cost
 * all exactly 0; SingleArmSpace.cu:1295-1340); its cost is the L2 length over all
 * joints of the recorded states.  states: [n * cap * L] or NULL; count[k] the number of
 * recorded states (only the first cap are stored).
 * ---------------------------------------------------------------------------------- */
static float cm_task_error(const or_robot *r, const or_projection *p, const float *poses)
{
    float P[16], v[6], c = 0.f;
    pr_task_frame(poses, p->task_link, p->offset, P, v);
    float e[6];
    e[0] = pr_dead(p->reference[3] - v[3], p->tolerance[3]);
    e[1] = pr_dead(p->reference[4] - v[4], p->tolerance[4]);
    e[2] = pr_dead(p->reference[5] - v[5], p->tolerance[5]);
    e[3] = pr_dead(p->reference[0] - v[0], p->tolerance[0]);
    e[4] = pr_dead(p->reference[1] - v[1], p->tolerance[1]);
    e[5] = pr_dead(p->reference[2] - v[2], p->tolerance[2]);
    (void)r;
    for (int k = 0; k < 6; ++k) c += e[k] * e[k];
    return sqrtf(c);
}

void or_constrained_motions(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs,
                            const float *thr, const uint8_t *active, const float *lower, const float *upper,
                            const or_projection *p, const float *from, const float *to, int64_t n, float res,
                            int32_t max_iters, uint8_t *ok, float *cost, int32_t *count, float *states, int32_t cap,
                            int32_t nthreads)
{
    const int L = r->L;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
    for (int64_t k = 0; k < n; ++k) {
        const float *goal = to + k * L;
        float q[64], prev[64], last[64], poses[64 * 16], gt[64], gb[64], C[3 * 257];
        float *Cb = r->S <= 256 ? C : (float *)malloc(sizeof(float) * 3 * (r->S + 1));
        memcpy(q, from + k * L, sizeof(float) * L);
        int approaching = 1, achieved = 0, feasible = 1;
        int32_t steps = 0;
        double len = 0.0;
        for (int32_t it = 0; it < max_iters && approaching; ++it) {
            memcpy(prev, q, sizeof(float) * L);
            float norm = 0.f;
            for (int j = 0; j < L; ++j) { const float d = goal[j] - q[j]; norm += d * d; }
            norm = sqrtf(norm);
            if (norm > 1e-6f)
                for (int j = 0; j < L; ++j) q[j] += (goal[j] - q[j]) / norm * res;
            float err = 0.f;
            for (int pass = 0; pass < 2; ++pass) {
                or_fk_f32(r, q, 1, poses);
                for (int j = 0; j < L; ++j) gt[j] = gb[j] = 0.f;
                float et = 0.f, eb = 0.f;
                if (p->task_link >= 0) {
                    pr_task_grad(r, active, p, poses, gt);
                    et = cm_task_error(r, p, poses);
                }
                if (p->use_boundary) {
                    for (int j = 0; j < L; ++j) {
                        if (!active[j]) continue;
                        if (q[j] < lower[j]) { gb[j] = lower[j] - q[j]; eb += gb[j] * gb[j]; }
                        else if (q[j] > upper[j]) { gb[j] = upper[j] - q[j]; eb += gb[j] * gb[j]; }
                    }
                    eb = sqrtf(eb);
                }
                err = et + eb;
                for (int j = 0; j < L; ++j)
                    if (active[j]) q[j] = q[j] + (gt[j] + gb[j]);
            }
            if (err > 1e-3f) { approaching = 0; break; }
            float dpg = 0.f, dcg = 0.f, dpc = 0.f;
            for (int j = 0; j < L; ++j) {
                dpg += (prev[j] - goal[j]) * (prev[j] - goal[j]);
                dcg += (q[j] - goal[j]) * (q[j] - goal[j]);
                dpc += (prev[j] - q[j]) * (prev[j] - q[j]);
            }
            if (sqrtf(dcg) > sqrtf(dpg) || sqrtf(dpc) > res * 5.0f) { approaching = 0; break; }
            /* a recorded state: checkStates on it */
            if (states && steps < cap) memcpy(states + ((size_t)k * cap + steps) * L, q, sizeof(float) * L);
            if (steps > 0) {
                double s2 = 0.0;
                for (int j = 0; j < L; ++j) s2 += (double)(q[j] - last[j]) * (q[j] - last[j]);
                len += sqrt(s2);
            }
            memcpy(last, q, sizeof(float) * L);
            ++steps;
            if (feasible) {
                or_fk_f32(r, q, 1, poses);
                centers_one_f32(r, poses, Cb);
                if (self_cost(Cb, np, pairs, thr) != 0.f || env_sphere_cost(r, e, Cb) != 0.f ||
                    env_cuboid_cost(r, e, Cb) != 0.f || env_cylinder_cost(r, e, Cb) != 0.f)
                    feasible = 0;
                else if (p->task_link >= 0 && pr_task_cost(p, poses) != 0.f)
                    feasible = 0;
                else if (p->use_boundary && pr_bound_cost(L, active, lower, upper, q) != 0.f)
                    feasible = 0;
            }
            if (sqrtf(dcg) < res) { achieved = 1; approaching = 0; }
        }
        ok[k] = (uint8_t)(achieved && feasible);
        cost[k] = ok[k] ? (float)len : 0.f;
        count[k] = steps;
        if (Cb != C) free(Cb);
    }
}
