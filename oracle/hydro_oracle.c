/*
 * hydro_oracle.c -- CPU oracle of the hydrodynamic wrench path.
 *
 * TEST INFRASTRUCTURE ONLY (tests, smoke check, CPU-baseline leg of the
 * benchmark); the GPU library neither links nor calls this code.  See
 * hydro_oracle.h for the variants and for why parity is unpinned.
 *
 * Build (see oracle/Makefile): gcc -O3 -std=c11 -ffp-contract=off, no -march,
 * like the reference's -O3 build without FMA contraction (CMakeLists.txt:18).
 */
#define _GNU_SOURCE
#include "hydro_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

/* ----------------------------------------------------- FP64 helpers */
typedef struct { double Fb[3], Tb[3], Fdq[3], Tdq[3], Fdf[3], Tdf[3], CB[3]; double Swet, V6; } dacc;

static inline void dacc_add3(double* a, double x, double y, double z) { a[0] += x; a[1] += y; a[2] += z; }

/* btVector3::dot / cross (3rdparty/LinearMath/btVector3.h), FP64 */
static inline double bdot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void bcross(const double* a, const double* b, double* r)
{
    double x = a[1] * b[2] - a[2] * b[1];
    double y = a[2] * b[0] - a[0] * b[2];
    double z = a[0] * b[1] - a[1] * b[0];
    r[0] = x; r[1] = y; r[2] = z;
}

/* Jet::GetVelocityAtPoint (Library/src/entities/forcefields/Jet.cpp:59-80) */
static void jet_velocity(const hydro_current* c, const double* p, double* out)
{
    double cp[3] = {p[0] - c->point[0], p[1] - c->point[1], p[2] - c->point[2]};
    double x[3];
    bcross(cp, c->dir, x);
    double d = sqrt(bdot(x, x));
    double t = bdot(cp, c->dir);
    out[0] = out[1] = out[2] = 0.0;
    if (t < 0.0) return;
    double r_ = 1.0 / 5.0 * (t + 5.0 * c->radius);
    if (d >= r_) return;
    double s = 10.0 * c->radius / (t + 5.0 * c->radius) * c->speed;
    double vmax[3] = {c->dir[0] * s, c->dir[1] * s, c->dir[2] * s};
    double f = exp(-50.0 * d * d / (t * t));
    out[0] = vmax[0] * f; out[1] = vmax[1] * f; out[2] = vmax[2] * f;
}

/* Pipe::GetVelocityAtPoint (Library/src/entities/forcefields/Pipe.cpp:57-79) */
static void pipe_velocity(const hydro_current* c, const double* p, double* out)
{
    double pp[3] = {p[0] - c->point[0], p[1] - c->point[1], p[2] - c->point[2]};
    double x[3];
    bcross(pp, c->dir, x);
    double d = sqrt(bdot(x, x));
    double t = bdot(pp, c->dir);
    out[0] = out[1] = out[2] = 0.0;
    if (t < 0.0 || t > c->length) return;
    double r = c->radius + (c->radius2 - c->radius) * t / c->length;
    if (d >= r) return;
    double s = c->radius / r * c->speed;
    double v[3] = {c->dir[0] * s, c->dir[1] * s, c->dir[2] * s};
    double f = pow(1.0 - d / r, c->gamma);
    out[0] = v[0] * f; out[1] = v[1] * f; out[2] = v[2] * f;
}

/* Ocean::GetFluidVelocity(const Vector3&) (Ocean.cpp:183-196): V0() plus
 * every enabled current, only when currents are enabled. */
static void current_velocity(const hydro_ocean* o, double x, double y, double z, double* fv)
{
    fv[0] = fv[1] = fv[2] = 0.0;
    if (!o->currents_enabled) return;
    double p[3] = {x, y, z};
    uint32_t n = o->n_currents < HYDRO_MAX_CURRENTS ? o->n_currents : HYDRO_MAX_CURRENTS;
    for (uint32_t i = 0; i < n; ++i) {
        const hydro_current* c = &o->currents[i];
        if (!c->enabled) continue;
        double u[3] = {0.0, 0.0, 0.0};
        if (c->type == HYDRO_CURRENT_UNIFORM) { u[0] = c->vel[0]; u[1] = c->vel[1]; u[2] = c->vel[2]; }
        else if (c->type == HYDRO_CURRENT_JET) jet_velocity(c, p, u);
        else if (c->type == HYDRO_CURRENT_PIPE) pipe_velocity(c, p, u);
        fv[0] += u[0]; fv[1] += u[1]; fv[2] += u[2];
    }
}

/* ------------------------------------------- core instantiations */
#define T float
#define SFX _f32
#define CUT64 0
#include "hydro_oracle_core.inc"
#undef T
#undef SFX
#undef CUT64

#define T float
#define SFX _f32c64
#define CUT64 1
#include "hydro_oracle_core.inc"
#undef T
#undef SFX
#undef CUT64

#define T double
#define SFX _f64
#define CUT64 0
#include "hydro_oracle_core.inc"
#undef T
#undef SFX
#undef CUT64

/* ------------------------------------------------------- depth queries */
float oracle_depth(int variant, const hydro_ocean* ocean, const oracle_waves* waves,
                   float x, float y, float z)
{
    (void)variant;
    return depth_f32(ocean, waves, x, y, z);
}

double oracle_depth64(const hydro_ocean* ocean, const oracle_waves* waves,
                      double x, double y, double z)
{
    return depth_f64(ocean, waves, x, y, z);
}

/* SolidEntity::CheckBodyFluidPosition (SolidEntity.cpp:1239-1261) with
 * Ocean::GetDepth(const Vector3&) (Ocean.cpp:170-173): each corner is cast
 * to float, queried, and compared > 0 in double.  Every variant classifies
 * the same way so that they take the same branch. */
int oracle_fluid_position(const hydro_ocean* ocean, const oracle_waves* waves,
                          const double mn[3], const double mx[3])
{
    double d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    double c[8][3] = {
        {mn[0], mn[1], mn[2]},
        {mx[0], mx[1], mx[2]},
        {mn[0] + d[0], mn[1] + 0.0, mn[2] + 0.0},
        {mn[0] + 0.0, mn[1] + d[1], mn[2] + 0.0},
        {mn[0] + d[0], mn[1] + d[1], mn[2] + 0.0},
        {mn[0] + 0.0, mn[1] + 0.0, mn[2] + d[2]},
        {mn[0] + d[0], mn[1] + 0.0, mn[2] + d[2]},
        {mn[0] + 0.0, mn[1] + d[1], mn[2] + d[2]},
    };
    unsigned under = 0;
    for (int k = 0; k < 8; ++k) {
        float dep = depth_f32(ocean, waves, (float)c[k][0], (float)c[k][1], (float)c[k][2]);
        if ((double)dep > 0.0) ++under;
    }
    if (under == 0) return HYDRO_OUTSIDE;
    if (under == 8) return HYDRO_INSIDE;
    return HYDRO_CROSSING_SURFACE;
}

/* ------------------------------------------------------------ drivers */
static void set3(double* d, double x, double y, double z) { d[0] = x; d[1] = y; d[2] = z; }
static void zero3(double* d) { d[0] = d[1] = d[2] = 0.0; }

/* Finalisation of the surface loop on FP64 sums (SolidEntity.cpp:1689-1720
 * with the float steps carried out in FP64): REF64 and the MIRROR variants. */
static void finalize_fp64(const hydro_settings* s, const hydro_ocean* ocean,
                          const hydro_transform* T_CG, double p0x, double p0y,
                          const dacc* a, double Fb[3], double Tb[3], double Fdq[3],
                          double Tdq[3], double Fdf[3], double Tdf[3], double* Swet,
                          double* Vsub)
{
    if (s->realistic_buoyancy && a->V6 > (double)1e-9f) {
        *Vsub = a->V6 / 6.0;
        if (ocean->waves) {
            double k = ocean->density * ocean->gravity;
            set3(Fb, a->Fb[0] * k, a->Fb[1] * k, a->Fb[2] * k);
            set3(Tb, a->Tb[0] * k, a->Tb[1] * k, a->Tb[2] * k);
        } else {
            double cb[3] = {a->CB[0] / a->V6 + p0x, a->CB[1] / a->V6 + p0y, a->CB[2] / a->V6 + 0.0};
            double k = -(*Vsub) * ocean->density;
            double f[3] = {0.0 * k, 0.0 * k, ocean->gravity * k};
            double r[3] = {cb[0] - T_CG->origin[0], cb[1] - T_CG->origin[1], cb[2] - T_CG->origin[2]};
            set3(Fb, f[0], f[1], f[2]);
            bcross(r, f, Tb);
        }
    }
    if (s->damping_forces) {
        memcpy(Fdq, a->Fdq, sizeof(double) * 3);
        memcpy(Tdq, a->Tdq, sizeof(double) * 3);
        memcpy(Fdf, a->Fdf, sizeof(double) * 3);
        memcpy(Tdf, a->Tdf, sizeof(double) * 3);
    }
    *Swet = a->Swet;
}

static void acc64_to_dacc(const acc_f64* x, dacc* a)
{
    set3(a->Fb, x->Fb.x, x->Fb.y, x->Fb.z);
    set3(a->Tb, x->Tb.x, x->Tb.y, x->Tb.z);
    set3(a->Fdq, x->Fdq.x, x->Fdq.y, x->Fdq.z);
    set3(a->Tdq, x->Tdq.x, x->Tdq.y, x->Tdq.z);
    set3(a->Fdf, x->Fdf.x, x->Fdf.y, x->Fdf.z);
    set3(a->Tdf, x->Tdf.x, x->Tdf.y, x->Tdf.z);
    set3(a->CB, x->CB.x, x->CB.y, x->CB.z);
    a->Swet = x->Swet;
    a->V6 = x->V6;
}

void oracle_surface_forces(int variant, const hydro_settings* settings,
                           const oracle_mesh* mesh, const hydro_ocean* ocean,
                           const oracle_waves* waves, const hydro_transform* T_CG,
                           const hydro_transform* T_C, const double v[3],
                           const double omega[3], double Fb[3], double Tb[3],
                           double Fdq[3], double Tdq[3], double Fdf[3], double Tdf[3],
                           double* Swet, double* Vsub)
{
    /* mesh == nullptr (:1293-1312) */
    if (mesh == NULL) {
        if (settings->realistic_buoyancy) { zero3(Fb); zero3(Tb); }
        if (settings->damping_forces) { zero3(Fdq); zero3(Tdq); zero3(Fdf); zero3(Tdf); }
        *Swet = 0.0;
        *Vsub = 0.0;
        return;
    }
    if (variant == ORACLE_REF32) {
        job_f32 J;
        acc_f32 a;
        job_init_f32(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                     settings->realistic_buoyancy, settings->damping_forces);
        loop_serial_f32(&J, 1, &a);
        /* :1689-1720 in the reference's own precision */
        if (settings->realistic_buoyancy && a.V6 > 1e-9f) {
            *Vsub = (double)(a.V6 / 6.f);
            if (ocean->waves) {
                float k = (float)(ocean->density * ocean->gravity);
                set3(Fb, a.Fb.x * k, a.Fb.y * k, a.Fb.z * k);
                set3(Tb, a.Tb.x * k, a.Tb.y * k, a.Tb.z * k);
            } else {
                float cbx = a.CB.x / a.V6 + J.p0.x;
                float cby = a.CB.y / a.V6 + J.p0.y;
                float cbz = a.CB.z / a.V6 + J.p0.z;
                double k = -(*Vsub) * ocean->density;
                double f[3] = {0.0 * k, 0.0 * k, ocean->gravity * k};
                double r[3] = {(double)cbx - T_CG->origin[0], (double)cby - T_CG->origin[1],
                               (double)cbz - T_CG->origin[2]};
                set3(Fb, f[0], f[1], f[2]);
                bcross(r, f, Tb);
            }
        }
        if (settings->damping_forces) {
            set3(Fdq, a.Fdq.x, a.Fdq.y, a.Fdq.z);
            set3(Tdq, a.Tdq.x, a.Tdq.y, a.Tdq.z);
            set3(Fdf, a.Fdf.x, a.Fdf.y, a.Fdf.z);
            set3(Tdf, a.Tdf.x, a.Tdf.y, a.Tdf.z);
        }
        *Swet = (double)a.Swet;
        return;
    }
    dacc d;
    double p0x, p0y;
    if (variant == ORACLE_REF64) {
        job_f64 J;
        acc_f64 a;
        job_init_f64(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                     settings->realistic_buoyancy, settings->damping_forces);
        loop_serial_f64(&J, 1, &a);
        acc64_to_dacc(&a, &d);
        p0x = J.p0.x; p0y = J.p0.y;
    } else if (variant == ORACLE_MIRROR64) {
        job_f32c64 J;
        job_init_f32c64(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                        settings->realistic_buoyancy, settings->damping_forces);
        loop_exact_f32c64(&J, 1, &d);
        p0x = J.p0.x; p0y = J.p0.y;
    } else {
        job_f32 J;
        job_init_f32(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                     settings->realistic_buoyancy, settings->damping_forces);
        loop_exact_f32(&J, 1, &d);
        p0x = J.p0.x; p0y = J.p0.y;
    }
    finalize_fp64(settings, ocean, T_CG, p0x, p0y, &d, Fb, Tb, Fdq, Tdq, Fdf, Tdf, Swet, Vsub);
}

void oracle_submerged_forces(int variant, const oracle_mesh* mesh,
                             const hydro_ocean* ocean, const hydro_transform* T_CG,
                             const hydro_transform* T_C, const double v[3],
                             const double omega[3], double Fdq[3], double Tdq[3],
                             double Fdf[3], double Tdf[3])
{
    if (mesh == NULL) { zero3(Fdq); zero3(Tdq); zero3(Fdf); zero3(Tdf); return; }  /* :1726-1733 */
    dacc d;
    if (variant == ORACLE_REF32) {
        job_f32 J;
        acc_f32 a;
        job_init_f32(&J, mesh, ocean, NULL, T_CG, T_C, v, omega, 0, 1);
        loop_serial_f32(&J, 0, &a);
        set3(Fdq, a.Fdq.x, a.Fdq.y, a.Fdq.z);
        set3(Tdq, a.Tdq.x, a.Tdq.y, a.Tdq.z);
        set3(Fdf, a.Fdf.x, a.Fdf.y, a.Fdf.z);
        set3(Tdf, a.Tdf.x, a.Tdf.y, a.Tdf.z);
        return;
    }
    if (variant == ORACLE_REF64) {
        job_f64 J;
        acc_f64 a;
        job_init_f64(&J, mesh, ocean, NULL, T_CG, T_C, v, omega, 0, 1);
        loop_serial_f64(&J, 0, &a);
        acc64_to_dacc(&a, &d);
    } else {
        /* the submerged loop has no cut points: both mirrors coincide */
        job_f32 J;
        job_init_f32(&J, mesh, ocean, NULL, T_CG, T_C, v, omega, 0, 1);
        loop_exact_f32(&J, 0, &d);
    }
    memcpy(Fdq, d.Fdq, sizeof(double) * 3);
    memcpy(Tdq, d.Tdq, sizeof(double) * 3);
    memcpy(Fdf, d.Fdf, sizeof(double) * 3);
    memcpy(Tdf, d.Tdf, sizeof(double) * 3);
}

/* btMatrix3x3::inverse (3rdparty/LinearMath/btMatrix3x3.h:1093-1103) */
static void binverse(const double* m, double* r)
{
#define M(i, j) m[3 * (i) + (j)]
#define COF(r1, c1, r2, c2) (M(r1, c1) * M(r2, c2) - M(r1, c2) * M(r2, c1))
    double co[3] = {COF(1, 1, 2, 2), COF(1, 2, 2, 0), COF(1, 0, 2, 1)};
    double det = M(0, 0) * co[0] + M(0, 1) * co[1] + M(0, 2) * co[2];
    double s = 1.0 / det;
    r[0] = co[0] * s; r[1] = COF(0, 2, 2, 1) * s; r[2] = COF(0, 1, 1, 2) * s;
    r[3] = co[1] * s; r[4] = COF(0, 0, 2, 2) * s; r[5] = COF(0, 2, 1, 0) * s;
    r[6] = co[2] * s; r[7] = COF(0, 1, 2, 0) * s; r[8] = COF(0, 0, 1, 1) * s;
#undef COF
#undef M
}

/* One vector of CorrectHydrodynamicForces (SolidEntity.cpp:1266-1286). */
static void correct_one(const double* inv, double* vec, const double* C, double k)
{
    double w[3] = {inv[0] * vec[0] + inv[1] * vec[1] + inv[2] * vec[2],
                   inv[3] * vec[0] + inv[4] * vec[1] + inv[5] * vec[2],
                   inv[6] * vec[0] + inv[7] * vec[1] + inv[8] * vec[2]};
    /* btVector3::safeNormalize (btVector3.h:286-299) */
    double l2 = bdot(w, w);
    if (l2 >= DBL_EPSILON * DBL_EPSILON) {
        double s = 1.0 / sqrt(l2);
        w[0] *= s; w[1] *= s; w[2] *= s;
    } else {
        w[0] = 1.0; w[1] = 0.0; w[2] = 0.0;
    }
    double c = fabs(w[0]) * C[0] + fabs(w[1]) * C[1] + fabs(w[2]) * C[2];
    double f = k * c;
    vec[0] = f * vec[0]; vec[1] = f * vec[1]; vec[2] = f * vec[2];
}

void oracle_correct_forces(const hydro_ocean* ocean, double Fdq[3], double Tdq[3],
                           double Fdf[3], double Tdf[3], const double Cd[3],
                           const double Cf[3], const double R_O[9])
{
    double inv[9];
    binverse(R_O, inv);
    correct_one(inv, Fdq, Cd, 0.5 * ocean->density);
    correct_one(inv, Tdq, Cd, 0.5 * ocean->density);
    correct_one(inv, Fdf, Cf, ocean->density);
    correct_one(inv, Tdf, Cf, ocean->density);
}

/* ---------------------------------------------------------- mesh ingest */
/* ComputePhysicalProperties (Library/src/utils/GeometryFileUtil.cpp:335-566),
 * serial FP64 sums as the reference; btVector3's "/ s" multiplies by 1 / s. */
static void pterms(const double* v1, const double* v2, const double* v3, double* P)
{
    double c[3];
    bcross(v2, v3, c);
    const double V6 = bdot(v1, c);
#define SQ(k) (v1[k] * v1[k] + v2[k] * v2[k] + v3[k] * v3[k] + v1[k] * v2[k] + v1[k] * v3[k] + v2[k] * v3[k])
#define PR(j, k) (2 * (v1[j] * v1[k] + v2[j] * v2[k] + v3[j] * v3[k]) + v1[j] * v2[k] + v1[k] * v2[j] + \
                  v1[j] * v3[k] + v1[k] * v3[j] + v2[j] * v3[k] + v2[k] * v3[j])
    P[0] += V6 * 2 * SQ(0);
    P[1] += V6 * 2 * SQ(1);
    P[2] += V6 * 2 * SQ(2);
    P[3] += V6 * PR(0, 1);
    P[4] += V6 * PR(0, 2);
    P[5] += V6 * PR(1, 2);
#undef SQ
#undef PR
}

void oracle_mesh_properties(const oracle_mesh* mesh, double thickness, double density, double out[7])
{
    double surface = 0.0, volume = 0.0, cg[3] = {0, 0, 0};
    for (uint32_t i = 0; i < mesh->n_faces; ++i) {
        double v[3][3];
        for (int a = 0; a < 3; ++a) {
            const float* q = mesh->xyz + (size_t)mesh->idx[3 * i + a] * mesh->stride;
            v[a][0] = q[0]; v[a][1] = q[1]; v[a][2] = q[2];
        }
        double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
        double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
        double n[3];
        bcross(e1, e2, n);
        const double A = sqrt(bdot(n, n)) / 2.0;
        surface += A;
        if (thickness > 0.0) {
            const double V = A * thickness;
            for (int k = 0; k < 3; ++k) cg[k] += ((v[0][k] + v[1][k]) + v[2][k]) * (1.0 / 3.0) * V;
            volume += V;
        } else {
            double c[3];
            bcross(v[1], v[2], c);
            const double V6 = bdot(v[0], c);
            for (int k = 0; k < 3; ++k) cg[k] += ((v[0][k] + v[1][k]) + v[2][k]) * 0.25 * V6;
            volume += V6;
        }
    }
    if (volume > 0.0) {
        const double iv = 1.0 / volume;
        for (int k = 0; k < 3; ++k) cg[k] *= iv;
    } else {
        cg[0] = cg[1] = cg[2] = 0.0;
    }
    if (!(thickness > 0.0)) volume /= 6.0;
    double P[6] = {0, 0, 0, 0, 0, 0}, Pi[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = 0; i < mesh->n_faces; ++i) {
        double v[3][3];
        for (int a = 0; a < 3; ++a) {
            const float* q = mesh->xyz + (size_t)mesh->idx[3 * i + a] * mesh->stride;
            v[a][0] = q[0]; v[a][1] = q[1]; v[a][2] = q[2];
        }
        if (thickness > 0.0) {
            double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
            double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
            double n[3];
            bcross(e1, e2, n);
            const double il = 1.0 / sqrt(bdot(n, n));
            const double u[3] = {n[0] * il, n[1] * il, n[2] * il};
            double o[3][3], in[3][3];
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < 3; ++k) {
                    o[a][k] = v[a][k] + u[k] * thickness / 2.0 - cg[k];
                    in[a][k] = v[a][k] - u[k] * thickness / 2.0 - cg[k];
                }
            pterms(o[0], o[1], o[2], P);
            pterms(in[0], in[1], in[2], Pi);
        } else {
            double r[3][3];
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < 3; ++k) r[a][k] = v[a][k] - cg[k];
            pterms(r[0], r[1], r[2], P);
        }
    }
    const double k = density / 120.0;
    double Ixx = (P[1] * k + P[2] * k), Iyy = (P[0] * k + P[2] * k), Izz = (P[0] * k + P[1] * k);
    if (thickness > 0.0) {
        Ixx -= (Pi[1] * k + Pi[2] * k);
        Iyy -= (Pi[0] * k + Pi[2] * k);
        Izz -= (Pi[0] * k + Pi[1] * k);
    }
    out[0] = volume * density;   /* mass */
    out[1] = volume;
    out[2] = surface;
    out[3] = cg[0]; out[4] = cg[1]; out[5] = cg[2];
    out[6] = Ixx + Iyy + Izz;    /* trace of the inertia tensor (invariant of the principal axes) */
}

/* ------------------------------------------------------------- compounds */
static int fluid_mode(int m) { return m == HYDRO_MODE_FLOATING || m == HYDRO_MODE_SUBMERGED; }

/* Compound::ComputeHydrodynamicForces (Library/src/entities/solids/Compound.cpp:291-436). */
void oracle_compound_forces(int variant, const hydro_body* cb, const hydro_compound_part* parts,
                            uint32_t n_parts, const oracle_mesh* const* part_meshes,
                            const hydro_ocean* ocean, const oracle_waves* waves,
                            const hydro_settings* settings, hydro_wrench* io)
{
    if (!fluid_mode(cb->mode)) {                                   /* :293 */
        io->position = HYDRO_SKIPPED;
        return;
    }
    int bf = oracle_fluid_position(ocean, waves, cb->aabb_min, cb->aabb_max);   /* :299 */
    io->position = bf;
    if (bf == HYDRO_OUTSIDE) {                                     /* :302-314 */
        zero3(io->Fb); zero3(io->Tb); zero3(io->Fdq); zero3(io->Tdq);
        zero3(io->Fdf); zero3(io->Tdf);
        io->Swet = 0.0;
        io->Vsub = 0.0;
        return;
    }
    if (bf == HYDRO_INSIDE) {                                      /* :316-357 */
        if (cb->buoyancy) {
            double k = -cb->volume * ocean->density;
            double f[3] = {0.0 * k, 0.0 * k, ocean->gravity * k};
            const double* R = cb->T_CG.basis;
            const double* o = cb->T_CG.origin;
            double c[3] = {(R[0] * cb->P_CB[0] + R[1] * cb->P_CB[1] + R[2] * cb->P_CB[2]) + o[0],
                           (R[3] * cb->P_CB[0] + R[4] * cb->P_CB[1] + R[5] * cb->P_CB[2]) + o[1],
                           (R[6] * cb->P_CB[0] + R[7] * cb->P_CB[1] + R[8] * cb->P_CB[2]) + o[2]};
            double r[3] = {c[0] - o[0], c[1] - o[1], c[2] - o[2]};
            set3(io->Fb, f[0], f[1], f[2]);
            bcross(r, f, io->Tb);
        }
        if (settings->damping_forces) {
            zero3(io->Fdq); zero3(io->Tdq); zero3(io->Fdf); zero3(io->Tdf);
            double Fq[3] = {0, 0, 0}, Tq[3] = {0, 0, 0}, Ff[3] = {0, 0, 0}, Tf[3] = {0, 0, 0};
            for (uint32_t i = 0; i < n_parts; ++i) {
                const hydro_compound_part* pt = &parts[i];
                if (!(pt->external && fluid_mode(pt->mode))) continue;
                oracle_submerged_forces(variant, part_meshes[i], ocean, &cb->T_CG, &pt->T_C, cb->v, cb->omega,
                                        Fq, Tq, Ff, Tf);
                oracle_correct_forces(ocean, Fq, Tq, Ff, Tf, pt->Cd, pt->Cf, pt->R_O);
                for (int k = 0; k < 3; ++k) {
                    io->Fdq[k] += Fq[k]; io->Tdq[k] += Tq[k]; io->Fdf[k] += Ff[k]; io->Tdf[k] += Tf[k];
                }
            }
        }
        io->Swet = cb->surface;
        io->Vsub = cb->volume;
        return;
    }
    if (!(settings->realistic_buoyancy || settings->damping_forces)) return;   /* :361 */
    if (settings->realistic_buoyancy) { zero3(io->Fb); zero3(io->Tb); }
    if (settings->damping_forces) { zero3(io->Fdq); zero3(io->Tdq); zero3(io->Fdf); zero3(io->Tdf); }
    io->Swet = 0.0;
    io->Vsub = 0.0;
    /* the per-part in-out values live across the loop (:379-386) */
    double Fbp[3] = {0, 0, 0}, Tbp[3] = {0, 0, 0}, Fqp[3] = {0, 0, 0}, Tqp[3] = {0, 0, 0};
    double Ffp[3] = {0, 0, 0}, Tfp[3] = {0, 0, 0}, Swetp = 0.0, Vsubp = 0.0;
    for (uint32_t i = 0; i < n_parts; ++i) {
        const hydro_compound_part* pt = &parts[i];
        if (!fluid_mode(pt->mode)) continue;
        hydro_settings ps = *settings;
        ps.realistic_buoyancy = ps.realistic_buoyancy && pt->buoyant;
        if (pt->external) {
            oracle_surface_forces(variant, &ps, part_meshes[i], ocean, waves, &cb->T_CG, &pt->T_C, cb->v,
                                  cb->omega, Fbp, Tbp, Fqp, Tqp, Ffp, Tfp, &Swetp, &Vsubp);
            oracle_correct_forces(ocean, Fqp, Tqp, Ffp, Tfp, pt->Cd, pt->Cf, pt->R_O);
            for (int k = 0; k < 3; ++k) {
                io->Fb[k] += Fbp[k]; io->Tb[k] += Tbp[k]; io->Fdq[k] += Fqp[k]; io->Tdq[k] += Tqp[k];
                io->Fdf[k] += Ffp[k]; io->Tdf[k] += Tfp[k];
            }
            io->Swet += Swetp;
            io->Vsub += Vsubp;
        } else if (ps.realistic_buoyancy) {
            ps.damping_forces = 0;
            oracle_surface_forces(variant, &ps, part_meshes[i], ocean, waves, &cb->T_CG, &pt->T_C, cb->v,
                                  cb->omega, Fbp, Tbp, Fqp, Tqp, Ffp, Tfp, &Swetp, &Vsubp);
            for (int k = 0; k < 3; ++k) { io->Fb[k] += Fbp[k]; io->Tb[k] += Tbp[k]; }
            io->Vsub += Vsubp;
        }
    }
}

/* ---------------------------------------------------------------- cables */
/* CableEntity::circularSegmentArea (CableEntity.cpp:218-238) with btAcos's clamp */
static double cable_acos(double x) { if (x < -1.0) x = -1.0; if (x > 1.0) x = 1.0; return acos(x); }

static double circular_segment_area(double h, double r)
{
    if (h <= 0.0) return 0.0;
    if (h >= 2.0 * r) return M_PI * r * r;
    if (h > r) {
        h = 2.0 * r - h;
        double theta = 2.0 * cable_acos((r - h) / r);
        return r * r * (M_PI - (theta - sin(theta)) / 2.0);
    }
    double theta = 2.0 * cable_acos((r - h) / r);
    return (r * r / 2.0) * (theta - sin(theta));
}

/* CableEntity::ComputeHydrodynamicForces (CableEntity.cpp:240-376). */
void oracle_cable_forces(const hydro_cable* cables, uint32_t n_cables, const double* x, const double* v,
                         uint32_t n_nodes_total, const hydro_ocean* ocean, const oracle_waves* waves,
                         const hydro_settings* settings, hydro_cable_node_forces* out)
{
    for (uint32_t c = 0; c < n_cables; ++c) {
        const hydro_cable* cb = &cables[c];
        if (cb->mode != HYDRO_MODE_FLOATING && cb->mode != HYDRO_MODE_SUBMERGED) continue;   /* :242 */
        uint32_t n = cb->n_nodes, f = cb->first_node;
        if (n == 0 || (uint64_t)f + n > n_nodes_total) continue;
        double r = cb->radius;
        for (uint32_t i = 0; i < n; ++i) memset(&out[f + i], 0, sizeof(out[f + i]));      /* :245-246 */
        for (uint32_t i = 0; i + 1 < n; ++i) {
            double p1[3], p2[3];
            memcpy(p1, x + 3 * (size_t)(f + i), sizeof(p1));
            memcpy(p2, x + 3 * (size_t)(f + i + 1), sizeof(p2));
            double d1 = (double)oracle_depth(ORACLE_REF32, ocean, waves, (float)p1[0], (float)p1[1], (float)p1[2]);
            double d2 = (double)oracle_depth(ORACLE_REF32, ocean, waves, (float)p2[0], (float)p2[1], (float)p2[2]);
            if (d1 > d2) {
                double t[3];
                memcpy(t, p1, sizeof(t)); memcpy(p1, p2, sizeof(t)); memcpy(p2, t, sizeof(t));
                double td = d1; d1 = d2; d2 = td;
            }
            double dz = d2 - d1;
            double hx = p2[0] - p1[0], hy = p2[1] - p1[1];
            double h2 = hx * hx + hy * hy + 0.0 * 0.0;          /* btVector3::safeNorm */
            double dxy = h2 > DBL_EPSILON ? sqrt(h2) : 0.0;
            double sv[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
            double L = sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
            double alpha = atan(dz / dxy);
            double margin = fabs(dxy) < DBL_EPSILON ? 0.0 : r * cos(alpha);
            double V = 0.0;
            if (d2 < -margin) continue;
            else if (d1 > margin) V = M_PI * r * r * L;
            else if (fabs(dxy) < DBL_EPSILON) V = M_PI * r * r * (d2 < dz ? d2 : dz);
            else if (fabs(dz) < DBL_EPSILON) V = circular_segment_area(d1 + r, r) * L;
            else if (fabs(d1) <= margin && fabs(d2) <= margin) {
                double A1 = circular_segment_area(d1 / cos(alpha) + r, r);
                double A2 = circular_segment_area(d2 / cos(alpha) + r, r);
                V = (A1 + A2) / 2.0 * L;
            } else if (d1 < -margin && d2 > margin) {
                double l1 = (d2 - r * cos(alpha)) / sin(alpha);
                double l2 = 2.0 * r * cos(alpha);
                V = M_PI * r * r * (l1 + l2 / 2.0);
            } else if (d2 <= margin) {
                double a = r + d2 / cos(alpha);
                double l = a / sin(alpha);
                V = circular_segment_area(a, r) * l / 2.0;
            } else if (d1 >= -margin) {
                double a = r - d1 / cos(alpha);
                double l = a / sin(alpha);
                V = M_PI * r * r * L - circular_segment_area(a, r) * l / 2.0;
            }
            if (cb->buoyancy && settings->realistic_buoyancy) {
                double k = -V * ocean->density;
                double b[3] = {k * 0.0, k * 0.0, k * ocean->gravity};
                for (int q = 0; q < 3; ++q) {
                    out[f + i].Fb[q] += b[q] / 2.0;
                    out[f + i + 1].Fb[q] += b[q] / 2.0;
                }
            }
            if (settings->damping_forces && V > 0.0) {
                double p[3] = {(p1[0] + p2[0]) / 2.0, (p1[1] + p2[1]) / 2.0, (p1[2] + p2[2]) / 2.0};
                const double* va = v + 3 * (size_t)(f + i);
                const double* vb = v + 3 * (size_t)(f + i + 1);
                double vm[3] = {(va[0] + vb[0]) / 2.0, (va[1] + vb[1]) / 2.0, (va[2] + vb[2]) / 2.0};
                double wv[3];
                current_velocity(ocean, p[0], p[1], p[2], wv);
                double rv[3] = {vm[0] - wv[0], vm[1] - wv[1], vm[2] - wv[2]};
                double f1 = fabs(sv[0] * rv[0] + sv[1] * rv[1] + sv[2] * rv[2]);
                double f2 = V / (M_PI * r * r * L);
                double rl = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
                double S = 2.0 * r * L;
                double qd = -(1.0 - f1) * f2 * 0.5 * ocean->density * 0.5 * S * rl;
                double Sf = f2 * ((2.0 * M_PI) * r * L);
                for (int q = 0; q < 3; ++q) {
                    double fq = qd * rv[q], ff = -Sf * rv[q];
                    out[f + i].Fdq[q] += fq / 2.0;
                    out[f + i + 1].Fdq[q] += fq / 2.0;
                    out[f + i].Fdf[q] += ff / 2.0;
                    out[f + i + 1].Fdf[q] += ff / 2.0;
                }
            }
        }
        for (int q = 0; q < 3; ++q) {                          /* :367-373 */
            out[f].Fb[q] *= 2.0; out[f + n - 1].Fb[q] *= 2.0;
            out[f].Fdq[q] *= 2.0; out[f + n - 1].Fdq[q] *= 2.0;
            out[f].Fdf[q] *= 2.0; out[f + n - 1].Fdf[q] *= 2.0;
        }
    }
}

/* ----------------------------------------------------------- aerodynamics */
/* Atmosphere::GetFluidVelocity sums every wind field (Atmosphere.cpp:146-152):
 * the winds as enabled currents of an ocean descriptor. */
static void atmosphere_ocean(const hydro_atmosphere* a, hydro_ocean* o)
{
    memset(o, 0, sizeof(*o));
    o->density = a->density;
    o->currents_enabled = 1;
    o->n_currents = a->n_winds < HYDRO_MAX_CURRENTS ? a->n_winds : HYDRO_MAX_CURRENTS;
    for (uint32_t i = 0; i < o->n_currents; ++i) {
        o->currents[i] = a->winds[i];
        o->currents[i].enabled = 1;
    }
}

/* SolidEntity::ComputeAerodynamicForces(mesh, atm, T_CG, T_C, v, omega, Fda, Tda)
 * (SolidEntity.cpp:1865-1923). */
void oracle_aero_forces(int variant, const oracle_mesh* mesh, const hydro_atmosphere* atm,
                        const hydro_transform* T_CG, const hydro_transform* T_C, const double v[3],
                        const double omega[3], double Fda[3], double Tda[3])
{
    if (mesh == NULL) { zero3(Fda); zero3(Tda); return; }  /* :1868-1873 */
    hydro_ocean o;
    atmosphere_ocean(atm, &o);
    double F[3] = {0, 0, 0}, Tq[3] = {0, 0, 0};
    if (variant == ORACLE_REF32) {
        job_f32 J;
        v3_f32 f = {0, 0, 0}, t = {0, 0, 0};
        job_init_f32(&J, mesh, &o, NULL, T_CG, T_C, v, omega, 0, 0);
        for (uint32_t i = 0; i < mesh->n_faces; ++i) face_aero_f32(&J, i, &f, &t);
        set3(F, f.x, f.y, f.z);
        set3(Tq, t.x, t.y, t.z);
    } else if (variant == ORACLE_REF64) {
        job_f64 J;
        v3_f64 f = {0, 0, 0}, t = {0, 0, 0};
        job_init_f64(&J, mesh, &o, NULL, T_CG, T_C, v, omega, 0, 0);
        for (uint32_t i = 0; i < mesh->n_faces; ++i) face_aero_f64(&J, i, &f, &t);
        set3(F, f.x, f.y, f.z);
        set3(Tq, t.x, t.y, t.z);
    } else {
        /* FP32 face terms summed in double: the GPU kernel's arithmetic */
        job_f32 J;
        job_init_f32(&J, mesh, &o, NULL, T_CG, T_C, v, omega, 0, 0);
        for (uint32_t i = 0; i < mesh->n_faces; ++i) {
            v3_f32 f = {0, 0, 0}, t = {0, 0, 0};
            face_aero_f32(&J, i, &f, &t);
            F[0] += (double)f.x; F[1] += (double)f.y; F[2] += (double)f.z;
            Tq[0] += (double)t.x; Tq[1] += (double)t.y; Tq[2] += (double)t.z;
        }
    }
    const double k = 0.5 * atm->density;                    /* :1918-1922 */
    set3(Fda, k * F[0], k * F[1], k * F[2]);
    set3(Tda, k * Tq[0], k * Tq[1], k * Tq[2]);
}

/* SolidEntity::CorrectAerodynamicForces (SolidEntity.cpp:1925-1956). */
void oracle_aero_correct(const hydro_aero_params* p, double Fda[3], double Tda[3])
{
    double inv[9];
    binverse(p->R_CG2H, inv);
    double n[3] = {inv[0] * Fda[0] + inv[1] * Fda[1] + inv[2] * Fda[2],
                   inv[3] * Fda[0] + inv[4] * Fda[1] + inv[5] * Fda[2],
                   inv[6] * Fda[0] + inv[7] * Fda[1] + inv[8] * Fda[2]};
    /* btVector3::safeNormalize; operator/= multiplies by the reciprocal */
    double l2 = bdot(n, n);
    if (l2 >= DBL_EPSILON * DBL_EPSILON) {
        double s = 1.0 / sqrt(l2);
        n[0] *= s; n[1] *= s; n[2] *= s;
    } else {
        n[0] = 1.0; n[1] = 0.0; n[2] = 0.0;
    }
    double cor = 1.0;
    if (p->approx_type == HYDRO_APPROX_CYLINDER) {
        double cd[3] = {0.5, 0.5, 1.0};
        cor = bdot(cd, n);
    } else if (p->approx_type == HYDRO_APPROX_ELLIPSOID) {
        double cd[3] = {1.0 / p->approx_params[0], 1.0 / p->approx_params[1], 1.0 / p->approx_params[2]};
        double mx = cd[0] > cd[1] ? cd[0] : cd[1];
        mx = mx > cd[2] ? mx : cd[2];
        double s = 1.0 / mx;
        cd[0] *= s; cd[1] *= s; cd[2] *= s;
        cor = bdot(cd, n);
    }
    cor = fabs(cor);
    for (int k = 0; k < 3; ++k) { Fda[k] *= cor; Tda[k] *= cor; }
}

/* SolidEntity::ComputeHydrodynamicForces (SolidEntity.cpp:1799-1850). */
void oracle_body_forces(int variant, const hydro_body* b, const oracle_mesh* mesh,
                        const hydro_ocean* ocean, const oracle_waves* waves,
                        const hydro_settings* settings, hydro_wrench* io)
{
    if (b->mode != HYDRO_MODE_FLOATING && b->mode != HYDRO_MODE_SUBMERGED) {
        io->position = HYDRO_SKIPPED;
        return;
    }
    int bf = oracle_fluid_position(ocean, waves, b->aabb_min, b->aabb_max);
    io->position = bf;
    if (bf == HYDRO_OUTSIDE) {
        zero3(io->Fb); zero3(io->Tb); zero3(io->Fdq); zero3(io->Tdq);
        zero3(io->Fdf); zero3(io->Tdf);
        io->Swet = 0.0;
        io->Vsub = 0.0;
        return;
    }
    int buoyant = b->buoyancy != 0;  /* isBuoyant(), :205-208 */
    if (bf == HYDRO_INSIDE) {
        if (buoyant) {
            double k = -b->volume * ocean->density;
            double f[3] = {0.0 * k, 0.0 * k, ocean->gravity * k};
            const double* R = b->T_CG.basis;
            const double* o = b->T_CG.origin;
            double cb[3] = {(R[0] * b->P_CB[0] + R[1] * b->P_CB[1] + R[2] * b->P_CB[2]) + o[0],
                            (R[3] * b->P_CB[0] + R[4] * b->P_CB[1] + R[5] * b->P_CB[2]) + o[1],
                            (R[6] * b->P_CB[0] + R[7] * b->P_CB[1] + R[8] * b->P_CB[2]) + o[2]};
            double r[3] = {cb[0] - o[0], cb[1] - o[1], cb[2] - o[2]};
            set3(io->Fb, f[0], f[1], f[2]);
            bcross(r, f, io->Tb);
        }
        if (settings->damping_forces)
            oracle_submerged_forces(variant, mesh, ocean, &b->T_CG, &b->T_C, b->v, b->omega,
                                    io->Fdq, io->Tdq, io->Fdf, io->Tdf);
        io->Swet = b->surface;
    } else {
        hydro_settings s = *settings;
        if (!buoyant) s.realistic_buoyancy = 0;
        oracle_surface_forces(variant, &s, mesh, ocean, waves, &b->T_CG, &b->T_C, b->v,
                              b->omega, io->Fb, io->Tb, io->Fdq, io->Tdq, io->Fdf, io->Tdf,
                              &io->Swet, &io->Vsub);
    }
    if (settings->damping_forces)
        oracle_correct_forces(ocean, io->Fdq, io->Tdq, io->Fdf, io->Tdf, b->Cd, b->Cf, b->R_O);
}

void oracle_surface_face_terms(int variant, const hydro_settings* settings,
                               const oracle_mesh* mesh, const hydro_ocean* ocean,
                               const oracle_waves* waves, const hydro_transform* T_CG,
                               const hydro_transform* T_C, const double v[3],
                               const double omega[3], float* out)
{
    if (variant == ORACLE_MIRROR64) {
        job_f32c64 J;
        job_init_f32c64(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                        settings->realistic_buoyancy, settings->damping_forces);
        face_terms_f32c64(&J, out);
    } else {
        job_f32 J;
        job_init_f32(&J, mesh, ocean, waves, T_CG, T_C, v, omega,
                     settings->realistic_buoyancy, settings->damping_forces);
        face_terms_f32(&J, out);
    }
}

/* --------------------------------------------------------- batch */
typedef struct {
    int variant;
    const hydro_body* bodies;
    uint32_t n;
    const oracle_mesh* meshes;
    uint32_t n_meshes;
    const hydro_ocean* ocean;
    const oracle_waves* waves;
    const hydro_settings* settings;
    hydro_wrench* io;
    atomic_uint next;
    pthread_barrier_t start;
} batch_job;

static void* batch_worker(void* arg)
{
    batch_job* B = (batch_job*)arg;
    pthread_barrier_wait(&B->start);
    for (;;) {
        unsigned i = atomic_fetch_add_explicit(&B->next, 1u, memory_order_relaxed);
        if (i >= B->n) break;
        const hydro_body* b = &B->bodies[i];
        const oracle_mesh* m = (b->mesh < B->n_meshes) ? &B->meshes[b->mesh] : NULL;
        oracle_body_forces(B->variant, b, m, B->ocean, B->waves, B->settings, &B->io[i]);
    }
    return NULL;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double oracle_batch(int variant, int threads, const hydro_body* bodies, uint32_t n_bodies,
                    const oracle_mesh* meshes, uint32_t n_meshes, const hydro_ocean* ocean,
                    const oracle_waves* waves, const hydro_settings* settings,
                    hydro_wrench* io)
{
    if (threads < 1) threads = 1;
    batch_job B;
    B.variant = variant;
    B.bodies = bodies;
    B.n = n_bodies;
    B.meshes = meshes;
    B.n_meshes = n_meshes;
    B.ocean = ocean;
    B.waves = waves;
    B.settings = settings;
    B.io = io;
    atomic_init(&B.next, 0u);
    pthread_barrier_init(&B.start, NULL, (unsigned)threads + 1u);
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, batch_worker, &B);
    double t0 = now_s();
    pthread_barrier_wait(&B.start);
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
    double t1 = now_s();
    pthread_barrier_destroy(&B.start);
    free(tid);
    return t1 - t0;
}

int oracle_hardware_threads(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}
