// hydro_kernels.cu -- GB300 kernels of the hydrodynamic wrench path.
//
// The batched step replaces the per-body loop of the hydrodynamics block of
// SimulationManager::SimulationTickCallback (SimulationManager.cpp:1620-1655)
// with three launches:
//   prep      one thread per body: fluid position (CheckBodyFluidPosition,
//             SolidEntity.cpp:1239-1261), loop kind and the body's FP32
//             parameters (the glm casts of ComputeHydrodynamicForcesSurface);
//   chunk     persistent CTAs.  One producer lane claims chunks (runs of up
//             to 16 tiles of <= 448 faces with their <= 448 distinct
//             vertices, contiguous in HBM) and streams their tiles into a
//             4-stage shared-memory ring with 1-D TMA bulk copies signalled
//             on mbarriers; 7 consumer warps transform each vertex once
//             (with its depth, Ocean::GetDepth) and evaluate the faces
//             (surface loop :1337-1687, submerged loop :1748-1789, or the
//             aerodynamic loop :1885-1915) from shared memory.  Per-face
//             quantities are summed in FP32 over at most kFlushFaces faces
//             per thread, then by a butterfly reduce-scatter across the warp
//             into a two-sum (float-float) accumulator per lane, combined
//             across warps and stored as one FP64 partial per chunk;
//   finalise  four threads per body: the body's chunk partials are added
//             in chunk order in FP64 and the FP64 finalisation is applied:
//             buoyancy (:1689-1720, :1828-1836), the stale-output rules and
//             CorrectHydrodynamicForces (:1263-1287).
// No result depends on scheduling: every sum has a fixed order.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "hydro_internal.h"
#include "hydro_pair.cuh"


namespace sfh {

// --------------------------------------------------------------- FP64 helpers
struct d3 { double x, y, z; };

// SolidEntity::CheckBodyFluidPosition with Ocean::GetDepth(const Vector3&):
// each AABB corner cast to float, depth compared > 0 in double.
__device__ int classify(const OceanDev& o, const double* mn, const double* mx)
{
    const double d0 = mx[0] - mn[0], d1 = mx[1] - mn[1], d2 = mx[2] - mn[2];
    const double c[8][3] = {
        {mn[0], mn[1], mn[2]},
        {mx[0], mx[1], mx[2]},
        {mn[0] + d0, mn[1] + 0.0, mn[2] + 0.0},
        {mn[0] + 0.0, mn[1] + d1, mn[2] + 0.0},
        {mn[0] + d0, mn[1] + d1, mn[2] + 0.0},
        {mn[0] + 0.0, mn[1] + 0.0, mn[2] + d2},
        {mn[0] + d0, mn[1] + 0.0, mn[2] + d2},
        {mn[0] + 0.0, mn[1] + d1, mn[2] + d2},
    };
    unsigned under = 0;
    for (int k = 0; k < 8; ++k) {
        float dep = depth_at(o, (float)c[k][0], (float)c[k][1], (float)c[k][2]);
        if ((double)dep > 0.0) ++under;
    }
    if (under == 0) return HYDRO_OUTSIDE;
    if (under == 8) return HYDRO_INSIDE;
    return HYDRO_CROSSING_SURFACE;
}

// btMatrix3x3::inverse (3rdparty/LinearMath/btMatrix3x3.h:1093-1103)
__device__ void binverse(const double* m, double* r)
{
#define M_(i, j) m[3 * (i) + (j)]
#define COF(r1, c1, r2, c2) (M_(r1, c1) * M_(r2, c2) - M_(r1, c2) * M_(r2, c1))
    double co0 = COF(1, 1, 2, 2), co1 = COF(1, 2, 2, 0), co2 = COF(1, 0, 2, 1);
    double det = M_(0, 0) * co0 + M_(0, 1) * co1 + M_(0, 2) * co2;
    double s = 1.0 / det;
    r[0] = co0 * s; r[1] = COF(0, 2, 2, 1) * s; r[2] = COF(0, 1, 1, 2) * s;
    r[3] = co1 * s; r[4] = COF(0, 0, 2, 2) * s; r[5] = COF(0, 2, 1, 0) * s;
    r[6] = co2 * s; r[7] = COF(0, 1, 2, 0) * s; r[8] = COF(0, 0, 1, 1) * s;
#undef COF
#undef M_
}

// One vector of CorrectHydrodynamicForces (SolidEntity.cpp:1266-1286) with
// btVector3::safeNormalize (btVector3.h:286-299).
__device__ void correct_one(const double* inv, double* vec, const double* C, double k)
{
    double w0 = inv[0] * vec[0] + inv[1] * vec[1] + inv[2] * vec[2];
    double w1 = inv[3] * vec[0] + inv[4] * vec[1] + inv[5] * vec[2];
    double w2 = inv[6] * vec[0] + inv[7] * vec[1] + inv[8] * vec[2];
    double l2 = w0 * w0 + w1 * w1 + w2 * w2;
    const double eps = 2.220446049250313080847e-16;   // DBL_EPSILON
    if (l2 >= eps * eps) {
        double s = 1.0 / sqrt(l2);
        w0 *= s; w1 *= s; w2 *= s;
    } else {
        w0 = 1.0; w1 = 0.0; w2 = 0.0;
    }
    double c = fabs(w0) * C[0] + fabs(w1) * C[1] + fabs(w2) * C[2];
    double f = k * c;
    vec[0] = f * vec[0]; vec[1] = f * vec[1]; vec[2] = f * vec[2];
}

__device__ void correct4(double density, double* Fdq, double* Tdq, double* Fdf, double* Tdf,
                         const double* Cd, const double* Cf, const double* R_O)
{
    double inv[9];
    binverse(R_O, inv);
    correct_one(inv, Fdq, Cd, 0.5 * density);
    correct_one(inv, Tdq, Cd, 0.5 * density);
    correct_one(inv, Fdf, Cf, density);
    correct_one(inv, Tdf, Cf, density);
}

__device__ __forceinline__ void set3(double* d, double x, double y, double z) { d[0] = x; d[1] = y; d[2] = z; }
__device__ __forceinline__ void zero3(double* d) { d[0] = 0.0; d[1] = 0.0; d[2] = 0.0; }
__device__ __forceinline__ void copy3(double* d, const double* s) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }

// Finalisation of the surface loop on FP64 sums (SolidEntity.cpp:1689-1720,
// the float steps carried out in FP64).
__device__ void finalize_surface(const OceanDev& o, int buoyancy, int damping,
                                 const double* T_CG_origin, double p0x, double p0y,
                                 const double* S, hydro_wrench& w)
{
    const double V6 = S[Q_V6];
    if (buoyancy && V6 > (double)1e-9f) {
        w.Vsub = V6 / 6.0;
        if (o.waves) {
            const double k = o.density * o.gravity;
            set3(w.Fb, S[Q_FB] * k, S[Q_FB + 1] * k, S[Q_FB + 2] * k);
            set3(w.Tb, S[Q_TB] * k, S[Q_TB + 1] * k, S[Q_TB + 2] * k);
        } else {
            double cb[3] = {S[Q_CB] / V6 + p0x, S[Q_CB + 1] / V6 + p0y, S[Q_CB + 2] / V6 + 0.0};
            double k = -w.Vsub * o.density;
            double f[3] = {0.0 * k, 0.0 * k, o.gravity * k};
            double r[3] = {cb[0] - T_CG_origin[0], cb[1] - T_CG_origin[1], cb[2] - T_CG_origin[2]};
            copy3(w.Fb, f);
            bcross(r, f, w.Tb);
        }
    }
    if (damping) {
        copy3(w.Fdq, S + Q_FDQ);
        copy3(w.Tdq, S + Q_TDQ);
        copy3(w.Fdf, S + Q_FDF);
        copy3(w.Tdf, S + Q_TDF);
    }
    w.Swet = S[Q_SWET];
}

// --------------------------------------------------------------- prologue
// Per-body FP32 parameters and loop kind (SolidEntity.cpp:1799-1846).
__device__ void body_prologue(const hydro_body* b, uint32_t batch_mesh, int op, const OceanDev& o,
                              SettingsDev st, int frame, BodyParams& B)
{
    int loop = LOOP_NONE, pos = HYDRO_SKIPPED, buoy = st.buoyancy, damp = st.damping;
    const int mismatch = (b->mesh != batch_mesh);
    if (op == OP_BODY) {
        if (!mismatch && (b->mode == HYDRO_MODE_FLOATING || b->mode == HYDRO_MODE_SUBMERGED)) {
            pos = classify(o, b->aabb_min, b->aabb_max);
            if (pos == HYDRO_INSIDE) {
                loop = damp ? LOOP_SUBMERGED : LOOP_NONE;
            } else if (pos == HYDRO_CROSSING_SURFACE) {
                loop = LOOP_SURFACE;
                buoy = buoy && (b->buoyancy != 0);
            }
        }
    } else if (op == OP_AERO_BODY) {
        // SolidEntity::ComputeAerodynamicForces(Atmosphere*) (:1852-1863)
        if (!mismatch && b->mode == HYDRO_MODE_AERODYNAMIC) {
            loop = LOOP_AERO;
            pos = HYDRO_OUTSIDE;   // any value but SKIPPED: outputs are written
        }
    } else if (op == OP_AERO) {
        if (!mismatch) {
            loop = LOOP_AERO;
            pos = HYDRO_OUTSIDE;
        }
    } else if (!mismatch) {
        loop = (op == OP_SURFACE) ? LOOP_SURFACE : LOOP_SUBMERGED;
        pos = (op == OP_SURFACE) ? HYDRO_CROSSING_SURFACE : HYDRO_INSIDE;
        if (op == OP_SUBMERGED) damp = 1;
    }
    if (batch_mesh == HYDRO_NO_MESH) loop = LOOP_NONE;
    // HYDRO_FRAME_CENTRED: translations relative to the CG's x and y rounded
    // to FP32, subtracted in FP64 before the cast, so that the face
    // arithmetic works on coordinates of the body's size instead of its
    // distance from the world origin.  HYDRO_FRAME_WORLD (default): the
    // reference's casts (glMatrixFromTransform, OpenGLDataStructs.cpp:148-165).
    const bool centred = frame == HYDRO_FRAME_CENTRED;
    const float ox = centred ? (float)b->T_CG.origin[0] : 0.f;
    const float oy = centred ? (float)b->T_CG.origin[1] : 0.f;
    const double shift[3] = {(double)ox, (double)oy, 0.0};
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) B.TC[4 * r + c] = (float)b->T_C.basis[3 * r + c];
        B.TC[4 * r + 3] = centred ? (float)(b->T_C.origin[r] - shift[r]) : (float)b->T_C.origin[r];
    }
    if (centred)
        B.p = mk((float)(b->T_CG.origin[0] - shift[0]), (float)(b->T_CG.origin[1] - shift[1]),
                 (float)b->T_CG.origin[2]);
    else
        B.p = mk((float)b->T_CG.origin[0], (float)b->T_CG.origin[1], (float)b->T_CG.origin[2]);
    B.p0 = mk(B.p.x, B.p.y, 0.f);
    B.off[0] = ox;
    B.off[1] = oy;
    B.centred = centred ? 1 : 0;
    B.v = mk((float)b->v[0], (float)b->v[1], (float)b->v[2]);
    B.omega = mk((float)b->omega[0], (float)b->omega[1], (float)b->omega[2]);
    B.loop = loop;
    B.buoyancy = buoy;
    B.damping = damp;
    B.position = pos;
    B.mismatch = mismatch;
}

// The CG origin in the frame of the body's FP32 parameters (FP64).
__device__ __forceinline__ void frame_origin(const hydro_body* b, const BodyParams& B, double* og)
{
    og[0] = B.centred ? b->T_CG.origin[0] - (double)B.off[0] : b->T_CG.origin[0];
    og[1] = B.centred ? b->T_CG.origin[1] - (double)B.off[1] : b->T_CG.origin[1];
    og[2] = b->T_CG.origin[2];
}

// CorrectAerodynamicForces (SolidEntity.cpp:1925-1956): both vectors scaled
// by |Cd . n|, n the force's direction in the proxy frame, Cd per
// approximation type.
__device__ void aero_correct(const hydro_aero_params& ap, double* Fda, double* Tda)
{
    double inv[9];
    binverse(ap.R_CG2H, inv);
    double n[3] = {inv[0] * Fda[0] + inv[1] * Fda[1] + inv[2] * Fda[2],
                   inv[3] * Fda[0] + inv[4] * Fda[1] + inv[5] * Fda[2],
                   inv[6] * Fda[0] + inv[7] * Fda[1] + inv[8] * Fda[2]};
    // btVector3::safeNormalize; btVector3::operator/= multiplies by 1 / s
    const double l2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
    const double eps = 2.220446049250313080847e-16;   // DBL_EPSILON
    if (l2 >= eps * eps) {
        const double s = 1.0 / sqrt(l2);
        n[0] *= s;
        n[1] *= s;
        n[2] *= s;
    } else {
        n[0] = 1.0;
        n[1] = 0.0;
        n[2] = 0.0;
    }
    double cor = 1.0;
    if (ap.approx_type == HYDRO_APPROX_CYLINDER) {
        cor = 0.5 * n[0] + 0.5 * n[1] + 1.0 * n[2];
    } else if (ap.approx_type == HYDRO_APPROX_ELLIPSOID) {
        double cd[3] = {1.0 / ap.approx_params[0], 1.0 / ap.approx_params[1], 1.0 / ap.approx_params[2]};
        const double mx = fmax(fmax(cd[0], cd[1]), cd[2]);   // btMax
        const double s = 1.0 / mx;
        cd[0] *= s;
        cd[1] *= s;
        cd[2] *= s;
        cor = cd[0] * n[0] + cd[1] * n[1] + cd[2] * n[2];
    }
    cor = fabs(cor);
    for (int k = 0; k < 3; ++k) {
        Fda[k] *= cor;
        Tda[k] *= cor;
    }
}

// Finalisation of the aerodynamic ops: Fda = 0.5 rho sum, Tda likewise
// (SolidEntity.cpp:1918-1922), then the correction for OP_AERO_BODY.
__device__ void aero_finalize(const KParams& P, uint32_t body, const BodyParams& B, const double* S, int status)
{
    hydro_aero_wrench w = P.aero_io[body];
    if (B.mismatch) {
        w.status = HYDRO_ERR_MISMATCH;
    } else if (B.position != HYDRO_SKIPPED) {
        const double k = 0.5 * P.ocean.density;
        for (int c = 0; c < 3; ++c) {
            w.Fda[c] = k * S[Q_FDQ + c];
            w.Tda[c] = k * S[Q_TDQ + c];
        }
        if (P.op == OP_AERO_BODY) aero_correct(P.aero_params[body], w.Fda, w.Tda);
        w.status = status;
    }
    P.aero_io[body] = w;
}

// Finalisation of one body from its FP64 sums S (kQ values).
// With `defer` set, the four damping vectors are written uncorrected and
// *correct tells whether CorrectHydrodynamicForces applies to them: each of
// them is then correct_one of its sum in S (zero sums for a null mesh).
__device__ void body_finalize(const KParams& P, uint32_t body, const BodyParams& B,
                              const double* S, int status, bool defer = false, bool* correct = nullptr)
{
    if (P.op == OP_AERO || P.op == OP_AERO_BODY) {
        aero_finalize(P, body, B, S, status);
        return;
    }
    const hydro_body* b = P.bodies + body;
    hydro_wrench w = P.io[body];
    const BodyInfo bi = P.binfo[body];
    const bool null_mesh = (bi.mesh == HYDRO_NO_MESH);
    if (B.mismatch) {
        w.status = HYDRO_ERR_MISMATCH;
        P.io[body] = w;
        return;
    }
    if (P.op == OP_SURFACE) {
        if (null_mesh) {          // mesh == nullptr (:1293-1312)
            if (B.buoyancy) { zero3(w.Fb); zero3(w.Tb); }
            if (B.damping) { zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf); }
            w.Swet = 0.0;
            w.Vsub = 0.0;
        } else {
            double og[3];
            frame_origin(b, B, og);
            finalize_surface(P.ocean, B.buoyancy, B.damping, og, (double)B.p0.x, (double)B.p0.y, S, w);
        }
    } else if (P.op == OP_SUBMERGED) {
        copy3(w.Fdq, S + Q_FDQ);
        copy3(w.Tdq, S + Q_TDQ);
        copy3(w.Fdf, S + Q_FDF);
        copy3(w.Tdf, S + Q_TDF);
    } else {
        w.position = B.position;
        if (B.position == HYDRO_SKIPPED) {
            // mode gate: outputs untouched (:1801)
        } else if (B.position == HYDRO_OUTSIDE) {
            zero3(w.Fb); zero3(w.Tb); zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf);
            w.Swet = 0.0;
            w.Vsub = 0.0;
        } else {
            if (B.position == HYDRO_INSIDE) {
                if (b->buoyancy) {       // :1831-1835
                    double k = -b->volume * P.ocean.density;
                    double f[3] = {0.0 * k, 0.0 * k, P.ocean.gravity * k};
                    const double* R = b->T_CG.basis;
                    const double* og = b->T_CG.origin;
                    const double* cb = b->P_CB;
                    double c[3] = {(R[0] * cb[0] + R[1] * cb[1] + R[2] * cb[2]) + og[0],
                                   (R[3] * cb[0] + R[4] * cb[1] + R[5] * cb[2]) + og[1],
                                   (R[6] * cb[0] + R[7] * cb[1] + R[8] * cb[2]) + og[2]};
                    double r[3] = {c[0] - og[0], c[1] - og[1], c[2] - og[2]};
                    copy3(w.Fb, f);
                    bcross(r, f, w.Tb);
                }
                if (B.damping) {
                    copy3(w.Fdq, S + Q_FDQ);
                    copy3(w.Tdq, S + Q_TDQ);
                    copy3(w.Fdf, S + Q_FDF);
                    copy3(w.Tdf, S + Q_TDF);
                }
                w.Swet = b->surface;
            } else if (null_mesh) {
                if (B.buoyancy) { zero3(w.Fb); zero3(w.Tb); }
                if (B.damping) { zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf); }
                w.Swet = 0.0;
                w.Vsub = 0.0;
            } else {
                double og[3];
                frame_origin(b, B, og);
                finalize_surface(P.ocean, B.buoyancy, B.damping, og, (double)B.p0.x, (double)B.p0.y, S, w);
            }
            if (B.damping) {
                if (defer) *correct = true;
                else correct4(P.ocean.density, w.Fdq, w.Tdq, w.Fdf, w.Tdf, b->Cd, b->Cf, b->R_O);
            }
        }
    }
    w.status = status;
    P.io[body] = w;
}

// ------------------------------------------------------------ reductions
// Butterfly reduce-scatter of 32 per-lane values: afterwards lane L holds
// the warp total of value L.  Fixed pairing, so the result is deterministic.
__device__ __forceinline__ float warp_reduce_scatter(float (&v)[32])
{
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
        const int half = 16 >> lvl;
        const bool upper = (lane & (unsigned)half) != 0u;
#pragma unroll
        for (int k = 0; k < half; ++k) {
            float send = upper ? v[k] : v[k + half];
            float keep = upper ? v[k + half] : v[k];
            float recv = __shfl_xor_sync(0xffffffffu, send, half);
            v[k] = keep + recv;
        }
    }
    return v[0];
}

// Knuth's TwoSum: hi + lo += x with the rounding error of the add kept.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x)
{
    float s = hi + x;
    float bb = s - hi;
    float err = (hi - (s - bb)) + (x - bb);
    hi = s;
    lo += err;
}

__device__ __forceinline__ void flush(Acc& a, float& hi, float& lo)
{
    float v[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = (k < kQ) ? a.q[k] : 0.f;
    float t = warp_reduce_scatter(v);
    two_sum_acc(hi, lo, t);
#pragma unroll
    for (int k = 0; k < kQ; ++k) a.q[k] = 0.f;
}

// ---------------------------------------------------- TMA / mbarrier PTX
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One try: true when the phase with `parity` has completed (the hardware
// may hold the thread for a short, implementation-defined time).
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: gives up (returns false) after about two seconds.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    return mbar_wait_for(bar, parity, kWaitLimitNs);
}

// The producer's wait for a free stage: it is ahead of the compute warps,
// so it sleeps between polls instead of taking their issue slots.
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity)
{
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        __nanosleep(200);
        if (global_ns() - t0 > kWaitLimitNs) return false;
    }
}

// 1-D bulk copy global -> shared (TMA), completion counted on `bar`.
__device__ __forceinline__ void tma_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(kBlock) : "memory");
}

// Barrier of the consumer warps that also ANDs a predicate across them, so
// that a wait that gave up in any thread is seen by all (no thread is left
// waiting at a later barrier).
__device__ __forceinline__ bool consumer_all(bool x)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)x), "n"(kBlock)
        : "memory");
    return r != 0u;
}

// ------------------------------------------------------------ prep kernel
// Requests the 128-byte lines part, part + parts, ... of [p, p + bytes) into
// L1: the per-body kernels read their records field by field behind
// branches, and the requests let those reads find the lines on the SM.
__device__ __forceinline__ void prefetch_lines(const void* p, size_t bytes, int part, int parts)
{
    const uintptr_t end = reinterpret_cast<uintptr_t>(p) + bytes;
    for (uintptr_t a = (reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)127) + 128u * (uintptr_t)part; a < end;
         a += 128u * (uintptr_t)parts)
        asm volatile("prefetch.global.L1 [%0];" ::"l"(a));
}

// Appends the chunks of a body that runs a face loop (`n` of them, 0 for a
// body without one or a lane without a body) to the launch's list of active
// chunks, each into the region of its claim class (its tile count), so that
// the producers never claim the chunks of bodies outside the water or
// switched off, and claim the largest chunks first.  Called by all 32 lanes
// of a warp.  A body's chunks are full (the work list's tiles per chunk)
// except its last: the warp's full chunks take one run of their class (one
// atomic, runs prefix-summed with shuffles, descriptors formed from the
// body's first chunk), the last chunks one atomic per class present.
__device__ __forceinline__ void list_chunks(const KParams& P, uint32_t body, const BodyInfo& bi, uint32_t n)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    const uint4* src = reinterpret_cast<const uint4*>(P.chunks + bi.first_chunk);
    uint4 d0 = make_uint4(0u, 0u, 0u, 0u), dl = d0;
    if (n > 0u) {
        d0 = __ldg(src);
        dl = n > 1u ? __ldg(src + (n - 1u)) : d0;
    }
    uint4* act = reinterpret_cast<uint4*>(P.active);
    // full chunks 0 .. n-2: the work lists give every full chunk of a batch
    // the same tile count, so the warp's full chunks form one run of one
    // class; a lane whose full chunks were of another class would place
    // them one atomic each
    const uint32_t nf = n > 1u ? n - 1u : 0u;
    const unsigned with_full = __ballot_sync(0xffffffffu, nf > 0u);
    if (with_full) {
        const uint32_t cf = claim_class(d0.z);
        const int leader = __ffs(with_full) - 1;
        const uint32_t cls = __shfl_sync(0xffffffffu, cf, leader);
        const bool in_run = nf > 0u && cf == cls;
        const uint32_t cnt = in_run ? nf : 0u;
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if ((int)lane >= d) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(P.n_listed + cls, total);
        base = __shfl_sync(0xffffffffu, base, leader) + incl - cnt;
        if (in_run) {
            for (uint32_t j = 0; j < nf; ++j)   // ActiveChunk{body, first_tile, n_tiles, chunk}
                act[P.class_start[cls] + base + j] = make_uint4(body, d0.y + j * d0.z, d0.z, bi.first_chunk + j);
        } else if (nf > 0u) {
            for (uint32_t j = 0; j < nf; ++j) {
                const uint4 dj = __ldg(src + j);
                const uint32_t c = claim_class(dj.z);
                act[P.class_start[c] + atomicAdd(P.n_listed + c, 1u)] =
                    make_uint4(body, dj.y, dj.z, bi.first_chunk + j);
            }
        }
    }
    // each body's last chunk
    const uint32_t cl = n > 0u ? claim_class(dl.z) : 0xFFFFFFFFu;
    const unsigned same = __match_any_sync(0xffffffffu, cl);
    const int leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (n > 0u && (int)lane == leader) base = atomicAdd(P.n_listed + cl, (uint32_t)__popc(same));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (n > 0u)
        act[P.class_start[cl] + base + __popc(same & lt)] = make_uint4(body, dl.y, dl.z, bi.first_chunk + n - 1u);
}

// One thread per body, grid-stride over the bodies to evaluate (the first
// *n_active of them when a device count is given).
__global__ void prep_kernel(const KParams P)
{
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) *P.err = 0u;
        if (threadIdx.x < (unsigned)kClaimClasses) P.work[threadIdx.x] = 0u;
    }
    const uint32_t limit = P.n_active ? min(P.n_bodies, *P.n_active) : P.n_bodies;
    // warp-uniform grid stride: every lane reaches list_chunks
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < limit; w0 += stride) {
        const uint32_t b = w0 + (threadIdx.x & 31u);
        BodyInfo bi{};
        uint32_t n = 0;
        if (b < limit) {
            prefetch_lines(P.bodies + b, sizeof(hydro_body), 0, 1);
            BodyParams B;
            bi = P.binfo[b];
            body_prologue(P.bodies + b, bi.mesh, P.op, P.ocean, P.st, P.frame, B);
            P.bparams[b] = B;
            n = B.loop != LOOP_NONE ? bi.n_chunks : 0u;
        }
        list_chunks(P, b, bi, n);
    }
}

// ------------------------------------------------------------ main kernel
// Persistent CTAs: warps 0..6 compute, warp 7 (one lane) streams the CTA's
// tiles into a ring of kStages shared-memory stages with 1-D TMA bulk
// copies.  The producer claims chunks from a global counter (reset by the
// prep kernel) and skips the chunks of bodies without a face loop; which CTA
// takes a chunk does not change the chunk's result.
constexpr int kStages = 4;
constexpr int kStageRaw = kTileVerts * 12 + kTileFaces * 4;   // 7168 bytes
constexpr int kThreads = kBlock + 32;
// Straddling faces wait in a per-warp queue until 32 of them (or the end of
// the chunk) fill one pass of the scalar clipping path: at most 31 wait
// while a tile adds up to 64.  The fully submerged faces of tiles that are
// not wholly under water wait likewise for 64 (one pass of pairs): at most
// 63 wait while a tile adds up to 64.
constexpr int kCutQueue = 96;
constexpr int kPairQueue = 127;

__device__ __forceinline__ int wrap_queue(int x)
{
    x = x >= kCutQueue ? x - kCutQueue : x;
    return x >= kCutQueue ? x - kCutQueue : x;
}

__device__ __forceinline__ int wrap_pair_queue(int x) { return x >= kPairQueue ? x - kPairQueue : x; }

enum : int { ITEM_FIRST = 1, ITEM_LAST = 2, ITEM_END = 4 };

struct ItemMeta {
    uint32_t chunk;
    int flags;
    uint16_t nv, nf;
    uint32_t pad;
};

struct __align__(128) StageBuf {
    BodyParams bp;
    unsigned char raw[kStageRaw];
};

struct __align__(128) ChunkSmem {
    StageBuf stage[kStages];
    float4 verts[2][kTileVerts];      // transformed vertices, double-buffered
    uint32_t tflags[2][8];            // per-warp vertex votes of each vertex buffer (bit 0 above, bit 1 under)
    static_assert(kWarps <= 8, "one vote slot per compute warp");
    float2 red[kWarps][32];
    float4 cutq[kWarps][kCutQueue][3];  // per-warp queues of straddling faces (corners with depth)
    float pairq[kWarps][kPairQueue * 9]; // per-warp queues of fully submerged faces (corner positions)
    ItemMeta meta[kStages];
    uint64_t full[kStages];
    uint64_t empty[kStages];
};

size_t chunk_kernel_smem() { return sizeof(ChunkSmem); }

// Whether the tile a producer lane describes is streamed.  On a flat
// surface a tile of a surface-loop body that lies wholly above the water
// (every vertex at depth < 0, so every face is skipped, SolidEntity.cpp:
// 1353-1354) is not loaded at all.  The highest vertex of the tile is bounded
// by its centre's height plus the smaller of two reaches along the row of
// T_C that gives z: the bounding sphere's radius times the row's norm (2^-20
// covers its FP32 evaluation) and the box's half extents weighted by the
// row's magnitudes.  The margin bounds the consumer's FP32 transform of each
// vertex far above its rounding error.
__device__ __forceinline__ bool tile_above_water(const float4 T, const TileDesc* d)
{
    const float ax = fabsf(T.x), ay = fabsf(T.y), az = fabsf(T.z);
    const float rn = sqrtf((T.x * T.x + T.y * T.y) + T.z * T.z) * (1.f + 0x1p-20f);
    const float4 c = __ldg(&d->sphere), h = __ldg(&d->half);
    const float zc = (T.x * c.x + T.y * c.y) + (T.z * c.z + T.w);
    const float reach = fminf(c.w * rn, (ax * h.x + ay * h.y) + az * h.z);
    const float margin = 1e-5f * ((ax * (fabsf(c.x) + h.x) + ay * (fabsf(c.y) + h.y)) +
                                  (az * (fabsf(c.z) + h.z) + fabsf(T.w))) + 1e-6f;
    return zc + reach + margin < 0.f;
}

// The producer warp.  Lane 0 claims chunks and issues the copies; for each
// chunk, lane t reads tile t's descriptor and tests it against the surface,
// so a chunk's tiles are described in one round trip.
__device__ __forceinline__ void producer(const KParams& P, ChunkSmem& S)
{
    const uint32_t lane = threadIdx.x & 31u;
    constexpr unsigned kAll = 0xffffffffu;
    uint32_t item = 0;
    bool ok = true;
    // Claims go class by class, largest chunks first: lane 0 moves to the
    // next class once its claim in the current one comes back past the
    // class's listed count.  They run one chunk ahead so that the atomic's
    // latency overlaps work; the list holds only chunks whose body runs a
    // face loop.
    uint32_t cls = 0;
    auto claim = [&]() -> uint32_t {
        uint32_t r = 0xFFFFFFFFu;
        if (lane == 0u) {
            while (cls < (uint32_t)kClaimClasses) {
                const uint32_t listed = min(P.n_listed[cls], P.class_start[cls + 1] - P.class_start[cls]);
                if (listed != 0u) {
                    const uint32_t i = atomicAdd(P.work + cls, 1u);
                    if (i < listed) {
                        r = P.class_start[cls] + i;
                        break;
                    }
                }
                ++cls;
            }
        }
        return __shfl_sync(kAll, r, 0);
    };
    uint32_t next = claim();
    while (ok && next != 0xFFFFFFFFu) {
        const ActiveChunk ch = P.active[next];
        next = claim();
        const uint32_t nt = ch.n_tiles < (uint32_t)kMaxTilesPerChunk ? ch.n_tiles : (uint32_t)kMaxTilesPerChunk;
        // the body's loop kind and z row, and this lane's tile
        const BodyParams* B = P.bparams + ch.body;
        const int loop = B->loop;
        const float4 T = *reinterpret_cast<const float4*>(B->TC + 8);   // row giving z
        const float* block = nullptr;
        uint32_t sizes = 0u;   // nv | nf << 16
        bool dry = false;
        if (lane < nt) {
            const TileDesc* d = P.tiles + ch.first_tile + lane;
            block = d->block;
            sizes = (uint32_t)d->nv | ((uint32_t)d->nf << 16);
            dry = !P.ocean.waves && tile_above_water(T, d);
        }
        const uint32_t all = nt >= 32u ? kAll : (1u << nt) - 1u;
        uint32_t keep = all;
        if (loop == LOOP_SURFACE) {
            keep &= ~__ballot_sync(kAll, dry);
            if (keep == 0u) keep = all & 1u;   // a chunk keeps one tile, which carries its (zero) partial
        }
        const uint32_t first_kept = (uint32_t)(__ffs(keep) - 1);
        const uint32_t last_kept = 31u - (uint32_t)__clz(keep);
        for (uint32_t rest = keep; rest != 0u; rest &= rest - 1u) {
            const uint32_t t = (uint32_t)(__ffs(rest) - 1);
            const uint64_t blk = __shfl_sync(kAll, (unsigned long long)reinterpret_cast<uintptr_t>(block), t);
            const uint32_t sz = __shfl_sync(kAll, sizes, t);
            if (lane == 0u) {
                const int s = (int)(item % kStages);
                if (item >= (uint32_t)kStages && !mbar_wait_sleep(&S.empty[s], ((item / kStages) - 1u) & 1u)) {
                    atomicOr(P.err, 1u);
                    ok = false;
                } else {
                    const uint32_t nv = sz & 0xFFFFu, nf = sz >> 16;
                    const uint32_t bytes = tile_bytes(nv, nf);
                    ItemMeta m;
                    m.chunk = ch.chunk;
                    m.flags = (t == first_kept ? ITEM_FIRST : 0) | (t == last_kept ? ITEM_LAST : 0);
                    m.nv = (uint16_t)nv;
                    m.nf = (uint16_t)nf;
                    m.pad = 0;
                    S.meta[s] = m;
                    mbar_arrive_expect_tx(&S.full[s], bytes + (uint32_t)sizeof(BodyParams));
                    tma_copy(&S.stage[s].bp, P.bparams + ch.body, (uint32_t)sizeof(BodyParams), &S.full[s]);
                    tma_copy(S.stage[s].raw, reinterpret_cast<const float*>(blk), bytes, &S.full[s]);
                }
            }
            ok = __shfl_sync(kAll, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            ++item;
        }
    }
    if (lane != 0u) return;
    // end of stream
    const int s = (int)(item % kStages);
    if (item >= (uint32_t)kStages && !mbar_wait_sleep(&S.empty[s], ((item / kStages) - 1u) & 1u)) {
        atomicOr(P.err, 1u);
    }
    ItemMeta m{0u, ITEM_END, 0, 0, 0u};
    S.meta[s] = m;
    mbar_arrive(&S.full[s]);
    // Stay until every copy this thread issued has landed (bounded).  Item
    // item - kStages shares its stage with the end marker, whose arrive has
    // already moved that barrier one phase further, and was consumed before
    // the end marker could be armed, so it is skipped.
    const uint32_t first = item >= (uint32_t)kStages ? item - (uint32_t)kStages + 1u : 0u;
    for (uint32_t i = first; i < item; ++i)
        if (!mbar_wait_sleep(&S.full[i % kStages], (i / kStages) & 1u)) atomicOr(P.err, 1u);
}

// Transforms the vertices of the tile in stage `st` into `out` (x, y, z,
// depth), each vertex once, and records per warp whether any of its
// vertices is above water (depth < 0, bit 0) or not (bit 1).
template <bool WAVES>
__device__ __forceinline__ void transform_tile(const KParams& P, const StageBuf& st, const ItemMeta& m,
                                               float4* out, uint32_t* flags)
{
    const float* raw = reinterpret_cast<const float*>(st.raw);
    const int nv = m.nv, nvp = (nv + 3) & ~3;
    float TC[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) TC[k] = st.bp.TC[k];
    bool above = false, under = false;
    for (int v = threadIdx.x; v < nv; v += kBlock) {
        v3 p = xform(TC, raw[v], raw[nvp + v], raw[2 * nvp + v]);
        float d = WAVES ? depth_at_b(P.ocean, st.bp, p.x, p.y, p.z) : p.z;
        out[v] = make_float4(p.x, p.y, p.z, d);
        above |= d < 0.f;
        under |= !(d < 0.f);
    }
    const unsigned a = __ballot_sync(0xffffffffu, above), u = __ballot_sync(0xffffffffu, under);
    if ((threadIdx.x & 31) == 0) flags[threadIdx.x >> 5] = (a ? 1u : 0u) | (u ? 2u : 0u);
}

// Per-warp queues: head slot and length (warp-uniform).
struct CutQueue {
    float4 (*q)[3];
    int head, len;
};

struct PairQueue {
    float* q;   // kPairQueue entries of 9 floats: x, y, z of the three corners
    int head, len;
};

// Faces of one tile.  A tile wholly under water is evaluated directly, two
// faces per lane on the packed path; in other tiles each face is classified
// and queued: fully submerged faces in the warp's pair queue, straddling
// faces in its clipping queue.  The queues run a pass when full enough for
// all 32 lanes (64 paired faces, 32 straddling faces) or when `drain` (the
// chunk's last tile).  Returns the number of faces each lane added at most
// (a pair pass counts two, a clipping pass one).
template <bool CUT64, bool WAVES, bool AERO, bool FIELD>
__device__ __forceinline__ int tile_faces(const KParams& P, const StageBuf& st, const ItemMeta& m,
                                          const float4* verts, const uint32_t* flags, PairQueue& pq,
                                          CutQueue& cq, bool drain, Acc& acc)
{
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // the body's vectors and flags as four 16-byte loads (BodyParams bytes 48..111)
    const float4* bq = reinterpret_cast<const float4*>(&st.bp) + 3;
    const float4 q0 = bq[0], q1 = bq[1], q2 = bq[2];
    const int4 fl = *reinterpret_cast<const int4*>(bq + 3);
    BodyParams Bl;
    Bl.p = mk(q0.x, q0.y, q0.z);
    Bl.p0 = mk(q0.w, q1.x, q1.y);
    Bl.v = mk(q1.z, q1.w, q2.x);
    Bl.omega = mk(q2.y, q2.z, q2.w);
    Bl.loop = fl.x; Bl.buoyancy = fl.y; Bl.damping = fl.z;
    Bl.centred = 0;
    if (WAVES || FIELD) {      // the frame offset, bytes 112..127
        const float4 q3 = bq[4];
        Bl.off[0] = q3.y;
        Bl.off[1] = q3.z;
        Bl.centred = __float_as_int(q3.w);
    }
    const int nf = m.nf, nvp = (m.nv + 3) & ~3;
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(reinterpret_cast<const float*>(st.raw) + 3 * nvp);
    if (AERO) {
        // every face, one per lane, on the scalar path (no clipping); an
        // aerodynamic launch lists only bodies of the aerodynamic loop
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int f = (k * 32 + lane) * kWarps + warp;
            if (f < nf) {
                const uint32_t w = idx[f];
                const float4 q1 = verts[w & 511u];
                const float4 q2 = verts[(w >> 9) & 511u];
                const float4 q3 = verts[w >> 18];
                face_aero<FIELD>(P.ocean, Bl, acc, mk(q1.x, q1.y, q1.z), mk(q2.x, q2.y, q2.z),
                                 mk(q3.x, q3.y, q3.z));
            }
        }
        return 2;
    }
    int added = 0;
    // Tiles of the surface loop wholly on one side of the surface: above
    // water every face is skipped (:1353-1354), under water every face is
    // fully submerged, as in the submerged loop.
    bool all_under = Bl.loop != LOOP_SURFACE, any_under = true;
    if (!all_under) {
        const uint4 f0 = *reinterpret_cast<const uint4*>(flags);
        const uint4 f1 = *reinterpret_cast<const uint4*>(flags + 4);
        const uint32_t tf = f0.x | f0.y | f0.z | f0.w | f1.x | f1.y | f1.z | f1.w;
        all_under = !(tf & 1u);
        any_under = (tf & 2u) != 0u;
    }
    // Warp w takes faces (k*32 + lane)*kWarps + w, k = 0, 1: a spread sample
    // of the tile, so that the warps get similar work.
    int direct = 0;   // faces of the direct pass: lane l pairs faces l*kWarps + w and (l+32)*kWarps + w
    if (all_under) {
        direct = nf > warp ? min(64, (nf - warp + kWarps - 1) / kWarps) : 0;
    } else if (any_under) {
        const unsigned lt = (1u << lane) - 1u;
        int nq = 0, nc = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int f = (k * 32 + lane) * kWarps + warp;
            int cls = 0;
            // the three corners are read once, whole: their depths classify
            // the face and their positions fill the queue entry
            float4 c1 = make_float4(0.f, 0.f, 0.f, 0.f), c2 = c1, c3 = c1;
            if (f < nf) {
                const uint32_t w = idx[f];
                c1 = verts[w & 511u];
                c2 = verts[(w >> 9) & 511u];
                c3 = verts[w >> 18];
                cls = face_class(c1.w, c2.w, c3.w);
            }
            const unsigned mf = __ballot_sync(0xffffffffu, cls == 1);
            const unsigned mc = __ballot_sync(0xffffffffu, cls == 2);
            if (cls == 1) {
                float* e = pq.q + 9 * wrap_pair_queue(pq.head + pq.len + nq + __popc(mf & lt));
                e[0] = c1.x; e[1] = c1.y; e[2] = c1.z;
                e[3] = c2.x; e[4] = c2.y; e[5] = c2.z;
                e[6] = c3.x; e[7] = c3.y; e[8] = c3.z;
            }
            if (cls == 2) {
                float4* e = cq.q[wrap_queue(cq.head + cq.len + nc + __popc(mc & lt))];
                e[0] = c1;
                e[1] = c2;
                e[2] = c3;
            }
            nq += __popc(mf);
            nc += __popc(mc);
        }
        pq.len += nq;
        cq.len += nc;
        __syncwarp();
    }
    // pair passes: the direct pass of a tile wholly under water, then the
    // queue's passes (one call site for the packed arithmetic)
    for (;;) {
        int n;
        bool from_queue;
        if (direct > 0) {
            n = direct;
            from_queue = false;
            direct = 0;
        } else if (pq.len >= 64 || (drain && pq.len > 0)) {
            n = pq.len < 64 ? pq.len : 64;
            from_queue = true;
        } else {
            break;
        }
        if (lane < n) {
            const bool hasB = lane + 32 < n;
            P3 p1, p2, p3;
            if (!from_queue) {
                const int fa = lane * kWarps + warp, fb = (lane + 32) * kWarps + warp;
                const uint32_t wa = idx[fa];
                const uint32_t wb = idx[hasB ? fb : fa];
                p1 = corners(verts[wa & 511u], verts[wb & 511u]);
                p2 = corners(verts[(wa >> 9) & 511u], verts[(wb >> 9) & 511u]);
                p3 = corners(verts[wa >> 18], verts[wb >> 18]);
            } else {
                const float* a = pq.q + 9 * wrap_pair_queue(pq.head + lane);
                const float* b = pq.q + 9 * wrap_pair_queue(pq.head + (hasB ? lane + 32 : lane));
                p1 = pk(f2(a[0], b[0]), f2(a[1], b[1]), f2(a[2], b[2]));
                p2 = pk(f2(a[3], b[3]), f2(a[4], b[4]), f2(a[5], b[5]));
                p3 = pk(f2(a[6], b[6]), f2(a[7], b[7]), f2(a[8], b[8]));
            }
            const BodyPair Bp = body_pair(Bl, P.ocean);
            if (Bl.loop == LOOP_SURFACE) face_full2<WAVES, FIELD>(P.ocean, Bl, Bp, acc, p1, p2, p3, hasB);
            else face_submerged2<FIELD>(P.ocean, Bl, Bp, acc, p1, p2, p3, hasB);
        }
        if (from_queue) {
            pq.head = wrap_pair_queue(pq.head + n);
            pq.len -= n;
        }
        added += 2;
        __syncwarp();
    }
    while (cq.len >= 32 || (drain && cq.len > 0)) {
        const int n = cq.len < 32 ? cq.len : 32;
        if (lane < n) {
            const float4* e = cq.q[wrap_queue(cq.head + lane)];
            const float4 q1 = e[0], q2 = e[1], q3 = e[2];
            face_cut<CUT64, WAVES, false, FIELD>(P.ocean, Bl, acc, mk(q1.x, q1.y, q1.z), mk(q2.x, q2.y, q2.z),
                                   mk(q3.x, q3.y, q3.z), q1.w, q2.w, q3.w);
        }
        cq.head = wrap_queue(cq.head + n);
        cq.len -= n;
        ++added;
        __syncwarp();
    }
    return added;
}

// Compute warps.  Iteration i evaluates the faces of tile i and transforms
// the vertices of tile i + 1 into the other vertex buffer; one barrier (which
// also checks that every thread's wait for tile i + 1 succeeded) separates
// iterations, so a warp that finishes its faces early starts transforming.
template <bool CUT64, bool WAVES, bool AERO, bool FIELD>
__device__ __forceinline__ void consumer(const KParams& P, ChunkSmem& S)
{
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    Acc acc;
#pragma unroll
    for (int k = 0; k < kQ; ++k) acc.q[k] = 0.f;
    float hi = 0.f, lo = 0.f;
    // A tile adds at most seven faces to a lane's run: two pair passes (a
    // direct or queued pass and the drain) and three clipping passes (up to
    // 95 queued faces, the last pass a drain), so a flush once a run has
    // passed kFlushFaces - 7 keeps every FP32 run at or below kFlushFaces
    // faces.
    int run = 0;
    CutQueue cq{S.cutq[warp], 0, 0};
    PairQueue pq{S.pairq[warp], 0, 0};

    // first tile
    bool ok = mbar_wait(&S.full[0], 0u);
    ItemMeta m = S.meta[0];
    if (ok && !(m.flags & ITEM_END)) transform_tile<WAVES>(P, S.stage[0], m, S.verts[0], S.tflags[0]);
    if (!consumer_all(ok)) {
        if (tid == 0) atomicOr(P.err, 1u);
        return;
    }
    for (uint32_t item = 0; !(m.flags & ITEM_END); ++item) {
        const int s = (int)(item % kStages);
        const bool last = (m.flags & ITEM_LAST) != 0;
        run += tile_faces<CUT64, WAVES, AERO, FIELD>(P, S.stage[s], m, S.verts[item & 1u], S.tflags[item & 1u], pq, cq,
                                                     last,
                                        acc);
        // next tile: wait, read its metadata, transform its vertices
        const uint32_t nx = item + 1u;
        const int sn = (int)(nx % kStages);
        ok = mbar_wait(&S.full[sn], (nx / kStages) & 1u);
        const ItemMeta mn = S.meta[sn];
        if (ok && !(mn.flags & ITEM_END))
            transform_tile<WAVES>(P, S.stage[sn], mn, S.verts[nx & 1u], S.tflags[nx & 1u]);
        if (!consumer_all(ok)) {
            if (tid == 0) atomicOr(P.err, 1u);
            return;
        }
        if (tid == 0) mbar_arrive(&S.empty[s]);
        if (last || run > kFlushFaces - 7) {
            flush(acc, hi, lo);
            run = 0;
        }
        if (last) {
            S.red[warp][lane] = make_float2(hi, lo);
            consumer_sync();
            if (warp == 0) {
                float H = S.red[0][lane].x, L = S.red[0][lane].y;
                for (int w = 1; w < kWarps; ++w) {
                    two_sum_acc(H, L, S.red[w][lane].x);
                    L += S.red[w][lane].y;
                }
                double* part = P.partials + (size_t)m.chunk * kPartialStride;
                if (lane < kQ) part[lane] = (double)H + (double)L;
                else if (lane == kQ) part[lane] = 0.0;
            }
            hi = 0.f;
            lo = 0.f;
            consumer_sync();
        }
        m = mn;
    }
}

// MINB = 2: two CTAs of eight warps per SM put four warps on each SM
// sub-partition, whose 16K registers then allow 128 per thread.  The cap is
// given as a register limit rather than a minimum block count, with which
// ptxas allocates the flat-surface variants without spills.
// AERO: an aerodynamic launch (every listed body in the aerodynamic loop);
// FIELD: jet or pipe currents are enabled.  The hydrodynamic variants carry
// no aerodynamic code, the aerodynamic ones no clipping or wave code, and
// those without field currents no FP64 current code, which keeps each
// one's instruction footprint small.
template <bool CUT64, bool WAVES, bool AERO, bool FIELD, int MINB>
__global__ void __launch_bounds__(kThreads) __maxnreg__(MINB == 2 ? 128 : 255) chunk_kernel(const KParams P)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    ChunkSmem& S = *reinterpret_cast<ChunkSmem*>(smem_raw);
    if (threadIdx.x < 16) (&S.tflags[0][0])[threadIdx.x] = 0u;   // slots of absent warps stay 0
    const int tid = threadIdx.x;
    if (tid == kBlock) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&S.full[s], 1u);
            mbar_init(&S.empty[s], 1u);
        }
        mbar_fence_init();
    }
    __syncthreads();
    if (tid >= kBlock) {
        producer(P, S);
        return;
    }
    consumer<CUT64, WAVES, AERO, FIELD>(P, S);
}

// ----------------------------------------------------------- finalise kernel
// Four threads per body.  GB300 executes FP64 at about two lanes per clock
// per SM and the finalisation is a chain of dependent FP64 operations, so
// the work of a body is split: thread k of the group adds quantities
// k, k + 4, ... of the chunk partials in chunk order, thread 0 finalises,
// and threads 0..3 apply CorrectHydrodynamicForces to one damping vector
// each (SolidEntity.cpp:1263-1287).  Warp-sized CTAs spread the bodies over
// all SMs.
constexpr int kBodyThreads = 32;
constexpr int kFinSub = 4;

__global__ void __launch_bounds__(kBodyThreads) finalize_kernel(const KParams P)
{
    constexpr uint32_t kPerCta = kBodyThreads / kFinSub;
    __shared__ double sums[kPerCta][kPartialStride];
    const int sub = (int)(threadIdx.x % kFinSub), slot = (int)(threadIdx.x / kFinSub);
    const int lane = (int)(threadIdx.x & 31u);
    if (blockIdx.x == 0 && threadIdx.x < (unsigned)kClaimClasses)
        P.n_listed[threadIdx.x] = 0u;   // the chunk kernel has finished with them
    const uint32_t limit = P.n_active ? min(P.n_bodies, *P.n_active) : P.n_bodies;
    // grid-stride over groups of kPerCta bodies (uniform across the warp)
    for (uint32_t base = blockIdx.x * kPerCta; base < limit; base += gridDim.x * kPerCta) {
        const uint32_t body = base + (uint32_t)slot;
        const bool live = body < limit;
        if (live && P.op != OP_AERO && P.op != OP_AERO_BODY) {
            prefetch_lines(P.bodies + body, sizeof(hydro_body), sub, kFinSub);
            prefetch_lines(P.io + body, sizeof(hydro_wrench), sub, kFinSub);
        }
        BodyParams B{};
        if (live) {
            B = P.bparams[body];
            const BodyInfo bi = P.binfo[body];
            // quantities sub, sub + 4, ...: each summed in chunk order from
            // +0, all of a chunk's loads in flight together
            constexpr int kPer = (kQ + kFinSub - 1) / kFinSub;
            double s[kPer];
#pragma unroll
            for (int i = 0; i < kPer; ++i) s[i] = 0.0;
            if (B.loop != LOOP_NONE) {
                const double* p = P.partials + (size_t)bi.first_chunk * kPartialStride + sub;
#pragma unroll 2
                for (uint32_t c = 0; c < bi.n_chunks; ++c, p += kPartialStride) {
#pragma unroll
                    for (int i = 0; i < kPer; ++i)
                        if (sub + kFinSub * i < kQ) s[i] += p[kFinSub * i];
                }
            }
#pragma unroll
            for (int i = 0; i < kPer; ++i)
                if (sub + kFinSub * i < kQ) sums[slot][sub + kFinSub * i] = s[i];
        }
        __syncwarp();
        bool correct = false;
        if (live && sub == 0) {
            const int status = (*P.err & 1u) ? HYDRO_ERR_TIMEOUT : 0;
            body_finalize(P, body, B, sums[slot], status, true, &correct);
        }
        correct = __shfl_sync(0xffffffffu, correct ? 1 : 0, lane & ~(kFinSub - 1)) != 0;
        __syncwarp();                  // thread 0's record is written before the corrected vectors
        if (live && correct) {
            const hydro_body* b = P.bodies + body;
            double inv[9], v[3];
            binverse(b->R_O, inv);
            copy3(v, sums[slot] + Q_FDQ + 3 * sub);
            correct_one(inv, v, sub < 2 ? b->Cd : b->Cf, sub < 2 ? 0.5 * P.ocean.density : P.ocean.density);
            hydro_wrench& w = P.io[body];
            double* dst = sub == 0 ? w.Fdq : sub == 1 ? w.Tdq : sub == 2 ? w.Fdf : w.Tdf;
            copy3(dst, v);
        }
        __syncwarp();                  // sums are reused by the next group
    }
}

template <int MINB, bool FIELD>
static void* kernel_ptr_f(int cut64, int waves, int aero)
{
    if (aero) return (void*)chunk_kernel<false, false, true, FIELD, MINB>;
    if (cut64)
        return waves ? (void*)chunk_kernel<true, true, false, FIELD, MINB>
                     : (void*)chunk_kernel<true, false, false, FIELD, MINB>;
    return waves ? (void*)chunk_kernel<false, true, false, FIELD, MINB>
                 : (void*)chunk_kernel<false, false, false, FIELD, MINB>;
}

template <int MINB>
static void* kernel_ptr(int cut64, int waves, int aero, int field)
{
    return field ? kernel_ptr_f<MINB, true>(cut64, waves, aero) : kernel_ptr_f<MINB, false>(cut64, waves, aero);
}

// The kernel variant compiled for `ctas_per_sm` resident CTAs (1 or 2).
static void* chunk_kernel_for(int cut64, int waves, int ctas_per_sm, int aero, int field)
{
    return ctas_per_sm >= 2 ? kernel_ptr<2>(cut64, waves, aero, field) : kernel_ptr<1>(cut64, waves, aero, field);
}

// The dynamic shared-memory attribute and the resident-CTA count of each
// chunk-kernel variant, set and queried once per device: both are host API
// calls that would otherwise sit in front of every step's first launch.
// Index: device (first 16), cut64, waves, aerodynamic, field currents, 1 or
// 2 CTAs per SM; occupancy is stored plus one (0 = not yet known).
constexpr int kDevCache = 16;
static std::atomic<int> g_chunk_occ[kDevCache][2][2][2][2][2];
static std::atomic<bool> g_chunk_attr[kDevCache][2][2][2][2][2];

static cudaError_t chunk_kernel_attr(int cut64, int waves, int ctas_per_sm, int aero, int field)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::atomic<bool>* flag = dev < kDevCache
        ? &g_chunk_attr[dev][cut64 != 0][waves != 0][aero != 0][field != 0][ctas_per_sm >= 2] : nullptr;
    if (flag && flag->load(std::memory_order_acquire)) return cudaSuccess;
    e = cudaFuncSetAttribute(chunk_kernel_for(cut64, waves, ctas_per_sm, aero, field),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ChunkSmem));
    if (e == cudaSuccess && flag) flag->store(true, std::memory_order_release);
    return e;
}

int chunk_kernel_occupancy(int cut64, int waves, int ctas_per_sm, int aero, int field)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::atomic<int>* slot = dev < kDevCache
        ? &g_chunk_occ[dev][cut64 != 0][waves != 0][aero != 0][field != 0][ctas_per_sm >= 2] : nullptr;
    if (slot) {
        const int known = slot->load(std::memory_order_acquire);
        if (known > 0) return known - 1;
    }
    int n = 0;
    const void* k = chunk_kernel_for(cut64, waves, ctas_per_sm, aero, field);
    if (chunk_kernel_attr(cut64, waves, ctas_per_sm, aero, field) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kThreads, sizeof(ChunkSmem)) != cudaSuccess)
        return 0;
    if (slot) slot->store(n + 1, std::memory_order_release);
    return n;
}

cudaError_t launch_step(const KParams& P, LaunchShape shape, int cut64, cudaStream_t s,
                        uint32_t* launches, cudaEvent_t* ev)
{
    *launches = 0;
    if (P.n_bodies == 0) return cudaSuccess;
    cudaError_t e;
    if (ev && (e = cudaEventRecord(ev[0], s))) return e;
    // per-body kernels: at most eight warp-sized CTAs per SM, grid-stride
    // beyond (a device count may leave most of a large batch idle)
    const uint32_t cap = 8u * (uint32_t)std::max(1, shape.grid / std::max(1, shape.ctas_per_sm));
    prep_kernel<<<std::min((P.n_bodies + kBodyThreads - 1) / kBodyThreads, cap), kBodyThreads, 0, s>>>(P);
    if ((e = cudaGetLastError())) return e;
    if (ev && (e = cudaEventRecord(ev[1], s))) return e;
    int grid = shape.grid;
    if (grid > (int)P.n_chunks) grid = (int)P.n_chunks;
    if (grid < 1) grid = 1;
    const int aero = (P.op == OP_AERO || P.op == OP_AERO_BODY) ? 1 : 0;
    const int field = P.ocean.field_currents ? 1 : 0;
    const void* k = chunk_kernel_for(cut64, P.ocean.waves != 0, shape.ctas_per_sm, aero, field);
    if ((e = chunk_kernel_attr(cut64, P.ocean.waves != 0, shape.ctas_per_sm, aero, field))) return e;
    void* args[] = {const_cast<KParams*>(&P)};
    if ((e = cudaLaunchKernel(k, dim3(grid), dim3(kThreads), args, sizeof(ChunkSmem), s))) return e;
    if (ev && (e = cudaEventRecord(ev[2], s))) return e;
    finalize_kernel<<<std::min((P.n_bodies + kBodyThreads / kFinSub - 1) / (kBodyThreads / kFinSub), cap),
                      kBodyThreads, 0, s>>>(P);
    if ((e = cudaGetLastError())) return e;
    if (ev && (e = cudaEventRecord(ev[3], s))) return e;
    *launches = 3;
    return cudaSuccess;
}

// ------------------------------------------------------------- compounds
// Compound::ComputeHydrodynamicForces (Compound.cpp:291-436).  The parts are
// the bodies of the chunk kernel: each part's faces are integrated about the
// compound's CG with the compound's velocities, in the part's mesh frame.

__device__ __forceinline__ bool fluid_mode(int m) { return m == HYDRO_MODE_FLOATING || m == HYDRO_MODE_SUBMERGED; }

// Loop kind and flags of one part for the compound's fluid position.
__device__ void compound_part_loop(int pos, const hydro_compound_part& pt, SettingsDev st, int& loop, int& buoy,
                                   int& damp)
{
    loop = LOOP_NONE;
    buoy = 0;
    damp = 0;
    if (!fluid_mode(pt.mode)) return;
    if (pos == HYDRO_INSIDE) {                                   // :331-353
        if (st.damping && pt.external) {
            loop = LOOP_SUBMERGED;
            damp = 1;
        }
    } else if (pos == HYDRO_CROSSING_SURFACE && (st.buoyancy || st.damping)) {   // :359-434
        const int pb = st.buoyancy && pt.buoyant;
        if (pt.external) {
            loop = LOOP_SURFACE;
            buoy = pb;
            damp = st.damping;
        } else if (pb) {
            loop = LOOP_SURFACE;
            buoy = 1;
        }
    }
}

// One thread per part (warp-sized CTAs; every lane reaches list_chunks).
__global__ void compound_prep_kernel(const KParams P, const CompoundParams C)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *P.err = 0u;
    if (p < (uint32_t)kClaimClasses) P.work[p] = 0u;
    BodyInfo part_info{};
    uint32_t n = 0;
    if (p < P.n_bodies) {
        const hydro_compound_part& pt = C.parts[p];
        const hydro_body& cb = C.compounds[C.part_compound[p]];
        int pos = HYDRO_SKIPPED;
        if (fluid_mode(cb.mode)) pos = classify(P.ocean, cb.aabb_min, cb.aabb_max);   // :293, :299
        int loop, buoy, damp;
        compound_part_loop(pos, pt, P.st, loop, buoy, damp);
        const BodyInfo bi = P.binfo[p];
        BodyParams B;
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) B.TC[4 * r + c] = (float)pt.T_C.basis[3 * r + c];
            B.TC[4 * r + 3] = (float)pt.T_C.origin[r];
        }
        B.p = mk((float)cb.T_CG.origin[0], (float)cb.T_CG.origin[1], (float)cb.T_CG.origin[2]);
        B.p0 = mk(B.p.x, B.p.y, 0.f);
        B.v = mk((float)cb.v[0], (float)cb.v[1], (float)cb.v[2]);
        B.omega = mk((float)cb.omega[0], (float)cb.omega[1], (float)cb.omega[2]);
        B.mismatch = (pt.mesh != bi.mesh);
        B.loop = (B.mismatch || bi.mesh == HYDRO_NO_MESH) ? LOOP_NONE : loop;
        B.buoyancy = buoy;
        B.damping = damp;
        B.position = pos;
        B.off[0] = B.off[1] = 0.f;   // compounds stay in the world frame
        B.centred = 0;
        P.bparams[p] = B;
        part_info = bi;
        n = B.loop != LOOP_NONE ? bi.n_chunks : 0u;
    }
    list_chunks(P, p, part_info, n);
}

__device__ __forceinline__ void add3(double* a, const double* b)
{
    a[0] += b[0];
    a[1] += b[1];
    a[2] += b[2];
}

// One thread per compound (FP64 work, as in finalize_kernel): it sums each
// part's chunk partials (chunk order) and applies the compound's rules part
// by part.
__global__ void __launch_bounds__(kBodyThreads) compound_finalize_kernel(const KParams P, const CompoundParams C)
{
    const uint32_t c = blockIdx.x * kBodyThreads + threadIdx.x;
    if (c < (uint32_t)kClaimClasses) P.n_listed[c] = 0u;
    if (c >= C.n_compounds) return;
    const hydro_body& cb = C.compounds[c];
    const CompoundInfo ci = C.cinfo[c];
    const int status = (*P.err & 1u) ? HYDRO_ERR_TIMEOUT : 0;
    int pos = HYDRO_SKIPPED;
    if (fluid_mode(cb.mode)) pos = classify(P.ocean, cb.aabb_min, cb.aabb_max);
    hydro_wrench w = C.io[c];
    hydro_wrench cw{};            // the per-part in-out values of the reference's loop (:379-386)
    int mismatch = 0;
    if (pos == HYDRO_INSIDE) {                                   // :316-356
        if (cb.buoyancy) {
            const double k = -cb.volume * P.ocean.density;
            double f[3] = {0.0 * k, 0.0 * k, P.ocean.gravity * k};
            const double* R = cb.T_CG.basis;
            const double* og = cb.T_CG.origin;
            const double* pc = cb.P_CB;
            double q[3] = {(R[0] * pc[0] + R[1] * pc[1] + R[2] * pc[2]) + og[0],
                           (R[3] * pc[0] + R[4] * pc[1] + R[5] * pc[2]) + og[1],
                           (R[6] * pc[0] + R[7] * pc[1] + R[8] * pc[2]) + og[2]};
            double r[3] = {q[0] - og[0], q[1] - og[1], q[2] - og[2]};
            copy3(w.Fb, f);
            bcross(r, f, w.Tb);
        }
        if (P.st.damping) {
            zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf);
        }
    } else if (pos == HYDRO_CROSSING_SURFACE && (P.st.buoyancy || P.st.damping)) {   // :359-381
        if (P.st.buoyancy) { zero3(w.Fb); zero3(w.Tb); }
        if (P.st.damping) { zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf); }
        w.Swet = 0.0;
        w.Vsub = 0.0;
    }
    for (uint32_t k = 0; k < ci.n_parts; ++k) {
        const uint32_t p = ci.first_part + k;
        const BodyParams B = P.bparams[p];
        const BodyInfo bi = P.binfo[p];
        double S[kQ];
#pragma unroll
        for (int q = 0; q < kQ; ++q) S[q] = 0.0;
        if (B.loop != LOOP_NONE) {
            const double* pp = P.partials + (size_t)bi.first_chunk * kPartialStride;
            for (uint32_t j = 0; j < bi.n_chunks; ++j, pp += kPartialStride) {
#pragma unroll
                for (int q = 0; q < kQ; ++q) S[q] += pp[q];
            }
        }
        {
            const hydro_compound_part& pt = C.parts[p];
            mismatch |= B.mismatch;
            const bool null_mesh = (bi.mesh == HYDRO_NO_MESH);
            if (pos == HYDRO_INSIDE && P.st.damping && pt.external && fluid_mode(pt.mode)) {
                // ComputeHydrodynamicForcesSubmerged then the part's correction (:337-352)
                double Fq[3], Tq[3], Ff[3], Tf[3];
                copy3(Fq, S + Q_FDQ); copy3(Tq, S + Q_TDQ); copy3(Ff, S + Q_FDF); copy3(Tf, S + Q_TDF);
                correct4(P.ocean.density, Fq, Tq, Ff, Tf, pt.Cd, pt.Cf, pt.R_O);
                add3(w.Fdq, Fq); add3(w.Tdq, Tq); add3(w.Fdf, Ff); add3(w.Tdf, Tf);
            } else if (pos == HYDRO_CROSSING_SURFACE && (P.st.buoyancy || P.st.damping) && fluid_mode(pt.mode)) {
                const int pb = P.st.buoyancy && pt.buoyant;
                if (pt.external || pb) {
                    const int dmp = pt.external ? P.st.damping : 0;
                    // ComputeHydrodynamicForcesSurface on the carried in-out values
                    if (null_mesh) {
                        if (pb) { zero3(cw.Fb); zero3(cw.Tb); }
                        if (dmp) { zero3(cw.Fdq); zero3(cw.Tdq); zero3(cw.Fdf); zero3(cw.Tdf); }
                        cw.Swet = 0.0;
                        cw.Vsub = 0.0;
                    } else {
                        finalize_surface(P.ocean, pb, dmp, cb.T_CG.origin, (double)B.p0.x, (double)B.p0.y, S,
                                         cw);
                    }
                    if (pt.external) {                           // :411-422
                        correct4(P.ocean.density, cw.Fdq, cw.Tdq, cw.Fdf, cw.Tdf, pt.Cd, pt.Cf, pt.R_O);
                        add3(w.Fb, cw.Fb); add3(w.Tb, cw.Tb);
                        add3(w.Fdq, cw.Fdq); add3(w.Tdq, cw.Tdq); add3(w.Fdf, cw.Fdf); add3(w.Tdf, cw.Tdf);
                        w.Swet += cw.Swet;
                        w.Vsub += cw.Vsub;
                    } else {                                     // :424-431
                        add3(w.Fb, cw.Fb); add3(w.Tb, cw.Tb);
                        w.Vsub += cw.Vsub;
                    }
                }
            }
        }
    }
    {
        if (pos == HYDRO_OUTSIDE) {                                  // :302-314
            zero3(w.Fb); zero3(w.Tb); zero3(w.Fdq); zero3(w.Tdq); zero3(w.Fdf); zero3(w.Tdf);
            w.Swet = 0.0;
            w.Vsub = 0.0;
        } else if (pos == HYDRO_INSIDE) {
            w.Swet = cb.surface;                                     // :355-356
            w.Vsub = cb.volume;
        }
        w.position = pos;
        w.status = mismatch ? HYDRO_ERR_MISMATCH : status;
        C.io[c] = w;
    }
}

cudaError_t launch_compound_step(const KParams& P, const CompoundParams& C, LaunchShape shape, int cut64,
                                 cudaStream_t s, uint32_t* launches)
{
    *launches = 0;
    if (C.n_compounds == 0) return cudaSuccess;
    cudaError_t e;
    if (P.n_bodies) {
        compound_prep_kernel<<<(P.n_bodies + kBodyThreads - 1) / kBodyThreads, kBodyThreads, 0, s>>>(P, C);
        if ((e = cudaGetLastError())) return e;
        int grid = shape.grid;
        if (grid > (int)P.n_chunks) grid = (int)P.n_chunks;
        if (grid < 1) grid = 1;
        const int field = P.ocean.field_currents ? 1 : 0;
        const void* k = chunk_kernel_for(cut64, P.ocean.waves != 0, shape.ctas_per_sm, 0, field);
        if ((e = chunk_kernel_attr(cut64, P.ocean.waves != 0, shape.ctas_per_sm, 0, field)))
            return e;
        void* args[] = {const_cast<KParams*>(&P)};
        if ((e = cudaLaunchKernel(k, dim3(grid), dim3(kThreads), args, sizeof(ChunkSmem), s))) return e;
        *launches = 2;
    }
    compound_finalize_kernel<<<(C.n_compounds + kBodyThreads - 1) / kBodyThreads, kBodyThreads, 0, s>>>(
        P, C);
    if ((e = cudaGetLastError())) return e;
    *launches += 1;
    return cudaSuccess;
}

// ------------------------------------------------------- debug face terms
template <bool CUT64>
__global__ void __launch_bounds__(kBlock) face_terms_kernel(const TileDesc* tiles, uint32_t first_tile,
                                                            const hydro_body* body, OceanDev ocean,
                                                            SettingsDev st, int frame, float* out, int packed)
{
    __shared__ float4 verts[kTileVerts];
    __shared__ BodyParams Bs;
    const int tid = threadIdx.x;
    const TileDesc td = tiles[first_tile + blockIdx.x];
    if (tid == 0) body_prologue(body, body->mesh, OP_SURFACE, ocean, st, frame, Bs);
    __syncthreads();
    const BodyParams B = Bs;
    const int nv = td.nv, nvp = (nv + 3) & ~3;
    for (int v = tid; v < nv; v += kBlock) {
        v3 p = xform(B.TC, td.block[v], td.block[nvp + v], td.block[2 * nvp + v]);
        verts[v] = make_float4(p.x, p.y, p.z, depth_at_b(ocean, B, p.x, p.y, p.z));
    }
    __syncthreads();
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(td.block + 3 * nvp);
    const uint32_t* face_id = reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(td.block) +
                                                                tile_bytes(td.nv, td.nf));
    // Thread t takes faces 2t and 2t+1: a pair of fully submerged faces goes
    // through the packed path (as in the batched kernel), any other face
    // through the scalar path, so that both are checked.
    for (int f = 2 * tid; f < td.nf; f += 2 * kBlock) {
        const bool hasB = f + 1 < td.nf;
        const uint32_t wa = idx[f], wb = idx[hasB ? f + 1 : f];
        const float4 a1 = verts[wa & 511u], a2 = verts[(wa >> 9) & 511u], a3 = verts[wa >> 18];
        const float4 b1 = verts[wb & 511u], b2 = verts[(wb >> 9) & 511u], b3 = verts[wb >> 18];
        const int ca = face_class(a1.w, a2.w, a3.w), cb = face_class(b1.w, b2.w, b3.w);
        float* oa = out + (size_t)face_id[f] * kQ;
        float* ob = out + (size_t)face_id[hasB ? f + 1 : f] * kQ;
        if (packed && ca == 1 && cb == 1 && hasB) {
            // the packed path adds face A then face B into one set of sums:
            // evaluate (A, B) with B's half switched off, then (B, A)
            const BodyPair Bp = body_pair(B, ocean);
            for (int h = 0; h < 2; ++h) {
                Acc a;
                for (int k = 0; k < kQ; ++k) a.q[k] = 0.f;
                const P3 c1 = h ? corners(b1, a1) : corners(a1, b1);
                const P3 c2 = h ? corners(b2, a2) : corners(a2, b2);
                const P3 c3 = h ? corners(b3, a3) : corners(a3, b3);
                if (ocean.waves) face_full2<true>(ocean, B, Bp, a, c1, c2, c3, false);
                else face_full2<false>(ocean, B, Bp, a, c1, c2, c3, false);
                float* o = h ? ob : oa;
                for (int k = 0; k < kQ; ++k) o[k] = a.q[k];
            }
            continue;
        }
        for (int h = 0; h < (hasB ? 2 : 1); ++h) {
            Acc a;
            for (int k = 0; k < kQ; ++k) a.q[k] = 0.f;
            const float4 q1 = h ? b1 : a1, q2 = h ? b2 : a2, q3 = h ? b3 : a3;
            if (ocean.waves)
                face_surface<CUT64, true>(ocean, B, a, q1, q2, q3);
            else
                face_surface<CUT64, false>(ocean, B, a, q1, q2, q3);
            float* o = h ? ob : oa;
            for (int k = 0; k < kQ; ++k) o[k] = a.q[k];
        }
    }
}

// The outlines the reference's DEBUG_HYDRO build records for one body in
// the surface loop: one thread per face on the scalar path, in the world
// frame like the reference; out receives 13 floats per face in uploaded
// face order (corner count 0, 3 or 4, then four corners).
template <bool CUT64>
__global__ void __launch_bounds__(kBlock) outline_kernel(const TileDesc* tiles, uint32_t first_tile,
                                                         const hydro_body* body, OceanDev ocean, SettingsDev st,
                                                         float* out)
{
    __shared__ float4 verts[kTileVerts];
    __shared__ BodyParams Bs;
    const int tid = threadIdx.x;
    const TileDesc td = tiles[first_tile + blockIdx.x];
    if (tid == 0) body_prologue(body, body->mesh, OP_SURFACE, ocean, st, HYDRO_FRAME_WORLD, Bs);
    __syncthreads();
    const BodyParams B = Bs;
    const int nv = td.nv, nvp = (nv + 3) & ~3;
    for (int v = tid; v < nv; v += kBlock) {
        v3 p = xform(B.TC, td.block[v], td.block[nvp + v], td.block[2 * nvp + v]);
        verts[v] = make_float4(p.x, p.y, p.z, depth_at_b(ocean, B, p.x, p.y, p.z));
    }
    __syncthreads();
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(td.block + 3 * nvp);
    const uint32_t* face_id = reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(td.block) +
                                                                tile_bytes(td.nv, td.nf));
    for (int f = tid; f < td.nf; f += kBlock) {
        const uint32_t w = idx[f];
        const float4 q1 = verts[w & 511u], q2 = verts[(w >> 9) & 511u], q3 = verts[w >> 18];
        float* o = out + (size_t)face_id[f] * 13;
        o[0] = 0.f;
        Acc a;
        for (int k = 0; k < kQ; ++k) a.q[k] = 0.f;
        if (ocean.waves)
            face_surface<CUT64, true, true>(ocean, B, a, q1, q2, q3, o);
        else
            face_surface<CUT64, false, true>(ocean, B, a, q1, q2, q3, o);
    }
}

cudaError_t launch_outline(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles, const hydro_body* body,
                           OceanDev ocean, SettingsDev st, int cut64, float* out, cudaStream_t s)
{
    if (n_tiles == 0) return cudaSuccess;
    if (cut64)
        outline_kernel<true><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, out);
    else
        outline_kernel<false><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, out);
    return cudaGetLastError();
}

cudaError_t launch_face_terms(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles,
                              const hydro_body* body, OceanDev ocean, SettingsDev st, int frame,
                              int cut64, int packed, float* out, cudaStream_t s)
{
    if (n_tiles == 0) return cudaSuccess;
    if (cut64)
        face_terms_kernel<true><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, frame, out, packed);
    else
        face_terms_kernel<false><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, frame, out, packed);
    return cudaGetLastError();
}

// --------------------------------------------------- surrogate: fluid gate
// Clears the gate mask of the bodies whose fluid position is INSIDE
// (CheckBodyFluidPosition, SolidEntity.cpp:1239-1261): the reference
// switches to its analytic buoyancy there (:1827-1843), a regime the learned
// surrogate sees rarely and fits worst, so those states go to the exact step.
__global__ void gate_inside_kernel(const hydro_body* __restrict__ bodies, uint32_t n, OceanDev o,
                                   uint8_t* __restrict__ mask)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || mask[i] == 0) return;
    const hydro_body& b = bodies[i];
    if (classify(o, b.aabb_min, b.aabb_max) == HYDRO_INSIDE) mask[i] = 0;
}

cudaError_t launch_gate_inside(const hydro_body* bodies, uint32_t n, OceanDev o, uint8_t* mask, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    gate_inside_kernel<<<(n + 127) / 128, 128, 0, s>>>(bodies, n, o, mask);
    return cudaGetLastError();
}

// ------------------------------------------------------------ small kernels
__global__ void correct_kernel(double density, double* io, const double* Cd, const double* Cf,
                               const double* R_O)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        correct4(density, io, io + 3, io + 6, io + 9, Cd, Cf, R_O);
}

__global__ void aero_correct_kernel(const hydro_aero_params* p, double* io6)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) aero_correct(*p, io6, io6 + 3);
}

cudaError_t launch_aero_correct(const hydro_aero_params* p, double* io6, cudaStream_t s)
{
    aero_correct_kernel<<<1, 32, 0, s>>>(p, io6);
    return cudaGetLastError();
}

cudaError_t launch_correct(double density, double* io12, const double* Cd, const double* Cf,
                           const double* R_O, cudaStream_t s)
{
    correct_kernel<<<1, 32, 0, s>>>(density, io12, Cd, Cf, R_O);
    return cudaGetLastError();
}

__global__ void fluid_position_kernel(OceanDev o, const double* aabb6, int* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *out = classify(o, aabb6, aabb6 + 3);
}

cudaError_t launch_fluid_position(OceanDev ocean, const double* aabb6, int* out, cudaStream_t s)
{
    fluid_position_kernel<<<1, 32, 0, s>>>(ocean, aabb6, out);
    return cudaGetLastError();
}

__global__ void depth_kernel(OceanDev o, const float* xyz, uint32_t n, float* out)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = depth_at(o, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

cudaError_t launch_depth(OceanDev ocean, const float* xyz, uint32_t n, float* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    depth_kernel<<<(n + 255) / 256, 256, 0, s>>>(ocean, xyz, n, out);
    return cudaGetLastError();
}

}  // namespace sfh

namespace sfh {

// ------------------------------------------------------ division self-check
__device__ __forceinline__ uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool same_float(float x, float y)
{
    return __float_as_uint(x) == __float_as_uint(y) || (x != x && y != y);
}

// counts[0]: a/3 over every float bit pattern; counts[1]: a/b over random
// pairs with b in [1e-6, 1e3] (the face-length range); counts[2]: a/b over
// random pairs of normal floats whose quotient is normal.
__global__ void division_check_kernel(uint64_t n_pairs, uint64_t seed, unsigned long long* counts)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long bad3 = 0, badr = 0, badw = 0;
    for (uint64_t i = tid; i < (1ull << 32); i += nthreads) {
        float a = __uint_as_float((uint32_t)i);
        if (!isfinite(a)) continue;
        if (!same_float(div3(a), __fdiv_rn(a, 3.f))) ++bad3;
    }
    uint64_t s = seed ^ (tid * 0x632BE59BD9B4E019ull);
    for (uint64_t i = tid; i < n_pairs; i += nthreads) {
        uint64_t r = splitmix64(s);
        // a: random sign/significand, exponent in [-40, 40]; b in [1e-6, 1e3]
        uint32_t ea = (uint32_t)(127 - 40 + (r % 81));
        float a = __uint_as_float(((uint32_t)(r >> 40) & 0x807FFFFFu) | (ea << 23));
        float b = 1e-6f * __powf(1e9f, (float)((r >> 8) & 0xFFFFFF) * 0x1p-24f);
        if (!same_float(div_by_rcp(a, b, __frcp_rn(b)), __fdiv_rn(a, b))) ++badr;
        uint64_t r2 = splitmix64(s);
        uint32_t eb = (uint32_t)(1 + (r2 % 253));
        float w = __uint_as_float(((uint32_t)(r2 >> 32) & 0x807FFFFFu) | (eb << 23));
        float q = __fdiv_rn(a, w);
        if (isfinite(q) && fabsf(q) >= 0x1p-126f && fabsf(q) < 0x1p126f &&
            !same_float(div_by_rcp(a, w, __frcp_rn(w)), q)) ++badw;
    }
    atomicAdd(counts + 0, bad3);
    atomicAdd(counts + 1, badr);
    atomicAdd(counts + 2, badw);
}

cudaError_t launch_division_check(uint64_t n_pairs, uint64_t seed, unsigned long long* counts,
                                  cudaStream_t s)
{
    division_check_kernel<<<1216, 256, 0, s>>>(n_pairs, seed, counts);
    return cudaGetLastError();
}

}  // namespace sfh

namespace sfh {

// --------------------------------------------------- packed FP32 self-check
// counts[k] mismatches of the packed op k (0 mul, 1 add, 2 sub, 3 fma)
// against the scalar IEEE op on both halves; ex[4k..4k+3] one failing
// operand set (a, b, c, packed result) of op k.
__global__ void packed_check_kernel(uint64_t n, uint64_t seed, unsigned long long* counts, float* ex)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    uint64_t s = seed ^ (tid * 0x9E3779B97F4A7C15ull);
    unsigned long long bad[4] = {0, 0, 0, 0};
    for (uint64_t i = tid; i < n; i += nthreads) {
        float v[6];
        for (int k = 0; k < 6; ++k) {
            uint64_t r = splitmix64(s);
            uint32_t e = (uint32_t)(127 - 30 + (r % 61));
            v[k] = __uint_as_float(((uint32_t)(r >> 32) & 0x807FFFFFu) | (e << 23));
        }
        const float2 a = make_float2(v[0], v[1]), b = make_float2(v[2], v[3]), c = make_float2(v[4], v[5]);
        float2 r[4] = {mul2(a, b), add2(a, b), sub2(a, b), fma2(a, b, c)};
        float2 w[4] = {make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)),
                       make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)),
                       make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y))};
        for (int k = 0; k < 4; ++k) {
            if (!same_float(r[k].x, w[k].x) || !same_float(r[k].y, w[k].y)) {
                if (bad[k] == 0) {
                    ex[4 * k + 0] = a.x; ex[4 * k + 1] = b.x; ex[4 * k + 2] = c.x;
                    ex[4 * k + 3] = r[k].x;
                }
                ++bad[k];
            }
        }
    }
    for (int k = 0; k < 4; ++k) atomicAdd(counts + 3 + k, bad[k]);
}

cudaError_t launch_packed_check(uint64_t n, uint64_t seed, unsigned long long* counts, float* ex,
                                cudaStream_t s)
{
    packed_check_kernel<<<1216, 256, 0, s>>>(n, seed, counts, ex);
    return cudaGetLastError();
}

}  // namespace sfh

namespace sfh {

// ------------------------------------------------------- bounded-wait check
// One CTA waits, with the bounded wait of the pipeline, on an mbarrier that
// nothing ever completes; it gives up after limit_ns and reports
// HYDRO_ERR_TIMEOUT in *status, leaving nothing in flight.
__global__ void wait_timeout_kernel(uint64_t limit_ns, int* status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1u);
        mbar_fence_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_for(&bar, 0u, limit_ns);
    const bool all = __syncthreads_and(ok ? 1 : 0) != 0;
    if (threadIdx.x == 0) *status = all ? 0 : HYDRO_ERR_TIMEOUT;
}

cudaError_t launch_wait_timeout(uint64_t limit_ns, int* status, cudaStream_t s)
{
    wait_timeout_kernel<<<1, 64, 0, s>>>(limit_ns, status);
    return cudaGetLastError();
}

}  // namespace sfh
