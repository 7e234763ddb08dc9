// hydro_pair.cuh -- two faces at a time on Blackwell's packed FP32 pipe.
//
// sm_100+ executes add/sub/mul/fma.rn.f32x2 on a pair of FP32 values per
// instruction, at twice the scalar FP32 rate.  The surface and submerged
// loops evaluate their fully submerged faces two at a time: face A in the
// .x half and face B in the .y half of every pair.  Each half performs the
// same IEEE round-to-nearest operations, in the same order, as the scalar
// code in hydro_device.cuh, so each face's contribution is bit-identical to
// the scalar evaluation; branches of the reference (degenerate face, the
// two damping thresholds) become per-half selects of the accumulators.
#pragma once

#include "hydro_device.cuh"

namespace sfh {

// ------------------------------------------------------------ packed ops
// CUDA's packed intrinsics (sm_100+) compute each half like __fadd_rn /
// __fmul_rn / __fmaf_rn, but ptxas contracts a packed multiply followed by a
// packed add into one FMA (the .rn modifier and --fmad=false do not stop it
// for packed operations), which would change the rounding of the reference
// arithmetic.  Products are therefore formed as fma(a, b, z) with z = -0
// read from device memory at run time: fma(a, b, -0) rounds a*b exactly
// once like a multiply (signed zeros included), and because ptxas cannot
// see that the addend is zero it neither turns the FMA back into a multiply
// nor merges it with the add that follows.  a - b is a + (-b), bit-identical
// in round-to-nearest.
__device__ float g_pair_negzero = -0.0f;

__device__ __forceinline__ float2 pair_zero()
{
    const float z = g_pair_negzero;
    return make_float2(z, z);
}

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __ffma2_rn(a, b, pair_zero()); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Per-half select: (ca ? n.x : o.x, cb ? n.y : o.y)
__device__ __forceinline__ float2 sel2(bool ca, bool cb, float2 n, float2 o)
{
    return make_float2(ca ? n.x : o.x, cb ? n.y : o.y);
}

// Three components, each a pair (face A, face B).
struct P3 {
    float2 x, y, z;
};

__device__ __forceinline__ P3 pk(float2 x, float2 y, float2 z) { P3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ P3 pbc(v3 a) { return pk(bc(a.x), bc(a.y), bc(a.z)); }
__device__ __forceinline__ P3 padd(P3 a, P3 b) { return pk(add2(a.x, b.x), add2(a.y, b.y), add2(a.z, b.z)); }
__device__ __forceinline__ P3 psub(P3 a, P3 b) { return pk(sub2(a.x, b.x), sub2(a.y, b.y), sub2(a.z, b.z)); }
__device__ __forceinline__ P3 pmul(P3 a, float2 s) { return pk(mul2(a.x, s), mul2(a.y, s), mul2(a.z, s)); }
// glm::dot order: (x*x' + y*y') + z*z'
__device__ __forceinline__ float2 pdot(P3 a, P3 b)
{
    return add2(add2(mul2(a.x, b.x), mul2(a.y, b.y)), mul2(a.z, b.z));
}
// glm::cross order
__device__ __forceinline__ P3 pcross(P3 a, P3 b)
{
    return pk(sub2(mul2(a.y, b.z), mul2(b.y, a.z)),
              sub2(mul2(a.z, b.x), mul2(b.z, a.x)),
              sub2(mul2(a.x, b.y), mul2(b.x, a.y)));
}

// a / b per half with the FMA correction of div_by_rcp (no tiny check).
__device__ __forceinline__ float2 pdiv_rcp_fast(float2 a, float2 b, float2 y)
{
    float2 q = mul2(a, y);
    float2 r = fma2(make_float2(-b.x, -b.y), q, a);
    return fma2(r, y, q);
}

// Vector / per-half scalar.  The FMA-corrected quotient is the IEEE one
// whenever the numerator is not tiny (see div_by_rcp); one test per vector
// sends the rare vectors with a tiny component to IEEE division.
__device__ __forceinline__ P3 pdiv_vec(P3 a, float2 b, float2 y)
{
    const float t = 0x1p-100f;
    const bool tiny = fminf(fminf(fabsf(a.x.x), fabsf(a.y.x)), fminf(fabsf(a.z.x), fminf(fabsf(a.x.y),
                      fminf(fabsf(a.y.y), fabsf(a.z.y))))) < t;
    if (!tiny) return pk(pdiv_rcp_fast(a.x, b, y), pdiv_rcp_fast(a.y, b, y), pdiv_rcp_fast(a.z, b, y));
    return pk(f2(div_by_rcp(a.x.x, b.x, y.x), div_by_rcp(a.x.y, b.y, y.y)),
              f2(div_by_rcp(a.y.x, b.x, y.x), div_by_rcp(a.y.y, b.y, y.y)),
              f2(div_by_rcp(a.z.x, b.x, y.x), div_by_rcp(a.z.y, b.y, y.y)));
}

__device__ __forceinline__ P3 pdvs_rcp(P3 a, float2 b)
{
#ifdef HYDRO_FAST_MATH
    const float2 y = f2(1.f / b.x, 1.f / b.y);
    return pmul(a, y);
#else
    return pdiv_vec(a, b, f2(__frcp_rn(b.x), __frcp_rn(b.y)));
#endif
}

__device__ __forceinline__ P3 pdvs3(P3 a)
{
#ifdef HYDRO_FAST_MATH
    return pmul(a, bc(0x1.555556p-2f));
#else
    return pdiv_vec(a, bc(3.f), bc(0x1.555556p-2f));
#endif
}

// Accumulation of the two halves of a packed term into the thread's scalar
// running sums (face A first, then face B).  A term the reference does not
// add (degenerate face, padding half, no drag or no friction on the face)
// reaches this point as exactly zero: the running sums start at +0 and an
// IEEE round-to-nearest sum is -0 only when both addends are -0, so a sum is
// never -0 and adding a zero of either sign leaves its bits unchanged.
__device__ __forceinline__ void acc_add2(float& acc, float2 v)
{
    acc = acc + v.x;
    acc = acc + v.y;
}

__device__ __forceinline__ void acc_add3p(Acc& a, int k, P3 v)
{
    acc_add2(a.q[k], v.x);
    acc_add2(a.q[k + 1], v.y);
    acc_add2(a.q[k + 2], v.z);
}

// Per-half zeroing of a scalar pair: (ca ? v.x : 0, cb ? v.y : 0)
__device__ __forceinline__ float2 keep2(bool ca, bool cb, float2 v)
{
    return make_float2(ca ? v.x : 0.f, cb ? v.y : 0.f);
}

__device__ __forceinline__ P3 corners(float4 qa, float4 qb)
{
    return pk(f2(qa.x, qb.x), f2(qa.y, qb.y), f2(qa.z, qb.z));
}

// Per-body values broadcast to both halves.
struct BodyPair {
    P3 p, p0, v, omega, U;
};

__device__ __forceinline__ BodyPair body_pair(const BodyParams& B, const OceanDev& o)
{
    BodyPair r;
    r.p = pbc(B.p);
    r.p0 = pbc(B.p0);
    r.v = pbc(B.v);
    r.omega = pbc(B.omega);
    r.U = pk(bc(o.U[0]), bc(o.U[1]), bc(o.U[2]));
    return r;
}

// Fluid velocity at both centroids (Ocean::GetFluidVelocity).
template <bool FIELD = true>
__device__ __forceinline__ P3 fluid_velocity2(const OceanDev& o, const BodyParams& B, const BodyPair& Bp, P3 fc)
{
    if (!FIELD || !o.field_currents) return Bp.U;
    v3 a = fluid_velocity_b<FIELD>(o, B, mk(fc.x.x, fc.y.x, fc.z.x));
    v3 b = fluid_velocity_b<FIELD>(o, B, mk(fc.x.y, fc.y.y, fc.z.y));
    return pk(f2(a.x, b.x), f2(a.y, b.y), f2(a.z, b.z));
}

// tri_props for two triangles.  A degenerate face (len^2 < 1e-12,
// :1385-1386) and the padding half (validB false) get a zero normal and
// area, which makes every term they would add zero (their corners are
// finite).
__device__ __forceinline__ void tri_props2(P3 p1, P3 p2, P3 p3, P3& fc, P3& fn1, float2& A, bool validB)
{
    P3 fv1 = psub(p2, p1);
    P3 fv2 = psub(p3, p1);
    fc = pdvs3(padd(padd(p1, p2), p3));
    P3 fn = pcross(fv1, fv2);
    float2 len = pdot(fn, fn);
    const bool okA = !(len.x < 1e-12f);
    const bool okB = !(len.y < 1e-12f) && validB;
    len = f2(sqrtf(len.x), sqrtf(len.y));
    fn1 = pdvs_rcp(fn, len);
    fn1 = pk(keep2(okA, okB, fn1.x), keep2(okA, okB, fn1.y), keep2(okA, okB, fn1.z));
    A = keep2(okA, okB, mul2(len, bc(0.5f)));
}

// Damping of two faces (:1661-1683).  Drag and skin friction of a face
// that does not get them are computed with a zero area.
template <bool FIELD = true>
__device__ __forceinline__ void damping2(const OceanDev& o, const BodyParams& B, const BodyPair& Bp, Acc& a,
                                         P3 fc, P3 fn1, float2 A)
{
    P3 r = psub(fc, Bp.p);
    P3 vc = psub(fluid_velocity2<FIELD>(o, B, Bp, fc), padd(Bp.v, pcross(Bp.omega, r)));
    float2 vc_n = pdot(vc, fn1);
    P3 vn = pk(mul2(vc_n, fn1.x), mul2(vc_n, fn1.y), mul2(vc_n, fn1.z));
    P3 vt = psub(vc, vn);
    const bool qa = vc_n.x < -1e-12f, qb = vc_n.y < -1e-12f;   // zero normal: false
    if (qa || qb) {
        float2 vmag2 = pdot(vc, vc);
        float2 s = f2(sqrtf(vmag2.x), sqrtf(vmag2.y));
        P3 q = pmul(pmul(pmul(vc, s), neg2(vc_n)), keep2(qa, qb, A));
        acc_add3p(a, Q_FDQ, q);
        acc_add3p(a, Q_TDQ, pcross(r, q));
    }
    float2 vt2 = pdot(vt, vt);
    P3 sk = pmul(vt, keep2(vt2.x > 1e-9f, vt2.y > 1e-9f, A));
    acc_add3p(a, Q_FDF, sk);
    acc_add3p(a, Q_TDF, pcross(r, sk));
}

// Two fully submerged faces of the surface loop (:1618-1647, :1650-1686).
// validB false: the B half is padding and contributes nothing.
template <bool WAVES, bool FIELD = true>
__device__ __forceinline__ void face_full2(const OceanDev& o, const BodyParams& B, const BodyPair& Bp,
                                           Acc& a, P3 p1, P3 p2, P3 p3, bool validB)
{
    {
        const P3 p01 = psub(p1, Bp.p0), p02 = psub(p2, Bp.p0), p03 = psub(p3, Bp.p0);
        P3 cg = pmul(padd(padd(p01, p02), p03), bc(0.25f));
        const float2 v6 = keep2(true, validB, pdot(p01, pcross(p02, p03)));
        acc_add3p(a, Q_CB, pmul(cg, v6));
        acc_add2(a.q[Q_V6], v6);
    }
    P3 fc, fn1;
    float2 A;
    tri_props2(p1, p2, p3, fc, fn1, A, validB);
    if (WAVES && B.buoyancy) {
        float2 dc = f2(depth_at_b(o, B, fc.x.x, fc.y.x, fc.z.x), depth_at_b(o, B, fc.x.y, fc.y.y, fc.z.y));
        P3 Fbi = pmul(pmul(pk(neg2(fn1.x), neg2(fn1.y), neg2(fn1.z)), A), dc);
        acc_add3p(a, Q_FB, Fbi);
        acc_add3p(a, Q_TB, pcross(psub(fc, Bp.p), Fbi));
    }
    if (B.damping) damping2<FIELD>(o, B, Bp, a, fc, fn1, A);
    acc_add2(a.q[Q_SWET], A);
}

// Two faces of the submerged loop (:1748-1789).
template <bool FIELD = true>
__device__ __forceinline__ void face_submerged2(const OceanDev& o, const BodyParams& B, const BodyPair& Bp, Acc& a,
                                                P3 p1, P3 p2, P3 p3, bool validB)
{
    P3 fc, fn1;
    float2 A;
    tri_props2(p1, p2, p3, fc, fn1, A, validB);
    damping2<FIELD>(o, B, Bp, a, fc, fn1, A);
}

}  // namespace sfh
