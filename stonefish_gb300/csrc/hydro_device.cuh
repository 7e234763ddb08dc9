// hydro_device.cuh -- device-side arithmetic of the hydrodynamic wrench path.
//
// Every per-face step restates Stonefish's SolidEntity hydrodynamics
// (Library/src/entities/SolidEntity.cpp:1289-1797) in FP32 with the
// operation order of the glm calls it uses (glm >= 0.9.9):
//   dot(a,b)   = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   M*vec4(p,1) = (c0*x + c1*y) + (c2*z + c3)
// The library is compiled with -fmad=false and IEEE division/square root, so
// each face's contribution is bit-identical to a CPU evaluation in the same
// order; the boundary and finalisation are FP64 as in the reference.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/stonefish_hydro.h"

namespace sfh {

// ------------------------------------------------------------ constants
constexpr int kBlock = 224;          // compute threads per CTA (seven warps)
constexpr int kWarps = kBlock / 32;
constexpr int kTileFaces = HYDRO_TILE_FACES;   // max faces per tile (64 per compute warp)
constexpr int kTileVerts = 448;      // max distinct vertices per tile (< 512: 9-bit indices)
static_assert(kTileFaces == 64 * kWarps, "a tile gives each compute warp 64 faces");
static_assert(kTileVerts < 512, "vertex indices are packed in 9 bits");
constexpr int kQ = 23;               // accumulated quantities per body
constexpr int kPartialStride = 24;   // doubles per chunk partial (23 + status)
constexpr int kFlushFaces = 32;      // faces a thread sums in FP32 before a flush

// indices of the accumulated quantities
enum : int {
    Q_FB = 0, Q_TB = 3, Q_FDQ = 6, Q_TDQ = 9, Q_FDF = 12, Q_TDF = 15,
    Q_SWET = 18, Q_V6 = 19, Q_CB = 20
};

// loop kinds of a body in one launch
enum : int { LOOP_NONE = 0, LOOP_SURFACE = 1, LOOP_SUBMERGED = 2, LOOP_AERO = 3 };
// launch operations
enum : int { OP_BODY = 0, OP_SURFACE = 1, OP_SUBMERGED = 2, OP_AERO = 3, OP_AERO_BODY = 4 };

// ------------------------------------------------------------- data layout
// One tile of a mesh: nv vertices stored as x[nvp], y[nvp], z[nvp] floats
// (nvp = nv rounded up to 4) followed by one uint32 per face holding its
// three local vertex indices (9 bits each: i0 | i1 << 9 | i2 << 18), padded
// to 16 bytes; that much is copied to shared memory.  Behind it, not
// copied, each face's index in the uploaded mesh (for per-face debug
// output).  `first_face` is the position of the tile's first face in the
// mesh's tile order.
// `sphere` and `half` bound the tile's vertices in mesh coordinates: the
// centre of their box (x, y, z) with the radius of a sphere about it, and
// the box's half extents, each rounded up so that every vertex lies inside.
// They live in this table (L2-resident) rather than in the tile block, so
// that the chunk kernel can test a chunk's tiles against the surface
// without an HBM read.
struct __align__(16) TileDesc {
    const float* block;
    uint16_t nv;
    uint16_t nf;
    uint32_t first_face;
    float4 sphere;      // centre x, y, z; radius
    float4 half;        // half extents x, y, z of the box about the centre; w unused
};

// Bytes of one tile block: x, y, z (nv rounded up to 4 each) and one packed
// index word per face, rounded up to 16 (the TMA size rule).
__host__ __device__ __forceinline__ uint32_t tile_bytes(uint32_t nv, uint32_t nf)
{
    const uint32_t nvp = (nv + 3u) & ~3u;
    return (nvp * 12u + nf * 4u + 15u) & ~15u;
}

// Bytes of a tile block with the faces' upload indices behind it.
__host__ __device__ __forceinline__ uint32_t tile_block_bytes(uint32_t nv, uint32_t nf)
{
    return tile_bytes(nv, nf) + ((nf * 4u + 15u) & ~15u);
}

// A chunk's tiles are described by one lane each of the producer warp.
constexpr int kMaxTilesPerChunk = 32;
// The active-chunk list is claimed largest chunks first, in one class per
// two tile counts: the last chunks a persistent CTA takes are the short
// ones, so the SMs run out of work at nearly the same time.
constexpr int kClaimClasses = kMaxTilesPerChunk / 2;

// One work item: tiles [first_tile, first_tile + n_tiles) of one body.
struct __align__(16) ChunkDesc {
    uint32_t body;
    uint32_t first_tile;
    uint32_t n_tiles;
    uint32_t chunk_in_body;
};

// A chunk whose body runs a face loop in this launch: the prep kernels
// append one per such chunk to the region of its claim class (in the order
// their atomics land, which no result depends on: every chunk writes its own
// partial) and the chunk kernel's producers claim them class by class.
struct __align__(16) ActiveChunk {
    uint32_t body;
    uint32_t first_tile;
    uint32_t n_tiles;
    uint32_t chunk;      // index of the chunk's partial
};
static_assert(sizeof(ChunkDesc) == 16 && sizeof(ActiveChunk) == 16, "chunk records are read and written as uint4");

// Per body of a batch.
struct BodyInfo {
    uint32_t first_chunk;
    uint32_t n_chunks;
    uint32_t mesh;       // mesh the batch was built with (HYDRO_NO_MESH = null)
    uint32_t n_faces;
};

// Ocean as the kernels see it (kernel parameter, by value).
struct OceanDev {
    double density;
    double gravity;
    int waves;
    int currents_enabled;
    int n_currents;
    int field_currents;          // 1 if an enabled JET/PIPE current exists
    float U[3];                  // (float) of the FP64 sum of uniform currents
    const float* wave_data;
    uint32_t wave_n;
    uint32_t wave_channels;
    uint32_t wave_layers;
    uint32_t wave_channel[HYDRO_MAX_WAVE_LAYERS];
    float wave_grid[HYDRO_MAX_WAVE_LAYERS];
    float wave_inv_grid[HYDRO_MAX_WAVE_LAYERS];   // RN(1 / wave_grid[l])
    float wave_half;             // 0.5f / (float)wave_n, the texel-centre offset
    hydro_current currents[HYDRO_MAX_CURRENTS];
};

struct SettingsDev {
    int damping;
    int buoyancy;
};

// ------------------------------------------------------------ FP32 vectors
struct v3 { float x, y, z; };

__device__ __forceinline__ v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 mul(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 dvs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b)
{
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ----------------------------------------------------- correctly rounded x/y
// Division with the result of IEEE round-to-nearest division, from a
// correctly rounded reciprocal and one FMA correction (Markstein's theorem:
// if y = RN(1/b) and q is within one ulp of a/b, then with the exact
// remainder r = a - b*q, RN(q + r*y) = RN(a/b); P. Markstein, "IA-64 and
// Elementary Functions", 2000; Muller et al., Handbook of Floating-Point
// Arithmetic, 2018, section 4.7).  The theorem needs a normal quotient, so
// tiny numerators take the IEEE division instead.  Bit-identity with IEEE
// division is checked on the GPU by hydro_debug_division_check.
__device__ __forceinline__ float div_by_rcp(float a, float b, float y)
{
    if (fabsf(a) < 0x1p-100f) return __fdiv_rn(a, b);
    float q = a * y;
    float r = __fmaf_rn(-b, q, a);
    return __fmaf_rn(r, y, q);
}

// a / 3 with RN(1/3) = 0x1.555556p-2
__device__ __forceinline__ float div3(float a) { return div_by_rcp(a, 3.f, 0x1.555556p-2f); }

#ifdef HYDRO_FAST_MATH
__device__ __forceinline__ v3 dvs_rcp(v3 a, float b) { const float y = 1.f / b; return mul(a, y); }
__device__ __forceinline__ v3 dvs3(v3 a) { return mul(a, 0x1.555556p-2f); }
#else
__device__ __forceinline__ v3 dvs_rcp(v3 a, float b)
{
    const float y = __frcp_rn(b);
    return mk(div_by_rcp(a.x, b, y), div_by_rcp(a.y, b, y), div_by_rcp(a.z, b, y));
}

__device__ __forceinline__ v3 dvs3(v3 a) { return mk(div3(a.x), div3(a.y), div3(a.z)); }
#endif

// Per-body FP32 parameters (glMatrixFromTransform / glVectorFromVector casts,
// Library/src/graphics/OpenGLDataStructs.cpp:148-171).
// 128 bytes, so that a copy can be staged next to each tile.
struct __align__(16) BodyParams {
    float TC[12];     // rows of T_C: R[r][0..2], origin[r]
    v3 p;             // (float) T_CG origin
    v3 p0;            // (p.x, p.y, 0)
    v3 v;
    v3 omega;
    int loop;         // LOOP_*
    int buoyancy;     // reallisticBuoyancy for this body
    int damping;
    int position;     // BodyFluidPosition or HYDRO_SKIPPED
    int mismatch;     // body.mesh differs from the batch's mesh
    // HYDRO_FRAME_CENTRED: TC, p and p0 are relative to (off[0], off[1], 0),
    // the body's CG x and y rounded to FP32; a point's world x and y are the
    // local ones plus off (wave lookups, position-dependent currents).
    float off[2];
    int centred;
};
static_assert(sizeof(BodyParams) == 128, "BodyParams is staged as a 128-byte block");
static_assert(offsetof(BodyParams, p) == 48 && offsetof(BodyParams, p0) == 60 && offsetof(BodyParams, v) == 72 &&
                  offsetof(BodyParams, omega) == 84 && offsetof(BodyParams, loop) == 96 &&
                  offsetof(BodyParams, buoyancy) == 100 && offsetof(BodyParams, damping) == 104,
              "the chunk kernel reads BodyParams bytes 48..111 as four 16-byte words");
static_assert(offsetof(BodyParams, mismatch) == 112 && offsetof(BodyParams, off) == 116 &&
                  offsetof(BodyParams, centred) == 124,
              "the chunk kernel reads the frame offset as BodyParams bytes 112..127");

__device__ __forceinline__ v3 xform(const float* M, float x, float y, float z)
{
    v3 r;
    r.x = (M[0] * x + M[1] * y) + (M[2] * z + M[3]);
    r.y = (M[4] * x + M[5] * y) + (M[6] * z + M[7]);
    r.z = (M[8] * x + M[9] * y) + (M[10] * z + M[11]);
    return r;
}

// ------------------------------------------------------------- wave height
__device__ __forceinline__ float fracf_(float x) { return x - truncf(x); }

// Texel offset j * N + i of the four bilinear taps, wrapped modulo N * N,
// times the channel count plus the channel.  The grid holds fewer than 2^32
// values (hydro_wave_grid_set), so 32 bits hold every offset, also the
// j * N + i of a tap one texel past the last row before it wraps.
__device__ __forceinline__ uint32_t texel_offset(uint32_t N, int j, int i, uint32_t C, uint32_t ch)
{
    const uint32_t NN = N * N;
    uint32_t l = (uint32_t)j * N + (uint32_t)i;
    if (l >= NN) l -= NN;
    return l * C + ch;
}

// OpenGLRealOcean::ComputeInterpolatedWaveData (OpenGLRealOcean.cpp:282-319),
// texel-centred periodic bilinear; the linear texel index wraps modulo N*N
// where the reference would read texel N of a row.
__device__ __forceinline__ float wave_interp(const OceanDev& o, float x, float y, uint32_t ch)
{
    const uint32_t N = o.wave_n;
    const float Nf = (float)N;
    const float half = o.wave_half;   // 0.5f / Nf, formed once on the host (IEEE division there too)
    float i0f = fracf_(x - half);
    float j0f = fracf_(y - half);
    if (i0f < 0.f) i0f = 1.f - fabsf(i0f);
    if (j0f < 0.f) j0f = 1.f - fabsf(j0f);
    int i0 = (int)truncf(i0f * Nf);
    int j0 = (int)truncf(j0f * Nf);
    float i1f = fracf_(x + half);
    float j1f = fracf_(y + half);
    if (i1f < 0.f) i1f = 1.f - fabsf(i1f);
    if (j1f < 0.f) j1f = 1.f - fabsf(j1f);
    int i1 = (int)truncf(i1f * Nf);
    int j1 = (int)truncf(j1f * Nf);
    float alpha = fracf_(i0f * Nf);
    float beta = fracf_(j0f * Nf);
    const float* d = o.wave_data;
    const uint32_t C = o.wave_channels;
    // 32-bit offsets: hydro_wave_grid_set keeps N * N * channels below 2^32
    // (one code path at every inlined lookup keeps the kernels' instruction
    // footprint small)
    const float t0 = __ldg(d + texel_offset(N, j0, i0, C, ch));
    const float t1 = __ldg(d + texel_offset(N, j0, i1, C, ch));
    const float t2 = __ldg(d + texel_offset(N, j1, i0, C, ch));
    const float t3 = __ldg(d + texel_offset(N, j1, i1, C, ch));
    return (1.f - alpha) * (1.f - beta) * t0 + alpha * (1.f - beta) * t1
         + (1.f - alpha) * beta * t2 + alpha * beta * t3;
}

// OpenGLRealOcean::ComputeWaveHeight (:321-331).  x / gs is the IEEE
// quotient, formed from RN(1 / gs) with one FMA correction (div_by_rcp).
__device__ __forceinline__ float wave_height(const OceanDev& o, float x, float y)
{
    float z = 0.f;
    if (o.wave_data == nullptr) return z;
    for (uint32_t l = 0; l < o.wave_layers; ++l) {
        const float gs = o.wave_grid[l], r = o.wave_inv_grid[l];
        z -= wave_interp(o, div_by_rcp(x, gs, r), div_by_rcp(y, gs, r), o.wave_channel[l]);
    }
    return z;
}

// Ocean::GetDepth(glm::vec3) (Ocean.cpp:149-168)
__device__ __forceinline__ float depth_at(const OceanDev& o, float x, float y, float z)
{
    if (o.waves) return z - wave_height(o, x, y);
    return z;
}

// ---------------------------------------------------------------- currents
__device__ __forceinline__ double bdot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ void bcross(const double* a, const double* b, double* r)
{
    double x = a[1] * b[2] - a[2] * b[1];
    double y = a[2] * b[0] - a[0] * b[2];
    double z = a[0] * b[1] - a[1] * b[0];
    r[0] = x; r[1] = y; r[2] = z;
}

// Jet::GetVelocityAtPoint (Jet.cpp:59-80), FP64
__device__ inline void jet_velocity(const hydro_current& c, const double* p, double* out)
{
    double cp[3] = {p[0] - c.point[0], p[1] - c.point[1], p[2] - c.point[2]};
    double x[3];
    bcross(cp, c.dir, x);
    double d = sqrt(bdot(x, x));
    double t = bdot(cp, c.dir);
    out[0] = out[1] = out[2] = 0.0;
    if (t < 0.0) return;
    double r_ = 1.0 / 5.0 * (t + 5.0 * c.radius);
    if (d >= r_) return;
    double s = 10.0 * c.radius / (t + 5.0 * c.radius) * c.speed;
    double f = exp(-50.0 * d * d / (t * t));
    out[0] = (c.dir[0] * s) * f; out[1] = (c.dir[1] * s) * f; out[2] = (c.dir[2] * s) * f;
}

// Pipe::GetVelocityAtPoint (Pipe.cpp:57-79), FP64
__device__ inline void pipe_velocity(const hydro_current& c, const double* p, double* out)
{
    double pp[3] = {p[0] - c.point[0], p[1] - c.point[1], p[2] - c.point[2]};
    double x[3];
    bcross(pp, c.dir, x);
    double d = sqrt(bdot(x, x));
    double t = bdot(pp, c.dir);
    out[0] = out[1] = out[2] = 0.0;
    if (t < 0.0 || t > c.length) return;
    double r = c.radius + (c.radius2 - c.radius) * t / c.length;
    if (d >= r) return;
    double s = c.radius / r * c.speed;
    double f = pow(1.0 - d / r, c.gamma);
    out[0] = (c.dir[0] * s) * f; out[1] = (c.dir[1] * s) * f; out[2] = (c.dir[2] * s) * f;
}

// Ocean::GetFluidVelocity(glm::vec3) (Ocean.cpp:183-201): FP64 sum of the
// enabled currents, cast to float.  Without position-dependent currents the
// value is the same everywhere and was precomputed on the host.
__device__ __forceinline__ v3 fluid_velocity(const OceanDev& o, v3 pt)
{
    if (!o.field_currents) return mk(o.U[0], o.U[1], o.U[2]);
    double p[3] = {(double)pt.x, (double)pt.y, (double)pt.z};
    double fv[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < o.n_currents; ++i) {
        const hydro_current& c = o.currents[i];
        if (!c.enabled) continue;
        double u[3] = {0.0, 0.0, 0.0};
        if (c.type == HYDRO_CURRENT_UNIFORM) { u[0] = c.vel[0]; u[1] = c.vel[1]; u[2] = c.vel[2]; }
        else if (c.type == HYDRO_CURRENT_JET) jet_velocity(c, p, u);
        else if (c.type == HYDRO_CURRENT_PIPE) pipe_velocity(c, p, u);
        fv[0] += u[0]; fv[1] += u[1]; fv[2] += u[2];
    }
    return mk((float)fv[0], (float)fv[1], (float)fv[2]);
}

// The same queries for a point given in a body's frame: the world frame, or
// the centred one of HYDRO_FRAME_CENTRED (local x, y plus the body's offset;
// the offset enters the currents in FP64).
__device__ __forceinline__ float depth_at_b(const OceanDev& o, const BodyParams& B, float x, float y, float z)
{
    if (!o.waves) return z;
    if (B.centred) return z - wave_height(o, x + B.off[0], y + B.off[1]);
    return z - wave_height(o, x, y);
}

// FIELD = false: compiled for launches without jet or pipe currents (the
// field-current code then takes no room in the kernel).
template <bool FIELD = true>
__device__ __forceinline__ v3 fluid_velocity_b(const OceanDev& o, const BodyParams& B, v3 pt)
{
    if (!FIELD || !o.field_currents) return mk(o.U[0], o.U[1], o.U[2]);
    if (!B.centred) return fluid_velocity(o, pt);
    double p[3] = {(double)pt.x + (double)B.off[0], (double)pt.y + (double)B.off[1], (double)pt.z};
    double fv[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < o.n_currents; ++i) {
        const hydro_current& c = o.currents[i];
        if (!c.enabled) continue;
        double u[3] = {0.0, 0.0, 0.0};
        if (c.type == HYDRO_CURRENT_UNIFORM) { u[0] = c.vel[0]; u[1] = c.vel[1]; u[2] = c.vel[2]; }
        else if (c.type == HYDRO_CURRENT_JET) jet_velocity(c, p, u);
        else if (c.type == HYDRO_CURRENT_PIPE) pipe_velocity(c, p, u);
        fv[0] += u[0]; fv[1] += u[1]; fv[2] += u[2];
    }
    return mk((float)fv[0], (float)fv[1], (float)fv[2]);
}

// ------------------------------------------------------- per-face terms
// Running FP32 sums of one thread (or the terms of one face).
struct Acc {
    float q[kQ];
};

__device__ __forceinline__ void acc_add3(Acc& a, int k, v3 v)
{
    a.q[k] += v.x; a.q[k + 1] += v.y; a.q[k + 2] += v.z;
}

// Cut point pa + (pb - pa) * (da / (|db| + da)) of the six clip cases
// (SolidEntity.cpp:1364-1617), FP64 interpolation rounded once when CUT64.
template <bool CUT64>
__device__ __forceinline__ v3 cut(v3 pa, v3 pb, float da, float db)
{
    if (CUT64) {
        double t = (double)da / (fabs((double)db) + (double)da);
        v3 r;
        r.x = (float)((double)pa.x + ((double)pb.x - (double)pa.x) * t);
        r.y = (float)((double)pa.y + ((double)pb.y - (double)pa.y) * t);
        r.z = (float)((double)pa.z + ((double)pb.z - (double)pa.z) * t);
        return r;
    }
    return add(pa, mul(sub(pb, pa), da / (fabsf(db) + da)));
}

// Volume properties of one fan tetra (e.g. :1372-1378)
__device__ __forceinline__ void tetra(Acc& a, v3 x, v3 y, v3 z)
{
    v3 cg = mul(add(add(x, y), z), 0.25f);     // /4 is exact: same bits as division
    float v6 = dot(x, cross(y, z));
    acc_add3(a, Q_CB, mul(cg, v6));
    a.q[Q_V6] += v6;
}

// Damping of one face (:1661-1683 and :1778-1789)
template <bool FIELD = true>
__device__ __forceinline__ void damping(const OceanDev& o, const BodyParams& B, Acc& a,
                                        v3 fc, v3 fn1, float A)
{
    v3 r = sub(fc, B.p);
    v3 vc = sub(fluid_velocity_b<FIELD>(o, B, fc), add(B.v, cross(B.omega, r)));
    float vc_n = dot(vc, fn1);
    v3 vn = mk(vc_n * fn1.x, vc_n * fn1.y, vc_n * fn1.z);
    v3 vt = sub(vc, vn);
    if (vc_n < -1e-12f) {
        float vmag2 = dot(vc, vc);
        v3 q = mul(mul(mul(vc, sqrtf(vmag2)), -vc_n), A);
        acc_add3(a, Q_FDQ, q);
        acc_add3(a, Q_TDQ, cross(r, q));
    }
    float vt2 = dot(vt, vt);
    if (vt2 > 1e-9f) {
        v3 s = mul(vt, A);
        acc_add3(a, Q_FDF, s);
        acc_add3(a, Q_TDF, cross(r, s));
    }
}

// Triangle properties after clipping; returns false for a degenerate face.
__device__ __forceinline__ bool tri_props(v3 p1, v3 p2, v3 p3, v3& fc, v3& fn1, float& A)
{
    v3 fv1 = sub(p2, p1);
    v3 fv2 = sub(p3, p1);
    fc = dvs3(add(add(p1, p2), p3));
    v3 fn = cross(fv1, fv2);
    float len = dot(fn, fn);
    if (len < 1e-12f) return false;
    len = sqrtf(len);
    fn1 = dvs_rcp(fn, len);
    A = len * 0.5f;
    return true;
}

// One face of SolidEntity::ComputeAerodynamicForces (SolidEntity.cpp:1885-1915):
// wind (the atmosphere's fields, passed as currents) relative to the face
// centroid, its normal part vn, and for faces it flows into the term
// vn * vn.length() * A, where glm's vec3::length() is the component count 3.
// Force and torque go to the Q_FDQ / Q_TDQ accumulators.
template <bool FIELD = true>
__device__ __forceinline__ void face_aero(const OceanDev& o, const BodyParams& B, Acc& a, v3 p1, v3 p2, v3 p3)
{
    v3 fc, fn1;
    float A;
    if (!tri_props(p1, p2, p3, fc, fn1, A)) return;
    const v3 r = sub(fc, B.p);
    const v3 vc = sub(fluid_velocity_b<FIELD>(o, B, fc), add(B.v, cross(B.omega, r)));
    const float s = dot(vc, fn1);
    const v3 vn = mk(s * fn1.x, s * fn1.y, s * fn1.z);
    if (dot(fn1, vn) < -1e-12f) {
        const v3 q = mul(mul(vn, 3.f), A);
        acc_add3(a, Q_FDQ, q);
        acc_add3(a, Q_TDQ, cross(r, q));
    }
}

// The part of a surface-loop face after its polygon is known (:1650-1686).
// WAVES is Ocean::hasWaves(): the pressure buoyancy is summed per face only
// with waves.
template <bool WAVES, bool FIELD = true>
__device__ __forceinline__ void face_forces(const OceanDev& o, const BodyParams& B, Acc& a,
                                            v3 fc, v3 fn1, float A)
{
    if (WAVES && B.buoyancy) {
        float depthc = depth_at_b(o, B, fc.x, fc.y, fc.z);
        v3 Fbi = mul(mul(neg(fn1), A), depthc);
        acc_add3(a, Q_FB, Fbi);
        acc_add3(a, Q_TB, cross(sub(fc, B.p), Fbi));
    }
    if (B.damping) damping<FIELD>(o, B, a, fc, fn1, A);
    a.q[Q_SWET] += A;
}

// One face straddling the surface: the six mixed clip cases (:1360-1617).
// The outline of an evaluated submerged part (the points the reference's
// DEBUG_HYDRO build records, SolidEntity.cpp:1390-1396 and the matching
// blocks of the other cases): ol[0] = corner count (3 or 4), then the
// corners in outline order.  OUTLINE = false compiles it away.
__device__ __forceinline__ void put_outline(float* ol, int n, v3 a, v3 b, v3 c, v3 d)
{
    ol[0] = (float)n;
    ol[1] = a.x; ol[2] = a.y; ol[3] = a.z;
    ol[4] = b.x; ol[5] = b.y; ol[6] = b.z;
    ol[7] = c.x; ol[8] = c.y; ol[9] = c.z;
    ol[10] = d.x; ol[11] = d.y; ol[12] = d.z;
}

template <bool CUT64, bool WAVES, bool OUTLINE = false, bool FIELD = true>
__device__ __forceinline__ void face_cut(const OceanDev& o, const BodyParams& B, Acc& a,
                                      v3 p1, v3 p2, v3 p3, float d0, float d1, float d2, float* ol = nullptr)
{
    v3 p4 = mk(0.f, 0.f, 0.f);
    bool quad = false;
    int kind = 0;
    if (d0 < 0.f) {
        if (d1 < 0.f) {
            p1 = cut<CUT64>(p3, p1, d2, d0);
            p2 = cut<CUT64>(p3, p2, d2, d1);
        } else if (d2 < 0.f) {
            p1 = cut<CUT64>(p2, p1, d1, d0);
            p3 = cut<CUT64>(p2, p3, d1, d2);
        } else {
            p4 = cut<CUT64>(p3, p1, d2, d0);
            p1 = cut<CUT64>(p2, p1, d1, d0);
            quad = true; kind = 0;
        }
    } else if (d1 < 0.f) {
        if (d2 < 0.f) {
            p2 = cut<CUT64>(p1, p2, d0, d1);
            p3 = cut<CUT64>(p1, p3, d0, d2);
        } else {
            p4 = cut<CUT64>(p3, p2, d2, d1);
            p2 = cut<CUT64>(p1, p2, d0, d1);
            quad = true; kind = 1;
        }
    } else {
        p4 = cut<CUT64>(p1, p3, d0, d2);
        p3 = cut<CUT64>(p2, p3, d1, d2);
        quad = true; kind = 0;
    }
    const v3 p01 = sub(p1, B.p0);
    const v3 p02 = sub(p2, B.p0);
    const v3 p03 = sub(p3, B.p0);
    tetra(a, p01, p02, p03);
    v3 fc, fn1;
    float A;
    if (!quad) {
        if (!tri_props(p1, p2, p3, fc, fn1, A)) return;
        if (OUTLINE) put_outline(ol, 3, p1, p2, p3, p3);
    } else {
        v3 p04 = sub(p4, B.p0);
        v3 fv1 = sub(p2, p1);
        v3 fv2;
        if (kind == 0) {
            tetra(a, p01, p03, p04);
            fv2 = sub(p4, p1);
        } else {
            tetra(a, p02, p04, p03);
            fv2 = sub(p3, p1);
        }
        v3 fv3 = sub(p2, p3);
        v3 fv4 = sub(p4, p3);
        fc = mul(add(add(add(p1, p2), p3), p4), 0.25f);
        v3 fn = cross(fv1, fv2);
        float len = dot(fn, fn);
        if (len < 1e-12f) return;
        if (OUTLINE) {
            if (kind == 0) put_outline(ol, 4, p1, p2, p3, p4);
            else put_outline(ol, 4, p1, p2, p4, p3);
        }
        len = sqrtf(len);
        fn1 = dvs_rcp(fn, len);
        v3 c2 = cross(fv3, fv4);
        A = (len + sqrtf(dot(c2, c2))) * 0.5f;
    }
    face_forces<WAVES, FIELD>(o, B, a, fc, fn1, A);
}

// A surface-loop face whose three corners are all under water
// (:1618-1647, then :1650-1686).
template <bool WAVES, bool OUTLINE = false>
__device__ __forceinline__ void face_full(const OceanDev& o, const BodyParams& B, Acc& a,
                                          float4 q1, float4 q2, float4 q3, float* ol = nullptr)
{
    v3 p1 = mk(q1.x, q1.y, q1.z), p2 = mk(q2.x, q2.y, q2.z), p3 = mk(q3.x, q3.y, q3.z);
    tetra(a, sub(p1, B.p0), sub(p2, B.p0), sub(p3, B.p0));
    v3 fc, fn1;
    float A;
    if (!tri_props(p1, p2, p3, fc, fn1, A)) return;
    if (OUTLINE) put_outline(ol, 3, p1, p2, p3, p3);
    face_forces<WAVES>(o, B, a, fc, fn1, A);
}

// Face class of the surface loop from the corner depths: 0 above water
// (skipped, :1353-1354), 1 all corners under water, 2 straddling.
__device__ __forceinline__ int face_class(float d0, float d1, float d2)
{
    if (d0 < 0.f && d1 < 0.f && d2 < 0.f) return 0;
    if (d0 < 0.f || d1 < 0.f || d2 < 0.f) return 2;
    return 1;
}

// One face of the surface loop (:1337-1687) given transformed vertices
// (x, y, z, depth).
template <bool CUT64, bool WAVES, bool OUTLINE = false>
__device__ __forceinline__ void face_surface(const OceanDev& o, const BodyParams& B, Acc& a,
                                             float4 q1, float4 q2, float4 q3, float* ol = nullptr)
{
    const int cls = face_class(q1.w, q2.w, q3.w);
    if (cls == 0) return;
    if (cls == 2) {
        face_cut<CUT64, WAVES, OUTLINE>(o, B, a, mk(q1.x, q1.y, q1.z), mk(q2.x, q2.y, q2.z),
                                        mk(q3.x, q3.y, q3.z), q1.w, q2.w, q3.w, ol);
        return;
    }
    face_full<WAVES, OUTLINE>(o, B, a, q1, q2, q3, ol);
}

// One face of the submerged loop (:1748-1789)
__device__ __forceinline__ void face_submerged(const OceanDev& o, const BodyParams& B, Acc& a,
                                               float4 q1, float4 q2, float4 q3)
{
    v3 p1 = mk(q1.x, q1.y, q1.z), p2 = mk(q2.x, q2.y, q2.z), p3 = mk(q3.x, q3.y, q3.z);
    v3 fc, fn1;
    float A;
    if (!tri_props(p1, p2, p3, fc, fn1, A)) return;
    damping(o, B, a, fc, fn1, A);
}

}  // namespace sfh
