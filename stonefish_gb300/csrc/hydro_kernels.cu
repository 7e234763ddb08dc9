// hydro_kernels.cu -- GB300 kernels of the hydrodynamic wrench path.
//
// The batched step replaces the per-body loop of the hydrodynamics block of
// SimulationManager::SimulationTickCallback (SimulationManager.cpp:1620-1655):
// one CTA per chunk (a run of tiles of one body's mesh).  A CTA
//   1. derives the body's FP32 parameters and its fluid position
//      (SolidEntity::ComputeHydrodynamicForces :1799-1850,
//      CheckBodyFluidPosition :1239-1261);
//   2. per tile, transforms each distinct vertex once into shared memory
//      with its depth (Ocean::GetDepth), then gives each thread faces that
//      gather their corners from shared memory (surface loop :1337-1687 or
//      submerged loop :1748-1789);
//   3. sums the 23 per-face quantities: FP32 per thread over at most
//      kFlushFaces faces, a butterfly reduce-scatter across the warp, then a
//      two-sum (float-float) accumulator per warp lane, combined across warps
//      and stored as one FP64 partial per chunk;
//   4. the CTA that completes a body's last chunk (per-body ticket counter)
//      adds the body's partials in chunk order in FP64 and applies the FP64
//      finalisation: buoyancy (:1689-1720, :1828-1836), the stale-output
//      rules and CorrectHydrodynamicForces (:1263-1287).
// The result does not depend on scheduling: every sum has a fixed order.
#include <cstdint>
#include <cuda_runtime.h>

#include "hydro_internal.h"

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
__device__ void body_prologue(const KParams& P, uint32_t body, const BodyInfo& bi,
                              BodyParams& B, int& mismatch)
{
    const hydro_body* b = P.bodies + body;
    int loop = LOOP_NONE, pos = HYDRO_SKIPPED, buoy = P.st.buoyancy, damp = P.st.damping;
    mismatch = (b->mesh != bi.mesh);
    if (P.op == OP_BODY) {
        if (!mismatch && (b->mode == HYDRO_MODE_FLOATING || b->mode == HYDRO_MODE_SUBMERGED)) {
            pos = classify(P.ocean, b->aabb_min, b->aabb_max);
            if (pos == HYDRO_INSIDE) {
                loop = damp ? LOOP_SUBMERGED : LOOP_NONE;
            } else if (pos == HYDRO_CROSSING_SURFACE) {
                loop = LOOP_SURFACE;
                buoy = buoy && (b->buoyancy != 0);
            }
        }
    } else if (!mismatch) {
        loop = (P.op == OP_SURFACE) ? LOOP_SURFACE : LOOP_SUBMERGED;
        pos = (P.op == OP_SURFACE) ? HYDRO_CROSSING_SURFACE : HYDRO_INSIDE;
        if (P.op == OP_SUBMERGED) damp = 1;
    }
    if (bi.mesh == HYDRO_NO_MESH) loop = LOOP_NONE;
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) B.TC[4 * r + c] = (float)b->T_C.basis[3 * r + c];
        B.TC[4 * r + 3] = (float)b->T_C.origin[r];
    }
    B.p = mk((float)b->T_CG.origin[0], (float)b->T_CG.origin[1], (float)b->T_CG.origin[2]);
    B.p0 = mk(B.p.x, B.p.y, 0.f);
    B.v = mk((float)b->v[0], (float)b->v[1], (float)b->v[2]);
    B.omega = mk((float)b->omega[0], (float)b->omega[1], (float)b->omega[2]);
    B.loop = loop;
    B.buoyancy = buoy;
    B.damping = damp;
    B.position = pos;
}

// Finalisation of one body by the CTA that completed its last chunk.
__device__ void body_finalize(const KParams& P, uint32_t body, const BodyParams& B,
                              int mismatch, const double* S, int status)
{
    const hydro_body* b = P.bodies + body;
    hydro_wrench w = P.io[body];
    const BodyInfo bi = P.binfo[body];
    const bool null_mesh = (bi.mesh == HYDRO_NO_MESH);
    if (mismatch) {
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
            finalize_surface(P.ocean, B.buoyancy, B.damping, b->T_CG.origin,
                             (double)B.p0.x, (double)B.p0.y, S, w);
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
                finalize_surface(P.ocean, B.buoyancy, B.damping, b->T_CG.origin,
                                 (double)B.p0.x, (double)B.p0.y, S, w);
            }
            if (B.damping)
                correct4(P.ocean.density, w.Fdq, w.Tdq, w.Fdf, w.Tdf, b->Cd, b->Cf, b->R_O);
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

// ------------------------------------------------------------ main kernel
struct __align__(16) ChunkSmem {
    float4 verts[kTileVerts];
    float2 red[kWarps][32];
    double sums[32];
    BodyParams B;
    int mismatch;
    int last;
};

template <bool CUT64, bool WAVES>
__global__ void __launch_bounds__(kBlock, 2) chunk_kernel(const KParams P)
{
    __shared__ ChunkSmem S;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const ChunkDesc ch = P.chunks[blockIdx.x];
    if (tid == 0) {
        const BodyInfo bi = P.binfo[ch.body];
        int mm = 0;
        body_prologue(P, ch.body, bi, S.B, mm);
        S.mismatch = mm;
    }
    __syncthreads();
    const BodyParams B = S.B;
    double* part = P.partials + (size_t)blockIdx.x * kPartialStride;

    if (B.loop != LOOP_NONE) {
        Acc acc;
#pragma unroll
        for (int k = 0; k < kQ; ++k) acc.q[k] = 0.f;
        float hi = 0.f, lo = 0.f;
        int since_flush = 0;
        for (uint32_t t = 0; t < ch.n_tiles; ++t) {
            const TileDesc td = P.tiles[ch.first_tile + t];
            const int nv = td.nv;
            const int nvp = (nv + 3) & ~3;
            for (int v = tid; v < nv; v += kBlock) {
                float x = __ldg(td.block + v);
                float y = __ldg(td.block + nvp + v);
                float z = __ldg(td.block + 2 * nvp + v);
                v3 p = xform(B.TC, x, y, z);
                float d = WAVES ? depth_at(P.ocean, p.x, p.y, p.z) : p.z;
                S.verts[v] = make_float4(p.x, p.y, p.z, d);
            }
            __syncthreads();
            const uint16_t* idx = reinterpret_cast<const uint16_t*>(td.block + 3 * nvp);
            for (int f = tid; f < td.nf; f += kBlock) {
                const int i0 = __ldg(idx + 3 * f);
                const int i1 = __ldg(idx + 3 * f + 1);
                const int i2 = __ldg(idx + 3 * f + 2);
                const float4 q1 = S.verts[i0], q2 = S.verts[i1], q3 = S.verts[i2];
                if (B.loop == LOOP_SURFACE) face_surface<CUT64>(P.ocean, B, acc, q1, q2, q3);
                else face_submerged(P.ocean, B, acc, q1, q2, q3);
            }
            __syncthreads();
            since_flush += (kTileFaces + kBlock - 1) / kBlock;
            if (since_flush + (kTileFaces + kBlock - 1) / kBlock > kFlushFaces) {
                flush(acc, hi, lo);
                since_flush = 0;
            }
        }
        flush(acc, hi, lo);
        S.red[warp][lane] = make_float2(hi, lo);
        __syncthreads();
        if (warp == 0) {
            float H = S.red[0][lane].x, L = S.red[0][lane].y;
            for (int w = 1; w < kWarps; ++w) {
                two_sum_acc(H, L, S.red[w][lane].x);
                L += S.red[w][lane].y;
            }
            if (lane < kQ) part[lane] = (double)H + (double)L;
            if (lane == kQ) part[lane] = 0.0;   // status slot
            __threadfence();
        }
    }
    __syncthreads();

    // ticket: the CTA finishing a body's last chunk finalises the body
    const BodyInfo bi = P.binfo[ch.body];
    if (tid == 0) {
        __threadfence();
        unsigned prev = atomicAdd(P.counters + ch.body, 1u);
        S.last = (prev + 1u == bi.n_chunks);
    }
    __syncthreads();
    if (!S.last) return;
    __threadfence();
    if (warp == 0) {
        double s = 0.0;
        int status = 0;
        if (B.loop != LOOP_NONE) {
            for (uint32_t c = 0; c < bi.n_chunks; ++c) {
                const double* pc = P.partials + (size_t)(bi.first_chunk + c) * kPartialStride;
                if (lane < kQ) s += __ldcg(pc + lane);
                else if (lane == kQ) status |= (int)__ldcg(pc + lane);
            }
        }
        S.sums[lane] = (lane < kQ) ? s : (double)status;
    }
    __syncthreads();
    if (tid == 0) {
        body_finalize(P, ch.body, B, S.mismatch, S.sums, (int)S.sums[kQ]);
        P.counters[ch.body] = 0u;
    }
}

cudaError_t launch_chunks(const KParams& P, uint32_t n_chunks, int cut64, cudaStream_t s)
{
    if (n_chunks == 0) return cudaSuccess;
    dim3 grid(n_chunks), block(kBlock);
    const bool waves = P.ocean.waves != 0;
    if (cut64) {
        if (waves) chunk_kernel<true, true><<<grid, block, 0, s>>>(P);
        else chunk_kernel<true, false><<<grid, block, 0, s>>>(P);
    } else {
        if (waves) chunk_kernel<false, true><<<grid, block, 0, s>>>(P);
        else chunk_kernel<false, false><<<grid, block, 0, s>>>(P);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------- debug face terms
template <bool CUT64>
__global__ void __launch_bounds__(kBlock) face_terms_kernel(const TileDesc* tiles, uint32_t first_tile,
                                                            const hydro_body* body, OceanDev ocean,
                                                            SettingsDev st, float* out)
{
    __shared__ float4 verts[kTileVerts];
    __shared__ BodyParams Bs;
    const int tid = threadIdx.x;
    const TileDesc td = tiles[first_tile + blockIdx.x];
    if (tid == 0) {
        KParams P{};
        P.bodies = body;
        P.ocean = ocean;
        P.st = st;
        P.op = OP_SURFACE;
        BodyInfo bi{0u, 1u, body->mesh, 0u};
        int mm = 0;
        body_prologue(P, 0, bi, Bs, mm);
    }
    __syncthreads();
    const BodyParams B = Bs;
    const int nv = td.nv, nvp = (nv + 3) & ~3;
    for (int v = tid; v < nv; v += kBlock) {
        v3 p = xform(B.TC, td.block[v], td.block[nvp + v], td.block[2 * nvp + v]);
        verts[v] = make_float4(p.x, p.y, p.z, depth_at(ocean, p.x, p.y, p.z));
    }
    __syncthreads();
    const uint16_t* idx = reinterpret_cast<const uint16_t*>(td.block + 3 * nvp);
    for (int f = tid; f < td.nf; f += kBlock) {
        Acc a;
        for (int k = 0; k < kQ; ++k) a.q[k] = 0.f;
        face_surface<CUT64>(ocean, B, a, verts[idx[3 * f]], verts[idx[3 * f + 1]], verts[idx[3 * f + 2]]);
        float* o = out + (size_t)(td.first_face + f) * kQ;
        for (int k = 0; k < kQ; ++k) o[k] = a.q[k];
    }
}

cudaError_t launch_face_terms(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles,
                              const hydro_body* body, OceanDev ocean, SettingsDev st,
                              int cut64, float* out, cudaStream_t s)
{
    if (n_tiles == 0) return cudaSuccess;
    if (cut64) face_terms_kernel<true><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, out);
    else face_terms_kernel<false><<<n_tiles, kBlock, 0, s>>>(tiles, first_tile, body, ocean, st, out);
    return cudaGetLastError();
}

// ------------------------------------------------------------ small kernels
__global__ void correct_kernel(double density, double* io, const double* Cd, const double* Cf,
                               const double* R_O)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        correct4(density, io, io + 3, io + 6, io + 9, Cd, Cf, R_O);
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
