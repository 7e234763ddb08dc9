// hydro_cable.cu -- CableEntity::ComputeHydrodynamicForces
// (Library/src/entities/CableEntity.cpp:240-376) for many cables at once.
//
// A cable is a chain of nodes; each segment between consecutive nodes is a
// cylinder of the cable's radius.  Per segment: the submerged volume from the
// depths of its end points (eight cases of partial submersion), buoyancy
// (-V rho g), form drag and skin friction from the mean node velocity
// relative to the current at the segment's midpoint; each segment gives half
// of each force to both of its nodes, and the end nodes' forces are doubled.
// One warp per cable: the lanes compute the segments into a scratch array,
// then the nodes gather their two segments in the reference's order (the
// segment before, then the segment after).  All arithmetic is FP64 as in the
// reference; depths go through the FP32 Ocean::GetDepth as there.
#include <cstdint>
#include <cuda_runtime.h>

#include "hydro_internal.h"

namespace sfh {

namespace cable {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps = 2.220446049250313080847e-16;   // SIMD_EPSILON (double)

__device__ __forceinline__ bool fuzzy_zero(double x) { return fabs(x) < kEps; }

__device__ __forceinline__ double bt_acos(double x)
{
    if (x < -1.0) x = -1.0;
    if (x > 1.0) x = 1.0;
    return acos(x);
}

// CableEntity::circularSegmentArea (CableEntity.cpp:218-238)
__device__ double circular_segment_area(double h, double r)
{
    if (h <= 0.0) return 0.0;
    if (h >= 2.0 * r) return kPi * r * r;
    if (h > r) {
        h = 2.0 * r - h;
        const double theta = 2.0 * bt_acos((r - h) / r);
        return r * r * (kPi - (theta - sin(theta)) / 2.0);
    }
    const double theta = 2.0 * bt_acos((r - h) / r);
    return (r * r / 2.0) * (theta - sin(theta));
}

// Ocean::GetFluidVelocity(const Vector3&) (Ocean.cpp:183-196): FP64 sum of
// the enabled currents.
__device__ void fluid_velocity64(const OceanDev& o, const double* p, double* fv)
{
    fv[0] = fv[1] = fv[2] = 0.0;
    for (int i = 0; i < o.n_currents; ++i) {
        const hydro_current& c = o.currents[i];
        if (!c.enabled) continue;
        double u[3] = {0.0, 0.0, 0.0};
        if (c.type == HYDRO_CURRENT_UNIFORM) {
            u[0] = c.vel[0];
            u[1] = c.vel[1];
            u[2] = c.vel[2];
        } else if (c.type == HYDRO_CURRENT_JET) {
            jet_velocity(c, p, u);
        } else if (c.type == HYDRO_CURRENT_PIPE) {
            pipe_velocity(c, p, u);
        }
        fv[0] += u[0];
        fv[1] += u[1];
        fv[2] += u[2];
    }
}

// Ocean::GetDepth(const Vector3&) (Ocean.cpp:170-173): through FP32
__device__ __forceinline__ double depth64(const OceanDev& o, const double* p)
{
    return (double)depth_at(o, (float)p[0], (float)p[1], (float)p[2]);
}

// One segment's contribution (Fb, Fdq, Fdf), to be halved onto its nodes.
__device__ void segment(const OceanDev& o, SettingsDev st, const hydro_cable& cb, const double* xa,
                        const double* xb, const double* va, const double* vb, double* out9)
{
    for (int k = 0; k < 9; ++k) out9[k] = 0.0;
    const double r = cb.radius;
    double p1[3] = {xa[0], xa[1], xa[2]}, p2[3] = {xb[0], xb[1], xb[2]};
    double d1 = depth64(o, p1), d2 = depth64(o, p2);
    if (d1 > d2) {                                            // shallower point first
        for (int k = 0; k < 3; ++k) {
            const double t = p1[k];
            p1[k] = p2[k];
            p2[k] = t;
        }
        const double t = d1;
        d1 = d2;
        d2 = t;
    }
    const double dz = d2 - d1;
    const double hx = p2[0] - p1[0], hy = p2[1] - p1[1];
    const double h2 = hx * hx + hy * hy + 0.0 * 0.0;          // btVector3::safeNorm
    const double dxy = h2 > kEps ? sqrt(h2) : 0.0;
    const double sv[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    const double L = sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
    const double alpha = atan(dz / dxy);
    const double margin = fuzzy_zero(dxy) ? 0.0 : r * cos(alpha);
    double V = 0.0;
    if (d2 < -margin) {
        return;                                               // out of the water
    } else if (d1 > margin) {
        V = kPi * r * r * L;                                  // fully submerged
    } else if (fuzzy_zero(dxy)) {                             // vertical
        const double l = d2 < dz ? d2 : dz;                   // btMin
        V = kPi * r * r * l;
    } else if (fuzzy_zero(dz)) {                              // horizontal
        V = circular_segment_area(d1 + r, r) * L;
    } else if (fabs(d1) <= margin && fabs(d2) <= margin) {    // both caps partly submerged
        const double A1 = circular_segment_area(d1 / cos(alpha) + r, r);
        const double A2 = circular_segment_area(d2 / cos(alpha) + r, r);
        V = (A1 + A2) / 2.0 * L;
    } else if (d1 < -margin && d2 > margin) {                 // first cap out, second submerged
        const double l1 = (d2 - r * cos(alpha)) / sin(alpha);
        const double l2 = 2.0 * r * cos(alpha);
        V = kPi * r * r * (l1 + l2 / 2.0);
    } else if (d2 <= margin) {                                // first cap out, second partly
        const double a = r + d2 / cos(alpha);
        const double l = a / sin(alpha);
        V = circular_segment_area(a, r) * l / 2.0;
    } else if (d1 >= -margin) {                               // first cap partly, second submerged
        const double a = r - d1 / cos(alpha);
        const double l = a / sin(alpha);
        V = kPi * r * r * L - circular_segment_area(a, r) * l / 2.0;
    }
    if (cb.buoyancy && st.buoyancy) {                         // :325-333
        const double k = -V * o.density;
        out9[0] = k * 0.0;
        out9[1] = k * 0.0;
        out9[2] = k * o.gravity;
    }
    if (st.damping && V > 0.0) {                              // :335-364
        const double p[3] = {(p1[0] + p2[0]) / 2.0, (p1[1] + p2[1]) / 2.0, (p1[2] + p2[2]) / 2.0};
        const double v[3] = {(va[0] + vb[0]) / 2.0, (va[1] + vb[1]) / 2.0, (va[2] + vb[2]) / 2.0};
        double wv[3];
        fluid_velocity64(o, p, wv);
        const double rv[3] = {v[0] - wv[0], v[1] - wv[1], v[2] - wv[2]};
        const double Cd = 0.5;
        const double f1 = fabs(sv[0] * rv[0] + sv[1] * rv[1] + sv[2] * rv[2]);
        const double f2 = V / (kPi * r * r * L);
        const double rl = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
        const double S = 2.0 * r * L;
        const double q = -(1.0 - f1) * f2 * 0.5 * o.density * Cd * S * rl;
        const double Sf = f2 * ((2.0 * kPi) * r * L);
        for (int k = 0; k < 3; ++k) {
            out9[3 + k] = q * rv[k];
            out9[6 + k] = -Sf * rv[k];
        }
    }
}

}  // namespace cable

__global__ void cable_kernel(const hydro_cable* __restrict__ cables, uint32_t n_cables, uint32_t n_nodes_total,
                             const double* __restrict__ x, const double* __restrict__ v, OceanDev o, SettingsDev st,
                             double* __restrict__ seg, hydro_cable_node_forces* __restrict__ out,
                             unsigned* __restrict__ bad)
{
    const int lane = threadIdx.x & 31;
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= n_cables) return;
    const hydro_cable cb = cables[c];
    if (cb.mode != HYDRO_MODE_FLOATING && cb.mode != HYDRO_MODE_SUBMERGED) return;   // :242
    const uint32_t n = cb.n_nodes, f = cb.first_node;
    if (n == 0) return;
    if ((uint64_t)f + n > n_nodes_total) {                   // node range outside the arrays
        if (lane == 0) atomicOr(bad, 1u);
        return;
    }
    for (uint32_t i = lane; i + 1 < n; i += 32)
        cable::segment(o, st, cb, x + 3 * (size_t)(f + i), x + 3 * (size_t)(f + i + 1), v + 3 * (size_t)(f + i),
                       v + 3 * (size_t)(f + i + 1), seg + 9 * (size_t)(f + i));
    __syncwarp();
    __threadfence_block();
    for (uint32_t i = lane; i < n; i += 32) {
        double acc[9];
        for (int k = 0; k < 9; ++k) acc[k] = 0.0;            // clearForces (:245-246)
        if (i > 0) {
            const double* s = seg + 9 * (size_t)(f + i - 1);
            for (int k = 0; k < 9; ++k) acc[k] += s[k] / 2.0;
        }
        if (i + 1 < n) {
            const double* s = seg + 9 * (size_t)(f + i);
            for (int k = 0; k < 9; ++k) acc[k] += s[k] / 2.0;
        }
        if (i == 0 || i + 1 == n)                             // end nodes (:367-373)
            for (int k = 0; k < 9; ++k) acc[k] *= 2.0;
        hydro_cable_node_forces& r = out[f + i];
        for (int k = 0; k < 3; ++k) {
            r.Fb[k] = acc[k];
            r.Fdq[k] = acc[3 + k];
            r.Fdf[k] = acc[6 + k];
        }
    }
}

cudaError_t launch_cable(const hydro_cable* cables, uint32_t n_cables, uint32_t n_nodes_total, const double* x,
                         const double* v, OceanDev o, SettingsDev st, double* seg, hydro_cable_node_forces* out,
                         unsigned* bad, cudaStream_t s)
{
    if (n_cables == 0) return cudaSuccess;
    const uint32_t warps_per_block = 4;
    const uint32_t blocks = (n_cables + warps_per_block - 1) / warps_per_block;
    cable_kernel<<<blocks, 32 * warps_per_block, 0, s>>>(cables, n_cables, n_nodes_total, x, v, o, st, seg, out,
                                                         bad);
    return cudaGetLastError();
}

}  // namespace sfh
