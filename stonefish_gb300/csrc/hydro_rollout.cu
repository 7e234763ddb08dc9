// hydro_rollout.cu -- device-resident rigid-body integration for rollouts of
// many independent hulls, without contacts, with the hydrodynamic wrench from
// either the exact step or the learned surrogate.  The reference steps its
// bodies with Bullet on the CPU; this restates, for free bodies only, how
// Bullet integrates a Stonefish rigid body (btRigidBody with
// BT_ENABLE_GYROSCOPIC_FORCE_IMPLICIT_BODY, set in SolidEntity.cpp:1086),
// so that thousands of environments can be rolled out without leaving the
// GPU.  Per step and hull, with R the body-to-world rotation of q:
//   F     = F_hydro + R f_thrust + (0, 0, mass g)           (NED: +z down)
//   tau_b = R^T T_hydro + t_thrust                           (body frame)
//   v'    = v + dt F / inertial_mass
//   w_b'  = w_b + dt I^-1 tau_b + dW_gyro(w_b)
//   p'    = p + dt v',   q' = exp(dt w') q   (exponential map, normalised)
// where dW_gyro is one Newton step of implicit Euler on I dw/dt = -w x I w
// (Catto, "Numerical Methods", GDC 2015; the method Bullet uses):
//   J = I + dt (skew(w) I - skew(I w)),  dW_gyro = -J^-1 (dt w x I w).
// The body record the hydrodynamics step reads is rewritten from the new
// state (T_CG = T_C = (R(q'), p'), R_O = R(q'), v', w', the rotated AABB).
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/stonefish_hydro.h"
#include "hydro_internal.h"

namespace sfh {

__device__ __forceinline__ void quat_to_rot(const double* q, double* R)
{
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    R[0] = 1 - 2 * (y * y + z * z);
    R[1] = 2 * (x * y - w * z);
    R[2] = 2 * (x * z + w * y);
    R[3] = 2 * (x * y + w * z);
    R[4] = 1 - 2 * (x * x + z * z);
    R[5] = 2 * (y * z - w * x);
    R[6] = 2 * (x * z - w * y);
    R[7] = 2 * (y * z + w * x);
    R[8] = 1 - 2 * (x * x + y * y);
}

__device__ __forceinline__ void write_body(const hydro_rigid_state& s, hydro_body& b)
{
    double R[9];
    quat_to_rot(s.q, R);
    for (int k = 0; k < 9; ++k) {
        b.T_CG.basis[k] = R[k];
        b.T_C.basis[k] = R[k];
        b.R_O[k] = R[k];
    }
    for (int k = 0; k < 3; ++k) {
        b.T_CG.origin[k] = s.p[k];
        b.T_C.origin[k] = s.p[k];
        b.v[k] = s.v[k];
        b.omega[k] = s.w[k];
        const double e = fabs(R[3 * k]) * s.half_extents[0] + fabs(R[3 * k + 1]) * s.half_extents[1] +
                         fabs(R[3 * k + 2]) * s.half_extents[2];
        b.aabb_min[k] = s.p[k] - e;
        b.aabb_max[k] = s.p[k] + e;
    }
}

// x = A^-1 b for a 3x3 row-major matrix (Cramer's rule; A is the Newton
// Jacobian I + O(dt), far from singular).
__device__ __forceinline__ void solve3(const double* A, const double* b, double* x)
{
    const double c0 = A[4] * A[8] - A[5] * A[7];
    const double c1 = A[5] * A[6] - A[3] * A[8];
    const double c2 = A[3] * A[7] - A[4] * A[6];
    const double inv = 1.0 / (A[0] * c0 + A[1] * c1 + A[2] * c2);
    x[0] = (b[0] * c0 + A[1] * (b[2] * A[5] - b[1] * A[8]) + A[2] * (b[1] * A[7] - b[2] * A[4])) * inv;
    x[1] = (A[0] * (b[1] * A[8] - b[2] * A[5]) + b[0] * c1 + A[2] * (b[2] * A[3] - b[1] * A[6])) * inv;
    x[2] = (A[0] * (b[2] * A[4] - b[1] * A[7]) + A[1] * (b[1] * A[6] - b[2] * A[3]) + b[0] * c2) * inv;
}

__global__ void rigid_step_kernel(hydro_rigid_state* __restrict__ states, hydro_body* __restrict__ bodies,
                                  const hydro_wrench* __restrict__ exact, const float* __restrict__ body_wrench,
                                  uint32_t n, double dt, double gravity)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hydro_rigid_state s = states[i];
    double R[9];
    quat_to_rot(s.q, R);
    double F[3] = {0, 0, 0}, Tb[3] = {0, 0, 0};
    if (exact) {
        const hydro_wrench& x = exact[i];
        double T[3];
        for (int k = 0; k < 3; ++k) {
            F[k] = x.Fb[k] + x.Fdq[k] + x.Fdf[k];
            T[k] = x.Tb[k] + x.Tdq[k] + x.Tdf[k];
        }
        for (int k = 0; k < 3; ++k) Tb[k] = R[k] * T[0] + R[3 + k] * T[1] + R[6 + k] * T[2];
    } else if (body_wrench) {
        const float* w = body_wrench + (size_t)i * 6;
        for (int k = 0; k < 3; ++k) F[k] = R[3 * k] * w[0] + R[3 * k + 1] * w[1] + R[3 * k + 2] * w[2];
        for (int k = 0; k < 3; ++k) Tb[k] = w[3 + k];
    }
    for (int k = 0; k < 3; ++k) {
        F[k] += R[3 * k] * s.thrust_force[0] + R[3 * k + 1] * s.thrust_force[1] + R[3 * k + 2] * s.thrust_force[2];
        Tb[k] += s.thrust_torque[k];
    }
    F[2] += s.mass * gravity;
    // angular velocity, body frame: external torque impulse plus the
    // implicit gyroscopic step, both from the current angular velocity
    const double* I = s.inertia;
    double wb[3];
    for (int k = 0; k < 3; ++k) wb[k] = R[k] * s.w[0] + R[3 + k] * s.w[1] + R[6 + k] * s.w[2];
    const double Iw[3] = {I[0] * wb[0], I[1] * wb[1], I[2] * wb[2]};
    const double f[3] = {dt * (wb[1] * Iw[2] - wb[2] * Iw[1]), dt * (wb[2] * Iw[0] - wb[0] * Iw[2]),
                         dt * (wb[0] * Iw[1] - wb[1] * Iw[0])};
    // J = I + dt (skew(w) diag(I) - skew(I w)), skew(a) = [0 -a2 a1; a2 0 -a0; -a1 a0 0]
    const double J[9] = {I[0],
                         dt * (-wb[2] * I[1] + Iw[2]),
                         dt * (wb[1] * I[2] - Iw[1]),
                         dt * (wb[2] * I[0] - Iw[2]),
                         I[1],
                         dt * (-wb[0] * I[2] + Iw[0]),
                         dt * (-wb[1] * I[0] + Iw[1]),
                         dt * (wb[0] * I[1] - Iw[0]),
                         I[2]};
    double dg[3];
    solve3(J, f, dg);
    for (int k = 0; k < 3; ++k) wb[k] += dt * Tb[k] / I[k] - dg[k];
    for (int k = 0; k < 3; ++k) s.w[k] = R[3 * k] * wb[0] + R[3 * k + 1] * wb[1] + R[3 * k + 2] * wb[2];
    // linear velocity and position
    for (int k = 0; k < 3; ++k) {
        s.v[k] += dt * F[k] / s.inertial_mass;
        s.p[k] += dt * s.v[k];
    }
    // orientation: rotation by |w| dt about w, applied in the world frame
    const double wn = sqrt(s.w[0] * s.w[0] + s.w[1] * s.w[1] + s.w[2] * s.w[2]);
    const double half = 0.5 * wn * dt;
    const double sc = wn > 1e-12 ? sin(half) / wn : 0.5 * dt;
    const double dq[4] = {cos(half), sc * s.w[0], sc * s.w[1], sc * s.w[2]};
    const double qw = s.q[0], qx = s.q[1], qy = s.q[2], qz = s.q[3];
    double nq[4] = {dq[0] * qw - dq[1] * qx - dq[2] * qy - dq[3] * qz,
                    dq[0] * qx + dq[1] * qw + dq[2] * qz - dq[3] * qy,
                    dq[0] * qy - dq[1] * qz + dq[2] * qw + dq[3] * qx,
                    dq[0] * qz + dq[1] * qy - dq[2] * qx + dq[3] * qw};
    const double inv = 1.0 / sqrt(nq[0] * nq[0] + nq[1] * nq[1] + nq[2] * nq[2] + nq[3] * nq[3]);
    for (int k = 0; k < 4; ++k) s.q[k] = nq[k] * inv;
    states[i] = s;
    write_body(s, bodies[i]);
}

__global__ void rigid_write_bodies_kernel(const hydro_rigid_state* __restrict__ states,
                                          hydro_body* __restrict__ bodies, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    write_body(states[i], bodies[i]);
}

cudaError_t launch_rigid_step(hydro_rigid_state* states, hydro_body* bodies, const hydro_wrench* exact,
                              const float* body_wrench, uint32_t n, double dt, double gravity, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    rigid_step_kernel<<<(n + 127) / 128, 128, 0, s>>>(states, bodies, exact, body_wrench, n, dt, gravity);
    return cudaGetLastError();
}

cudaError_t launch_rigid_write_bodies(const hydro_rigid_state* states, hydro_body* bodies, uint32_t n,
                                      cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    rigid_write_bodies_kernel<<<(n + 127) / 128, 128, 0, s>>>(states, bodies, n);
    return cudaGetLastError();
}

}  // namespace sfh
