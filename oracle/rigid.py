"""CPU restatement of the device rigid-body step (hydro_rigid_step), for
checking the kernel (test infrastructure only).  FP64, the kernel's
equations: external force and torque impulses plus one Newton step of
implicit Euler for the gyroscopic term (Catto, GDC 2015 -- the method
Bullet's btRigidBody uses when BT_ENABLE_GYROSCOPIC_FORCE_IMPLICIT_BODY is
set, as SolidEntity.cpp:1086 does), position from the new velocity and
orientation by the exponential map of the new angular velocity.  The
reference integrates with Bullet on the CPU; this restatement covers free
bodies only (no contacts)."""
from __future__ import annotations

import numpy as np


def quat_to_rot(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = 1 - 2 * (y * y + z * z)
    R[..., 0, 1] = 2 * (x * y - w * z)
    R[..., 0, 2] = 2 * (x * z + w * y)
    R[..., 1, 0] = 2 * (x * y + w * z)
    R[..., 1, 1] = 1 - 2 * (x * x + z * z)
    R[..., 1, 2] = 2 * (y * z - w * x)
    R[..., 2, 0] = 2 * (x * z - w * y)
    R[..., 2, 1] = 2 * (y * z + w * x)
    R[..., 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _skew(a):
    z = np.zeros_like(a[:, 0])
    return np.stack([np.stack([z, -a[:, 2], a[:, 1]], 1), np.stack([a[:, 2], z, -a[:, 0]], 1),
                     np.stack([-a[:, 1], a[:, 0], z], 1)], 1)


def gyro_newton(wb: np.ndarray, I: np.ndarray, dt: float) -> np.ndarray:
    """Change of the body-frame angular velocity from one Newton step of
    implicit Euler on I dw/dt = -w x I w, starting at w."""
    Iw = I * wb
    f = dt * np.cross(wb, Iw)
    J = np.einsum("ij,nj->nij", np.eye(3), I) + dt * (_skew(wb) * I[:, None, :] - _skew(Iw))
    return -np.linalg.solve(J, f[:, :, None])[:, :, 0]


def step(st: np.ndarray, F_hydro: np.ndarray, T_hydro_body: np.ndarray, dt: float, g: float) -> np.ndarray:
    """st: structured hydro_rigid_state array; F_hydro world frame [n,3];
    T_hydro_body body frame [n,3].  Returns the new states."""
    s = st.copy()
    R = quat_to_rot(s["q"])
    F = F_hydro + np.einsum("nij,nj->ni", R, s["thrust_force"])
    F[:, 2] += s["mass"] * g
    Tb = T_hydro_body + s["thrust_torque"]
    I = s["inertia"]
    wb = np.einsum("nji,nj->ni", R, s["w"])
    wb = wb + dt * Tb / I + gyro_newton(wb, I, dt)
    w = np.einsum("nij,nj->ni", R, wb)
    s["w"] = w
    s["v"] = s["v"] + dt * F / s["inertial_mass"][:, None]
    s["p"] = s["p"] + dt * s["v"]
    wn = np.linalg.norm(w, axis=1)
    half = 0.5 * wn * dt
    sc = np.where(wn > 1e-12, np.sin(half) / np.where(wn > 1e-12, wn, 1.0), 0.5 * dt)
    d = np.concatenate([np.cos(half)[:, None], sc[:, None] * w], axis=1)
    q = s["q"]
    nq = np.stack([
        d[:, 0] * q[:, 0] - d[:, 1] * q[:, 1] - d[:, 2] * q[:, 2] - d[:, 3] * q[:, 3],
        d[:, 0] * q[:, 1] + d[:, 1] * q[:, 0] + d[:, 2] * q[:, 3] - d[:, 3] * q[:, 2],
        d[:, 0] * q[:, 2] - d[:, 1] * q[:, 3] + d[:, 2] * q[:, 0] + d[:, 3] * q[:, 1],
        d[:, 0] * q[:, 3] + d[:, 1] * q[:, 2] - d[:, 2] * q[:, 1] + d[:, 3] * q[:, 0],
    ], axis=1)
    s["q"] = nq / np.linalg.norm(nq, axis=1)[:, None]
    return s


def body_pose(st: np.ndarray):
    """(R row-major [n,9], origin, aabb_min, aabb_max) written to the body records."""
    R = quat_to_rot(st["q"])
    e = np.einsum("nij,nj->ni", np.abs(R), st["half_extents"])
    return R.reshape(-1, 9), st["p"].copy(), st["p"] - e, st["p"] + e
