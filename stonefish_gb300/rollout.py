"""Device-resident rollouts of many independent hulls: every step computes
the hydrodynamic wrench (exact step, or the learned surrogate with its gate)
and advances each hull by semi-implicit Euler (``hydro_rigid_step``); a
whole rollout is captured once as a CUDA graph and replayed.

The reference advances bodies with Bullet on the CPU and recomputes
hydrodynamics every few physics steps (SimulationManager.cpp:1584); here the
wrench is recomputed at every step, and there are no contacts.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import abi, meshes
from . import surrogate as S
from .hydro import HydroContext, _check

# thrusters: body-frame position and unit direction; each hull draws one
# fixed thrust per thruster (two surge thrusters astern, two heave thrusters)
THRUSTERS = (
    ((-0.9, 0.2, 0.0), (1.0, 0.0, 0.0)),
    ((-0.9, -0.2, 0.0), (1.0, 0.0, 0.0)),
    ((0.6, 0.0, 0.0), (0.0, 0.0, 1.0)),
    ((-0.6, 0.0, 0.0), (0.0, 0.0, 1.0)),
)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def hull_inertia(mass: float, radius: float, length: float) -> tuple[float, float, float]:
    """Diagonal inertia of a solid cylinder of the hull's overall length
    (axis x) -- a simple stand-in for a ballasted hull."""
    L = length + 2.0 * radius
    ixx = 0.5 * mass * radius * radius
    iyy = mass * (3.0 * radius * radius + L * L) / 12.0
    return ixx, iyy, iyy


def cylinder_added_mass(radius: float, overall_length: float, rho: float):
    """Added mass and inertia of an x-axis cylinder as the reference's
    cylindrical approximation defines them (SolidEntity::ComputeCylindricalApprox,
    SolidEntity.cpp:826-839): m1 = rho pi r^2 along the axis, m2 = rho pi r^2 l
    across it, I1 = 0 about the axis, I2 = pi rho l^2 r^3 / 12 across it;
    returns ((m1, m2, m2), (0, I2, I2)) in the body frame."""
    m1 = rho * math.pi * radius * radius
    m2 = m1 * overall_length
    i2 = math.pi * rho * overall_length * overall_length * radius ** 3 / 12.0
    return (m1, m2, m2), (0.0, i2, i2)


def yaw_roll_pitch_quaternions(rng: np.random.Generator, n: int, tilt: float) -> np.ndarray:
    """(w, x, y, z) quaternions: uniform yaw, roll and pitch uniform in
    [-tilt, tilt] (Z-Y-X order)."""
    yaw = rng.uniform(-math.pi, math.pi, n)
    pitch = rng.uniform(-tilt, tilt, n)
    roll = rng.uniform(-tilt, tilt, n)
    cy, sy = np.cos(yaw / 2), np.sin(yaw / 2)
    cp, sp = np.cos(pitch / 2), np.sin(pitch / 2)
    cr, sr = np.cos(roll / 2), np.sin(roll / 2)
    return np.stack([cr * cp * cy + sr * sp * sy, sr * cp * cy - cr * sp * sy,
                     cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy], axis=1)


FLOAT_HEIGHT = 0.166  # CG height above the surface of a level 50 kg hull (8.4 cm immersed)


def initial_states(rng: np.random.Generator, n: int, mass: float = 50.0, thrust: float = 20.0,
                   extent: float = 102.4, surface=None, height=(FLOAT_HEIGHT - 0.04, FLOAT_HEIGHT + 0.04),
                   tilt: float = 0.1, rho: float = 1025.0) -> np.ndarray:
    """Hulls at rest near their floating height with fixed thrusts drawn
    U(-thrust, thrust) N.  ``surface(xy) -> z`` gives the surface z (NED) under
    each hull (flat: 0); the CG starts ``height`` above it.  The hulls are in
    the reference's SUBMERGED physics mode, so the rigid body carries the
    added mass and inertia of the cylindrical approximation
    (SolidEntity::getAugmentedMass/getAugmentedInertia, SolidEntity.cpp:657-670):
    inertial mass = mass + mean(added mass), inertia = solid inertia + added."""
    st = np.zeros(n, dtype=abi.RIGID_DTYPE)
    st["p"][:, 0] = rng.uniform(0.0, extent, n)
    st["p"][:, 1] = rng.uniform(0.0, extent, n)
    z_s = np.zeros(n) if surface is None else surface(st["p"][:, :2])
    st["p"][:, 2] = z_s - rng.uniform(height[0], height[1], n)
    st["q"] = yaw_roll_pitch_quaternions(rng, n, tilt)
    f = rng.uniform(-thrust, thrust, (n, len(THRUSTERS)))
    F = np.zeros((n, 3))
    T = np.zeros((n, 3))
    for k, (r, d) in enumerate(THRUSTERS):
        fk = f[:, k:k + 1] * np.asarray(d)[None, :]
        F += fk
        T += np.cross(np.asarray(r)[None, :], fk)
    st["thrust_force"] = F
    st["thrust_torque"] = T
    am, ai = cylinder_added_mass(S.HULL_RADIUS, S.HULL_LENGTH + 2.0 * S.HULL_RADIUS, rho)
    st["mass"] = mass
    st["inertial_mass"] = mass + sum(am) / 3.0
    st["inertia"] = np.asarray(hull_inertia(mass, S.HULL_RADIUS, S.HULL_LENGTH)) + np.asarray(ai)
    st["half_extents"] = (0.5 * S.HULL_LENGTH + S.HULL_RADIUS, S.HULL_RADIUS, S.HULL_RADIUS)
    return st


def static_bodies(n: int, mesh_id: int) -> np.ndarray:
    """Body records with the hull's coefficients; poses come from the states."""
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    b["Cd"] = S.HULL_CD
    b["Cf"] = S.HULL_CF
    b["volume"] = meshes.capped_cylinder_volume(S.HULL_RADIUS, S.HULL_LENGTH)
    b["surface"] = meshes.capped_cylinder_surface(S.HULL_RADIUS, S.HULL_LENGTH)
    b["mesh"] = mesh_id
    b["mode"] = abi.MODE_SUBMERGED
    b["buoyancy"] = 1
    return b


class Rollout:
    """n hulls stepped on the device; ``mode`` is "exact" or "surrogate"."""

    def __init__(self, hctx: HydroContext, mesh_id: int, n: int, ocean: abi.Ocean, settings: abi.Settings,
                 mode: str = "exact", predictor: S.GatedPredictor | None = None, dt: float = 0.01):
        assert mode in ("exact", "surrogate")
        assert mode == "exact" or (predictor is not None and predictor.n == n)
        self.h = hctx
        self.lib = hctx.lib
        self.n = n
        self.ocean = ocean
        self.settings = settings
        self.mode = mode
        self.pred = predictor
        self.dt = dt
        self.gravity = float(ocean.gravity)
        dev = torch.device("cuda", hctx.device)
        self.states = torch.zeros(n * abi.RIGID_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.bodies = torch.zeros(n * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.io = torch.zeros(n * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.batch = hctx.batch(np.full(n, mesh_id, dtype=np.uint32)) if mode == "exact" else None
        self.mesh_id = mesh_id
        self.graph = None
        self.snaps = None

    def _ck(self, st):
        _check(self.lib, self.h.ctx, st)

    def reset(self, states: np.ndarray) -> None:
        assert states.dtype == abi.RIGID_DTYPE and states.size == self.n
        self.states.copy_(torch.from_numpy(np.frombuffer(states.tobytes(), dtype=np.uint8).copy()))
        self.bodies.copy_(torch.from_numpy(np.frombuffer(static_bodies(self.n, self.mesh_id).tobytes(),
                                                         dtype=np.uint8).copy()))
        self.io.zero_()
        s = torch.cuda.current_stream().cuda_stream
        self._ck(self.lib.hydro_rigid_write_bodies(self.h.ctx, _ptr(self.states), _ptr(self.bodies), self.n, s))

    def step(self) -> int:
        """Enqueues one step; returns the number of kernels it launched."""
        s = torch.cuda.current_stream().cuda_stream
        if self.mode == "exact":
            self.batch.compute_device(self.bodies.data_ptr(), self.ocean, self.settings, self.io.data_ptr(), s)
            self._ck(self.lib.hydro_rigid_step(self.h.ctx, _ptr(self.states), _ptr(self.bodies), _ptr(self.io),
                                               None, self.n, self.dt, self.gravity, s))
            return self.batch.last_launches() + 1
        out = self.pred.predict(self.bodies)
        self._ck(self.lib.hydro_rigid_step(self.h.ctx, _ptr(self.states), _ptr(self.bodies), None, _ptr(out),
                                           self.n, self.dt, self.gravity, s))
        return self.pred.launches + 1

    def capture(self, steps: int, snap_every: int = 100) -> int:
        """Captures ``steps`` steps (with a state snapshot every snap_every
        steps) into one CUDA graph; returns the kernels per replay."""
        n_snap = steps // snap_every
        self.snaps = torch.zeros((n_snap, self.states.numel()), dtype=torch.uint8, device=self.states.device)
        # one eager wrench evaluation first (the state is not advanced) so that
        # every lazily created resource exists before the capture
        s = torch.cuda.current_stream().cuda_stream
        if self.mode == "exact":
            self.batch.compute_device(self.bodies.data_ptr(), self.ocean, self.settings, self.io.data_ptr(), s)
            self.io.zero_()
        else:
            self.pred.predict(self.bodies)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        kernels = 0
        with torch.cuda.graph(self.graph):
            for i in range(steps):
                kernels += self.step()
                if (i + 1) % snap_every == 0:
                    self.snaps[(i + 1) // snap_every - 1].copy_(self.states)
        return kernels

    def replay(self) -> None:
        self.graph.replay()

    def host_states(self) -> np.ndarray:
        return np.frombuffer(self.states.cpu().numpy().tobytes(), dtype=abi.RIGID_DTYPE).copy()

    def snapshots(self) -> list[np.ndarray]:
        return [np.frombuffer(s.cpu().numpy().tobytes(), dtype=abi.RIGID_DTYPE).copy() for s in self.snaps]

    def close(self):
        if self.batch is not None:
            self.batch.close()


def surface_z(hctx: HydroContext, ocean: abi.Ocean):
    """surface(xy) -> surface z (NED) from the library's own depth lookup."""
    def f(xy):
        pts = np.zeros((len(xy), 3), dtype=np.float32)
        pts[:, :2] = xy
        return -hctx.depth(ocean, pts).astype(np.float64)   # depth of z = 0 is -surface z
    return f


def divergence(a: np.ndarray, b: np.ndarray, start: np.ndarray) -> dict:
    """Position and attitude differences between two sets of hull states,
    with the distance travelled (from ``start``) for scale; hulls whose state
    is not finite in either run are counted and left out."""
    ok = np.all(np.isfinite(a["p"]), axis=1) & np.all(np.isfinite(b["p"]), axis=1)
    ok &= np.all(np.isfinite(a["q"]), axis=1) & np.all(np.isfinite(b["q"]), axis=1)
    a, b, start = a[ok], b[ok], start[ok]
    if a.size == 0:
        return {"finite_envs": 0}
    dp = np.linalg.norm(a["p"] - b["p"], axis=1)
    dot = np.abs(np.sum(a["q"] * b["q"], axis=1)).clip(0.0, 1.0)
    ang = 2.0 * np.arccos(dot)
    # the angle between the hulls' long (body x) axes: the attitude up to the
    # roll about that axis, which an axisymmetric hull's hydrodynamics do not
    # see and nothing restores
    axis = np.arccos(np.sum(body_x_axis(a["q"]) * body_x_axis(b["q"]), axis=1).clip(-1.0, 1.0))
    travel = np.linalg.norm(a["p"] - start["p"], axis=1)
    q = lambda x, p: float(np.quantile(x, p))
    return {"pos_median_m": q(dp, 0.5), "pos_p95_m": q(dp, 0.95), "pos_max_m": float(dp.max()),
            "att_median_rad": q(ang, 0.5), "att_p95_rad": q(ang, 0.95),
            "axis_median_rad": q(axis, 0.5), "axis_p95_rad": q(axis, 0.95),
            "travel_median_m": q(travel, 0.5), "finite_envs": int(ok.sum())}


def body_x_axis(q: np.ndarray) -> np.ndarray:
    """World direction of the body x axis for quaternions (w, x, y, z)."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([1.0 - 2.0 * (y * y + z * z), 2.0 * (x * y + z * w), 2.0 * (x * z - y * w)], axis=1)


def state_stats(s: np.ndarray) -> dict:
    ok = np.all(np.isfinite(s["p"]), axis=1)
    v = np.linalg.norm(s["v"][ok], axis=1)
    w = np.linalg.norm(s["w"][ok], axis=1)
    return {"finite_envs": int(ok.sum()), "speed_p50": float(np.median(v)) if v.size else None,
            "speed_max": float(v.max()) if v.size else None,
            "rate_p50": float(np.median(w)) if w.size else None,
            "rate_max": float(w.max()) if w.size else None,
            "z_p50": float(np.median(s["p"][ok, 2])) if v.size else None}
