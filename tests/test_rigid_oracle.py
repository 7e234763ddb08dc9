"""The CPU restatement of the rollout's rigid-body step on cases with known
answers (no GPU)."""
import numpy as np

from oracle import rigid
from stonefish_gb300 import abi


def _state(n=1):
    s = np.zeros(n, dtype=abi.RIGID_DTYPE)
    s["q"][:, 0] = 1.0
    s["mass"] = 2.0
    s["inertial_mass"] = 2.0
    s["inertia"] = (1.0, 2.0, 3.0)
    s["half_extents"] = (1.0, 0.5, 0.25)
    return s


def test_free_fall_is_semi_implicit_euler():
    s = _state()
    dt, g = 0.01, 9.81
    for k in range(1, 101):
        s = rigid.step(s, np.zeros((1, 3)), np.zeros((1, 3)), dt, g)
    # v_k = k g dt, p_k = g dt^2 k (k+1) / 2
    assert np.isclose(s["v"][0, 2], 100 * g * dt)
    assert np.isclose(s["p"][0, 2], g * dt * dt * 100 * 101 / 2)
    assert np.allclose(s["q"][0], [1, 0, 0, 0])


def test_spin_about_principal_axis_keeps_rate_and_unit_quaternion():
    s = _state()
    s["w"][0] = (0.0, 0.0, 1.5)
    for _ in range(200):
        s = rigid.step(s, np.zeros((1, 3)), np.zeros((1, 3)), 0.01, 0.0)
    assert np.allclose(s["w"][0], (0.0, 0.0, 1.5))
    assert np.isclose(np.linalg.norm(s["q"][0]), 1.0)
    # exponential map: exactly 3 rad about z after 2 s at 1.5 rad/s
    ang = 2 * np.arctan2(s["q"][0, 3], s["q"][0, 0])
    assert abs(ang - 3.0) < 1e-9


def test_implicit_gyroscopic_step_is_stable_and_keeps_momentum_bounded():
    """Torque-free spin about the intermediate axis with a small wobble: the
    implicit gyroscopic term keeps |L| from growing (explicit Euler gains
    energy at this step size)."""
    s = _state()
    s["inertia"] = (1.0, 2.0, 3.0)
    s["w"][0] = (0.01, 6.0, 0.01)
    L0 = np.linalg.norm(s["inertia"][0] * s["w"][0])
    for _ in range(500):
        s = rigid.step(s, np.zeros((1, 3)), np.zeros((1, 3)), 0.02, 0.0)
        R = rigid.quat_to_rot(s["q"])[0]
        L = np.linalg.norm(s["inertia"][0] * (R.T @ s["w"][0]))
        assert L <= L0 * (1 + 1e-9)


def test_gyro_newton_solves_the_linearised_implicit_equation():
    rng = np.random.default_rng(3)
    wb = rng.normal(size=(5, 3))
    I = rng.uniform(0.5, 3.0, (5, 3))
    dt = 0.05
    dw = rigid.gyro_newton(wb, I, dt)
    # residual of I dw + dt (w x Iw) + dt (dw x Iw + w x I dw) (first order) vanishes
    Iw = I * wb
    r = I * dw + dt * np.cross(wb, Iw) + dt * (np.cross(dw, Iw) + np.cross(wb, I * dw))
    assert np.allclose(r, 0.0, atol=1e-12)


def test_body_torque_gives_body_angular_acceleration():
    s = _state()
    R = rigid.quat_to_rot(np.array([[np.cos(0.3), 0.0, np.sin(0.3), 0.0]]))[0]
    s["q"][0] = (np.cos(0.3), 0.0, np.sin(0.3), 0.0)
    t = np.array([[0.0, 0.0, 3.0]])
    s2 = rigid.step(s, np.zeros((1, 3)), t, 0.1, 0.0)
    wb = R.T @ s2["w"][0]
    assert np.allclose(wb, (0.0, 0.0, 0.1 * 3.0 / 3.0))


def test_inertial_mass_divides_force_and_mass_weighs():
    s = _state()
    s["inertial_mass"] = 8.0
    s2 = rigid.step(s, np.array([[4.0, 0.0, 0.0]]), np.zeros((1, 3)), 0.1, 10.0)
    assert np.allclose(s2["v"][0], (0.05, 0.0, 0.1 * 2.0 * 10.0 / 8.0))


def test_body_pose_aabb():
    s = _state()
    s["q"][0] = (np.cos(np.pi / 4), 0.0, 0.0, np.sin(np.pi / 4))   # 90 deg about z
    s["p"][0] = (1.0, 2.0, 3.0)
    R, o, lo, hi = rigid.body_pose(s)
    assert np.allclose(hi[0] - o[0], (0.5, 1.0, 0.25))
    assert np.allclose(o[0] - lo[0], (0.5, 1.0, 0.25))
