"""Known-answer tests of the oracle's aerodynamic path (no GPU):
SolidEntity::ComputeAerodynamicForces / CorrectAerodynamicForces
(Library/src/entities/SolidEntity.cpp:1852-1956)."""
import numpy as np
import pytest

from oracle import MIRROR32, REF32, REF64
from stonefish_gb300 import abi, meshes
from tests.helpers import body_transform

RHO_AIR = 1.225


def atmosphere(*winds):
    a = abi.Atmosphere()
    a.density = RHO_AIR
    a.n_winds = len(winds)
    for i, w in enumerate(winds):
        a.winds[i].type = abi.CURRENT_UNIFORM
        a.winds[i].enabled = 0          # ignored: the atmosphere sums every field
        for k in range(3):
            a.winds[i].vel[k] = w[k]
    return a


def identity_transforms(origin=(0.0, 0.0, 0.0)):
    b = np.zeros(1, dtype=abi.BODY_DTYPE)
    b["T_CG"]["basis"][0] = np.eye(3).ravel()
    b["T_CG"]["origin"][0] = origin
    b["T_C"] = b["T_CG"]
    return body_transform(b, "T_CG"), body_transform(b, "T_C")


@pytest.mark.parametrize("variant", (REF32, REF64, MIRROR32))
@pytest.mark.parametrize("u", (0.5, 3.0))
def test_box_moving_in_still_air(oracle, variant, u):
    """Only the face moving into the air contributes: Fda = 1/2 rho * (vn * 3 * A)
    = -1.5 rho a^2 u x  (glm's vec3::length() is 3, so the law is linear in
    u), no torque by symmetry."""
    a = 0.8
    mesh = meshes.build_box((a / 2, a / 2, a / 2), 2)
    tcg, tc = identity_transforms()
    F, T = oracle.aero_forces(variant, mesh, atmosphere(), tcg, tc, (u, 0, 0), (0, 0, 0))
    tol = 1e-5 if variant != REF64 else 1e-12
    side = 2.0 * float(np.float32(a / 2))      # the mesh's vertices are FP32
    assert F[0] == pytest.approx(-1.5 * RHO_AIR * side * side * u, rel=tol)
    assert abs(F[1]) < tol * abs(F[0]) and abs(F[2]) < tol * abs(F[0])
    assert np.all(np.abs(T) < tol * abs(F[0]) * a)


def test_wind_equal_to_body_velocity_gives_no_force(oracle):
    mesh = meshes.build_icosphere(0.5, 2)
    tcg, tc = identity_transforms((1.0, -2.0, 0.5))
    F, T = oracle.aero_forces(REF64, mesh, atmosphere((1.0, 2.0, -0.5)), tcg, tc, (1.0, 2.0, -0.5), (0, 0, 0))
    assert np.all(F == 0.0) and np.all(T == 0.0)


def test_wind_fields_are_summed_and_frame_independent(oracle):
    """Two winds act as their sum; translating the body and its CG together
    leaves the wrench unchanged."""
    mesh = meshes.build_icosphere(0.4, 2)
    tcg, tc = identity_transforms()
    F1, T1 = oracle.aero_forces(REF64, mesh, atmosphere((2.0, 0, 0), (0, -1.0, 0.5)), tcg, tc, (0.1, 0, 0), (0, 0, 0.3))
    F2, T2 = oracle.aero_forces(REF64, mesh, atmosphere((2.0, -1.0, 0.5)), tcg, tc, (0.1, 0, 0), (0, 0, 0.3))
    assert np.allclose(F1, F2, rtol=1e-12, atol=1e-12) and np.allclose(T1, T2, rtol=1e-12, atol=1e-12)
    tcg3, tc3 = identity_transforms((5.0, 6.0, -7.0))
    F3, T3 = oracle.aero_forces(REF64, mesh, atmosphere((2.0, -1.0, 0.5)), tcg3, tc3, (0.1, 0, 0), (0, 0, 0.3))
    assert np.allclose(F3, F2, rtol=1e-9) and np.allclose(T3, T2, rtol=1e-9, atol=1e-12)


def test_null_mesh_gives_zeros(oracle):
    tcg, tc = identity_transforms()
    F, T = oracle.aero_forces(REF32, None, atmosphere((3, 0, 0)), tcg, tc, (0, 0, 0), (0, 0, 0))
    assert np.all(F == 0) and np.all(T == 0)


def _params(kind, R=np.eye(3), axes=(1.0, 1.0, 1.0)):
    p = abi.AeroParams()
    p.approx_type = kind
    for i in range(9):
        p.R_CG2H[i] = float(np.asarray(R).ravel()[i])
    for i in range(3):
        p.approx_params[i] = axes[i]
    return p


@pytest.mark.parametrize("kind,direction,factor", [
    (abi.APPROX_AUTO, (1, 2, 3), 1.0),
    (abi.APPROX_SPHERE, (0, 0, -4), 1.0),
    (abi.APPROX_CYLINDER, (0, 0, 2), 1.0),
    (abi.APPROX_CYLINDER, (-3, 0, 0), 0.5),
    (abi.APPROX_ELLIPSOID, (0, 5, 0), 0.5),
    (abi.APPROX_ELLIPSOID, (1, 0, 0), 1.0),
])
def test_correction_factor(oracle, kind, direction, factor):
    p = _params(kind, axes=(1.0, 2.0, 4.0))
    F0 = np.array(direction, float)
    T0 = np.array([0.3, -0.2, 0.1])
    F, T = oracle.aero_correct(p, F0, T0)
    assert np.allclose(F, factor * F0, rtol=1e-15) and np.allclose(T, factor * T0, rtol=1e-15)


def test_correction_uses_proxy_frame_and_safe_normalize(oracle):
    # proxy frame rotated 90 deg about y: the body x axis is the proxy z axis
    R = np.array([[0.0, 0.0, 1.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0]])
    F, _ = oracle.aero_correct(_params(abi.APPROX_CYLINDER, R), np.array([2.0, 0.0, 0.0]), np.zeros(3))
    # R^-1 (2,0,0) = (0,0,2) -> factor 1; a zero force normalises to (1,0,0) -> factor 0.5 on zeros
    assert np.allclose(F, (2.0, 0.0, 0.0))
    F, T = oracle.aero_correct(_params(abi.APPROX_CYLINDER), np.zeros(3), np.array([1.0, 1.0, 1.0]))
    assert np.all(F == 0.0) and np.allclose(T, 0.5)
