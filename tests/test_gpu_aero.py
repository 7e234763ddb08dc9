"""GPU parity of the aerodynamic path (SolidEntity::ComputeAerodynamicForces /
CorrectAerodynamicForces, SolidEntity.cpp:1852-1956) against the oracle:
per-body wrenches within 2e-6 of the force scale of MIRROR32 (FP32 face
terms, exact sums), the correction bit for bit."""
import math

import numpy as np
import pytest

from oracle import MIRROR32, REF64
from stonefish_gb300 import abi, meshes, scenarios
from tests.helpers import body_transform

pytestmark = pytest.mark.gpu
TOL = 2e-6


def atmosphere(rng, jet=True):
    a = abi.Atmosphere()
    a.density = 1.225
    a.n_winds = 2 if jet else 1
    a.winds[0].type = abi.CURRENT_UNIFORM
    for k, x in enumerate(rng.uniform(-3, 3, 3)):
        a.winds[0].vel[k] = x
    if jet:
        c = a.winds[1]
        c.type = abi.CURRENT_JET
        for k in range(3):
            c.point[k] = (0.2, -0.1, 0.0)[k]
            c.dir[k] = (0.0, 0.6, 0.8)[k]
        c.radius = 0.7
        c.speed = 4.0
    return a


def random_params(rng, n):
    p = np.zeros(n, dtype=abi.AERO_PARAMS_DTYPE)
    p["approx_type"] = rng.integers(0, 4, n)
    q = scenarios.random_quaternions(rng, n)
    p["R_CG2H"] = scenarios.quat_to_matrix(q).reshape(n, 9)
    p["approx_params"] = rng.uniform(0.2, 1.5, (n, 3))
    return p


def params_struct(row):
    s = abi.AeroParams()
    s.approx_type = int(row["approx_type"])
    for i in range(9):
        s.R_CG2H[i] = float(row["R_CG2H"][i])
    for i in range(3):
        s.approx_params[i] = float(row["approx_params"][i])
    return s


def scaled(F, T, Fr, Tr, L):
    S = max(np.linalg.norm(Fr), 1e-300)
    return np.linalg.norm(F - Fr) / S, np.linalg.norm(T - Tr) / (S * L)


def test_static_aero_matches_oracle(oracle, hctx):
    rng = np.random.default_rng(41)
    meshes_ = [meshes.build_icosphere(0.5, 3), meshes.build_box((0.4, 0.3, 0.2), 3),
               meshes.capped_cylinder_for_faces(0.2, 1.6, 3000)]
    ids = [hctx.upload_mesh(*m) for m in meshes_]
    for trial in range(24):
        k = trial % 3
        atm = atmosphere(rng, jet=bool(trial % 2))
        R = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))
        b = scenarios.fill_bodies(1, R, rng.uniform(-1, 1, (1, 3)), rng.uniform(-2, 2, (1, 3)),
                                  rng.uniform(-1, 1, (1, 3)), np.ones((1, 3)), 1.0, 1.0, (1, 1, 1), (0.1, 0.1, 0.1), 0)
        tcg, tc = body_transform(b, "T_CG"), body_transform(b, "T_C")
        v, w = b["v"][0], b["omega"][0]
        Fg, Tg = hctx.aero_forces(ids[k], atm, tcg, tc, v, w)
        Fm, Tm = oracle.aero_forces(MIRROR32, meshes_[k], atm, tcg, tc, v, w)
        F6, T6 = oracle.aero_forces(REF64, meshes_[k], atm, tcg, tc, v, w)
        eF, eT = scaled(Fg, Tg, Fm, Tm, 1.0)
        assert eF < TOL and eT < TOL, (trial, eF, eT)
        eF, eT = scaled(Fg, Tg, F6, T6, 1.0)
        assert eF < 1e-4 and eT < 1e-4, (trial, eF, eT)
    # null mesh
    tcg, tc = body_transform(b, "T_CG"), body_transform(b, "T_C")
    Fg, Tg = hctx.aero_forces(abi.NO_MESH, atm, tcg, tc, (1, 2, 3), (0, 0, 0))
    assert np.all(Fg == 0) and np.all(Tg == 0)


def test_aero_correction_bit_identical(oracle, hctx):
    rng = np.random.default_rng(42)
    p = random_params(rng, 40)
    for i in range(40):
        F0 = rng.normal(size=3) * 10 ** rng.uniform(-3, 3)
        if i == 0:
            F0[:] = 0.0                      # safeNormalize's fallback
        T0 = rng.normal(size=3)
        s = params_struct(p[i])
        Fg, Tg = hctx.aero_correct(s, F0, T0)
        Fo, To = oracle.aero_correct(s, F0, T0)
        assert np.array_equal(Fg, Fo) and np.array_equal(Tg, To), i


def test_aero_batch_matches_oracle_and_gates_modes(oracle, hctx):
    rng = np.random.default_rng(43)
    sc = scenarios.mixed_batch(n_bodies=72, seed=44, scale_faces=0.05)
    ids = np.asarray([hctx.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids[sc["bodies"]["mesh"]]
    n = len(bodies)
    bodies["mode"] = np.where(np.arange(n) % 4 == 3, abi.MODE_SUBMERGED, abi.MODE_AERODYNAMIC)
    bodies["v"] = rng.uniform(-3, 3, (n, 3))
    params = random_params(rng, n)
    atm = atmosphere(rng)
    out = np.zeros(n, dtype=abi.AERO_WRENCH_DTYPE)
    out["Fda"] = 7.0                                   # sentinel for gated bodies
    batch = hctx.batch(bodies["mesh"])
    batch.compute_aero(bodies, params, atm, out)
    L = 0.5 * np.linalg.norm(np.maximum(bodies["aabb_max"] - bodies["aabb_min"], 0), axis=1)
    for i in range(n):
        if bodies["mode"][i] != abi.MODE_AERODYNAMIC:
            assert np.all(out["Fda"][i] == 7.0)
            continue
        mesh = sc["meshes"][sc["bodies"]["mesh"][i]]
        tcg = abi.Transform()
        tc = abi.Transform()
        for k in range(9):
            tcg.basis[k] = bodies["T_CG"]["basis"][i][k]
            tc.basis[k] = bodies["T_C"]["basis"][i][k]
        for k in range(3):
            tcg.origin[k] = bodies["T_CG"]["origin"][i][k]
            tc.origin[k] = bodies["T_C"]["origin"][i][k]
        Fm, Tm = oracle.aero_forces(MIRROR32, mesh, atm, tcg, tc, bodies["v"][i], bodies["omega"][i])
        Fm, Tm = oracle.aero_correct(params_struct(params[i]), Fm, Tm)
        eF, eT = scaled(out["Fda"][i], out["Tda"][i], Fm, Tm, max(L[i], 1e-3))
        assert eF < TOL and eT < TOL, (i, eF, eT)
        assert out["status"][i] == 0
    batch.close()
