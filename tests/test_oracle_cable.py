"""Known-answer tests of the oracle's CableEntity::ComputeHydrodynamicForces
(Library/src/entities/CableEntity.cpp:240-376), no GPU."""
import math

import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios

RHO, G = 1025.0, 9.81


def run(oracle, xs, r=0.05, v=None, mode=abi.MODE_SUBMERGED, buoyancy=1, settings=None, ocean=None):
    x = np.asarray(xs, float)
    n = len(x)
    cables = np.zeros(1, dtype=abi.CABLE_DTYPE)
    cables["n_nodes"] = n
    cables["radius"] = r
    cables["mode"] = mode
    cables["buoyancy"] = buoyancy
    out = np.zeros(n, dtype=abi.CABLE_FORCES_DTYPE)
    oracle.cable_forces(cables, x, np.zeros_like(x) if v is None else v,
                        ocean or scenarios.flat_ocean(current=None), settings or scenarios.settings(), out)
    return out


def test_two_node_submerged_cable_each_node_carries_the_full_buoyancy(oracle):
    """One segment gives half to each node, and the end nodes are doubled:
    with two nodes each node carries the segment's whole buoyancy."""
    r, L = 0.05, 2.0
    out = run(oracle, [(0, 0, 1.0), (L, 0, 1.0)], r=r)
    V = math.pi * r * r * L
    for i in range(2):
        assert out["Fb"][i][2] == pytest.approx(-V * RHO * G, rel=1e-14)
        assert out["Fb"][i][0] == 0.0 and out["Fb"][i][1] == 0.0


def test_horizontal_cable_half_submerged(oracle):
    r, L = 0.04, 1.5
    out = run(oracle, [(0, 0, 0.0), (L / 2, 0, 0.0), (L, 0, 0.0)], r=r)
    V_seg = math.pi * r * r * (L / 2) / 2           # circular segment of height r: half the disc
    total = out["Fb"][:, 2].sum()
    # middle node: two halves; end nodes: doubled halves
    assert out["Fb"][1][2] == pytest.approx(-V_seg * RHO * G, rel=1e-12)
    assert total == pytest.approx(-3 * V_seg * RHO * G, rel=1e-12)


def test_vertical_cable_submerged_length(oracle):
    r = 0.03
    out = run(oracle, [(0, 0, -0.5), (0, 0, 0.7)], r=r)
    V = math.pi * r * r * 0.7                        # min(d2, dz) of the submerged part
    assert out["Fb"][0][2] == pytest.approx(-V * RHO * G, rel=1e-6)


def test_dry_cable_and_mode_gate(oracle):
    out = run(oracle, [(0, 0, -2.0), (1, 0, -2.5)])
    assert np.all(out["Fb"] == 0) and np.all(out["Fdq"] == 0) and np.all(out["Fdf"] == 0)
    cables = np.zeros(1, dtype=abi.CABLE_DTYPE)
    cables["n_nodes"] = 2
    cables["radius"] = 0.05
    cables["mode"] = abi.MODE_DISABLED
    out = np.zeros(2, dtype=abi.CABLE_FORCES_DTYPE)
    out["Fb"] = 4.0
    oracle.cable_forces(cables, np.array([(0, 0, 1.0), (1, 0, 1.0)]), np.zeros((2, 3)), scenarios.flat_ocean(),
                        scenarios.settings(), out)
    assert np.all(out["Fb"] == 4.0)


def test_drag_opposes_relative_motion_and_skin_friction_is_linear(oracle):
    r, L = 0.05, 1.0
    x = [(0, 0, 1.0), (L, 0, 1.0)]
    v = np.array([(0, 0.3, 0.0), (0, 0.3, 0.0)])
    out = run(oracle, x, r=r, v=v)
    assert out["Fdq"][0][1] < 0 and out["Fdf"][0][1] < 0
    out2 = run(oracle, x, r=r, v=2 * v)
    # skin friction -S relV is linear in the velocity (per node: doubled end halves)
    assert out2["Fdf"][0][1] == pytest.approx(2 * out["Fdf"][0][1], rel=1e-14)
    S = 2 * math.pi * r * L
    assert out["Fdf"][0][1] == pytest.approx(-S * 0.3, rel=1e-14)


def test_random_cables_are_finite_and_buoyancy_points_up(oracle):
    sc = scenarios.cable_set(n_cables=30, seed=3)
    out = np.zeros(len(sc["x"]), dtype=abi.CABLE_FORCES_DTYPE)
    oracle.cable_forces(sc["cables"], sc["x"], sc["v"], sc["ocean"], scenarios.settings(), out)
    assert np.all(np.isfinite(out["Fb"])) and np.all(np.isfinite(out["Fdq"]))
    assert np.all(out["Fb"][:, 2] <= 0.0)
