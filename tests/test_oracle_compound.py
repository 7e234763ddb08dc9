"""The oracle's Compound::ComputeHydrodynamicForces (Compound.cpp:291-436)
against the single-body path it is built from (no GPU)."""
import numpy as np
import pytest

from oracle import MIRROR32, REF64
from stonefish_gb300 import abi, meshes, scenarios


def one_part_compound(body):
    p = np.zeros(1, dtype=abi.COMPOUND_PART_DTYPE)
    p["T_C"] = body["T_C"]
    p["R_O"] = body["R_O"]
    p["Cd"] = body["Cd"]
    p["Cf"] = body["Cf"]
    p["mesh"] = 0
    p["mode"] = abi.MODE_SUBMERGED
    p["buoyant"] = 1
    p["external"] = 1
    return p


@pytest.mark.parametrize("depth", [-0.2, 0.1, 2.0, -3.0])
@pytest.mark.parametrize("variant", [REF64, MIRROR32])
def test_single_external_part_equals_the_body(oracle, depth, variant):
    sc = scenarios.single_sphere(steps=1, seed=3)
    body = sc["bodies"].copy()
    body["T_CG"]["origin"][0, 2] = depth
    body["T_C"]["origin"][0, 2] = depth
    body["aabb_min"][0, 2] = depth - 0.5
    body["aabb_max"][0, 2] = depth + 0.5
    mesh = sc["meshes"][0]
    st = scenarios.settings()
    ref = scenarios.new_wrenches(1)
    oracle.body_forces(variant, body, mesh, sc["ocean"], st, ref)
    got = scenarios.new_wrenches(1)
    oracle.compound_forces(variant, body, one_part_compound(body), [mesh], sc["ocean"], st, got)
    assert got["position"][0] == ref["position"][0]
    for k in abi.WRENCH_VECTORS + ("Swet",):
        assert np.allclose(got[k], ref[k], rtol=1e-12, atol=1e-12), k
    if ref["position"][0] == abi.INSIDE:
        assert got["Vsub"][0] == body["volume"][0]      # the compound sets Vsub; a body keeps it
    else:
        assert np.allclose(got["Vsub"], ref["Vsub"], rtol=1e-12, atol=1e-15)


def test_internal_parts_add_buoyancy_only_and_disabled_parts_nothing(oracle):
    sc = scenarios.compound_batch(n_compounds=12, seed=9, depth=(-0.1, 0.1))
    ms = sc["meshes"]
    st = scenarios.settings()
    ppc = sc["parts_per_compound"]
    first = np.concatenate([[0], np.cumsum(ppc)[:-1]]).astype(int)
    checked = 0
    for c in range(len(ppc)):
        comp = sc["compounds"][c:c + 1]
        parts = sc["parts"][first[c]:first[c] + int(ppc[c])]
        pm = [ms[i] for i in parts["mesh"]]
        full = scenarios.new_wrenches(1)
        oracle.compound_forces(REF64, comp, parts, pm, sc["ocean"], st, full)
        if full["position"][0] != abi.CROSSING_SURFACE:
            continue
        # without the internal ballast part: damping identical, buoyancy differs by its share
        keep = parts["external"] == 1
        part2 = parts[keep]
        less = scenarios.new_wrenches(1)
        oracle.compound_forces(REF64, comp, part2, [ms[i] for i in part2["mesh"]], sc["ocean"], st, less)
        for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
            assert np.allclose(full[k], less[k], rtol=1e-12, atol=1e-12)
        assert full["Swet"][0] == pytest.approx(less["Swet"][0], rel=1e-12)
        # the disabled part changes nothing
        act = parts["mode"] != abi.MODE_DISABLED
        part3 = parts[act]
        same = scenarios.new_wrenches(1)
        oracle.compound_forces(REF64, comp, part3, [ms[i] for i in part3["mesh"]], sc["ocean"], st, same)
        assert same.tobytes() == full.tobytes()
        checked += 1
    assert checked >= 3


def test_mode_gate_and_outside(oracle):
    sc = scenarios.compound_batch(n_compounds=2, seed=10, depth=(-5.0, -4.0))
    st = scenarios.settings()
    ms = sc["meshes"]
    parts = sc["parts"][: int(sc["parts_per_compound"][0])]
    io = scenarios.new_wrenches(1)
    io["Fb"] = 3.0
    oracle.compound_forces(REF64, sc["compounds"][:1], parts, [ms[i] for i in parts["mesh"]], sc["ocean"], st, io)
    assert io["position"][0] == abi.OUTSIDE and np.all(io["Fb"] == 0.0)
    comp = sc["compounds"][:1].copy()
    comp["mode"] = abi.MODE_DISABLED
    io["Fb"] = 3.0
    oracle.compound_forces(REF64, comp, parts, [ms[i] for i in parts["mesh"]], sc["ocean"], st, io)
    assert io["position"][0] == abi.SKIPPED and np.all(io["Fb"] == 3.0)
