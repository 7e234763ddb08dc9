"""Known-answer tests of the CPU oracle (no GPU).

The reference's own tests pin nothing on this path, so the oracle is pinned
here by analytic results of the method it restates
(Library/src/entities/SolidEntity.cpp:1239-1850) and by agreement between its
FP32 (reference arithmetic) and FP64 variants."""
import math

import numpy as np
import pytest

from oracle import MIRROR32, MIRROR64, REF32, REF64
from stonefish_gb300 import abi, meshes, scenarios
from tests.helpers import body_transform, io_dict, scaled_errors

RHO, G = 1025.0, 9.81
ALL = (REF32, REF64, MIRROR64, MIRROR32)


def sphere_body(depth, R=np.eye(3), r=0.5, v=(0, 0, 0), w=(0, 0, 0), buoyancy=1, mode=abi.MODE_SUBMERGED):
    half = np.array([[r, r, r]])
    return scenarios.fill_bodies(1, np.asarray(R)[None], np.array([[0.0, 0.0, depth]]),
                                 np.array([v], float), np.array([w], float), half,
                                 4 / 3 * math.pi * r ** 3, 4 * math.pi * r * r, (1, 1, 1),
                                 (0.1, 0.1, 0.1), 0, mode=mode, buoyancy=buoyancy)


@pytest.fixture(scope="module")
def sphere():
    return meshes.build_icosphere(0.5, 3)


def still_ocean():
    return scenarios.flat_ocean(current=None)


@pytest.mark.parametrize("variant", ALL)
def test_inside_buoyancy_is_rho_g_V(oracle, sphere, variant):
    b = sphere_body(2.0)
    io = scenarios.new_wrenches(1)
    io["Vsub"] = 123.0
    oracle.body_forces(variant, b, sphere, still_ocean(), scenarios.settings(), io)
    assert io["position"][0] == abi.INSIDE
    V = 4 / 3 * math.pi * 0.125
    assert io["Fb"][0][2] == -V * RHO * G          # SolidEntity.cpp:1833 exactly
    assert np.all(io["Tb"][0] == 0.0)
    assert io["Vsub"][0] == 123.0                   # INSIDE keeps Vsub
    assert io["Swet"][0] == 4 * math.pi * 0.25      # Swet = surface
    assert np.all(io["Fdq"][0] == 0) and np.all(io["Fdf"][0] == 0)   # no flow


@pytest.mark.parametrize("variant", ALL)
def test_all_faces_submerged_volume_is_mesh_volume(oracle, sphere, variant):
    io = io_dict()
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    T.origin[2] = 3.0
    oracle.surface_forces(variant, scenarios.settings(), sphere, still_ocean(), T, T,
                          np.zeros(3), np.zeros(3), io)
    V = meshes.mesh_volume(*sphere)
    tol = 5e-5 if variant == REF32 else 2e-6      # REF32 sums 1280 terms serially in FP32
    assert io["Vsub"][0] == pytest.approx(V, rel=tol)
    assert io["Fb"][2] == pytest.approx(-V * RHO * G, rel=tol)
    assert io["Swet"][0] == pytest.approx(meshes.mesh_area(*sphere), rel=tol)


@pytest.mark.parametrize("variant", ALL)
def test_half_sphere_volume_and_centre_of_buoyancy(oracle, sphere, variant):
    # the icosphere is symmetric under z -> -z, so half its volume is below z=0
    io = io_dict()
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    oracle.surface_forces(variant, scenarios.settings(), sphere, still_ocean(), T, T,
                          np.zeros(3), np.zeros(3), io)
    V = meshes.mesh_volume(*sphere)
    assert io["Vsub"][0] == pytest.approx(V / 2, rel=5e-5 if variant == REF32 else 2e-6)
    # torque of buoyancy about the CG: CB at depth ~3r/8 straight below -> no torque
    assert np.linalg.norm(io["Tb"]) < 1e-6 * np.linalg.norm(io["Fb"])


@pytest.mark.parametrize("variant", ALL)
@pytest.mark.parametrize("draft", [0.05, 0.2, 0.37])
def test_box_draft_volume_exact(oracle, variant, draft):
    a, b_, c = 0.4, 0.3, 0.25
    xyz, faces = meshes.build_box((a, b_, c), 2)
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    T.origin[2] = draft - c          # bottom at z = draft (NED, z down)
    io = io_dict()
    oracle.surface_forces(variant, scenarios.settings(), (xyz, faces), still_ocean(), T, T,
                          np.zeros(3), np.zeros(3), io)
    tol = 2e-5 if variant == REF32 else 2e-6
    assert io["Vsub"][0] == pytest.approx(4 * a * b_ * draft, rel=tol)
    # wetted area: bottom + four side strips
    assert io["Swet"][0] == pytest.approx(4 * a * b_ + 2 * (2 * a + 2 * b_) * draft, rel=tol)


@pytest.mark.parametrize("variant", ALL)
def test_zero_relative_velocity_gives_zero_damping(oracle, sphere, variant):
    b = sphere_body(0.1)
    io = scenarios.new_wrenches(1)
    oracle.body_forces(variant, b, sphere, still_ocean(), scenarios.settings(), io)
    assert io["position"][0] == abi.CROSSING_SURFACE
    for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
        assert np.all(io[k][0] == 0.0)
    assert io["Vsub"][0] > 0


def test_current_equals_opposite_body_velocity(oracle, sphere):
    """Only the relative velocity matters: a still body in a current u and a body
    moving at -u in still water give the same damping."""
    u = (0.3, -0.2, 0.1)
    oc = scenarios.flat_ocean(current=u)
    b1 = sphere_body(0.1)
    b2 = sphere_body(0.1, v=tuple(-x for x in u))
    io1, io2 = scenarios.new_wrenches(1), scenarios.new_wrenches(1)
    oracle.body_forces(REF64, b1, sphere, oc, scenarios.settings(), io1)
    oracle.body_forces(REF64, b2, sphere, still_ocean(), scenarios.settings(), io2)
    for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
        np.testing.assert_allclose(io1[k], io2[k], rtol=1e-12, atol=1e-12)


def test_outside_zeroes_everything(oracle, sphere):
    b = sphere_body(-3.0, v=(1, 0, 0))
    io = scenarios.new_wrenches(1)
    for k in abi.WRENCH_VECTORS:
        io[k] = 5.0
    io["Swet"] = io["Vsub"] = 5.0
    oracle.body_forces(REF32, b, sphere, still_ocean(), scenarios.settings(), io)
    assert io["position"][0] == abi.OUTSIDE
    for k in abi.WRENCH_VECTORS:
        assert np.all(io[k] == 0.0)
    assert io["Swet"][0] == 0.0 and io["Vsub"][0] == 0.0


@pytest.mark.parametrize("mode", [abi.MODE_DISABLED, abi.MODE_SURFACE, abi.MODE_AERODYNAMIC])
def test_mode_gate_leaves_outputs_untouched(oracle, sphere, mode):
    b = sphere_body(0.0, mode=mode)
    io = scenarios.new_wrenches(1)
    io["Fb"] = 7.0
    oracle.body_forces(REF32, b, sphere, still_ocean(), scenarios.settings(), io)
    assert io["position"][0] == abi.SKIPPED
    assert np.all(io["Fb"][0] == 7.0)


@pytest.mark.parametrize("variant", ALL)
def test_tiny_submerged_volume_keeps_stale_buoyancy(oracle, sphere, variant):
    # the lowest vertex 1e-5 m under water: Vsub6 below 1e-9
    zmax = float(sphere[0][:, 2].max())
    b = sphere_body(-(zmax - 1e-5), r=zmax)   # AABB just reaching below the surface
    io = scenarios.new_wrenches(1)
    io["Fb"] = (1.0, 2.0, 3.0)
    io["Tb"] = (4.0, 5.0, 6.0)
    io["Vsub"] = 9.0
    oracle.body_forces(variant, b, sphere, still_ocean(), scenarios.settings(), io)
    assert io["position"][0] == abi.CROSSING_SURFACE
    assert tuple(io["Fb"][0]) == (1.0, 2.0, 3.0)
    assert tuple(io["Tb"][0]) == (4.0, 5.0, 6.0)
    assert io["Vsub"][0] == 9.0


def test_non_buoyant_body_keeps_buoyancy_outputs(oracle, sphere):
    b = sphere_body(0.0, buoyancy=0)
    io = scenarios.new_wrenches(1)
    io["Fb"] = 3.0
    oracle.body_forces(REF32, b, sphere, still_ocean(), scenarios.settings(), io)
    assert np.all(io["Fb"][0] == 3.0)
    assert io["Swet"][0] > 0


def test_null_mesh_rules(oracle):
    b = sphere_body(0.0)
    io = scenarios.new_wrenches(1)
    io["Fb"] = 2.0
    io["Fdq"] = 2.0
    io["Swet"] = io["Vsub"] = 2.0
    oracle.body_forces(REF32, b, None, still_ocean(), scenarios.settings(), io)
    assert np.all(io["Fb"][0] == 0) and np.all(io["Fdq"][0] == 0)
    assert io["Swet"][0] == 0 and io["Vsub"][0] == 0
    # with buoyancy off only the damping and Swet/Vsub are reset (:1293-1312)
    io["Fb"] = 2.0
    oracle.body_forces(REF32, b, None, still_ocean(), scenarios.settings(buoyancy=False), io)
    assert np.all(io["Fb"][0] == 2.0)


def test_degenerate_face_counts_volume_not_area(oracle):
    # one regular face and one 1e-7 m sliver far from the fan apex
    xyz = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1],
                    [0.5, 0.5, 2], [0.5 + 1e-6, 0.5, 2], [0.5, 0.5 + 1e-6, 2.5]], dtype=np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5]], dtype=np.uint32)
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    t = oracle.face_terms(MIRROR64, scenarios.settings(), (xyz, faces), still_ocean(), T, T,
                          np.zeros(3), np.zeros(3))
    assert t[1, 19] != 0.0            # V6 of the sliver's tetra is accumulated
    assert t[1, 18] == 0.0            # no wetted area
    assert t[0, 18] == pytest.approx(0.5)


def test_thresholds_tangent_flow_gives_only_skin_friction(oracle):
    # a horizontal face (normal along z) in a purely horizontal flow
    xyz = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1]], dtype=np.float32)
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    t = oracle.face_terms(REF32, scenarios.settings(), (xyz, faces), scenarios.flat_ocean((0.5, 0, 0)),
                          T, T, np.zeros(3), np.zeros(3))
    assert np.all(t[0, 6:12] == 0.0)            # vc_n = 0: no quadratic drag
    assert t[0, 12] == pytest.approx(0.5 * 0.5)  # skin = vt * A


def test_correction_factor(oracle):
    io = io_dict()
    io["Fdq"][:] = (2.0, 0.0, 0.0)
    io["Fdf"][:] = (0.0, 0.0, -4.0)
    oracle.correct_forces(still_ocean(), io, (0.7, 0.5, 0.3), (0.07, 0.05, 0.03), np.eye(3))
    assert io["Fdq"][0] == pytest.approx(0.5 * RHO * 0.7 * 2.0, rel=1e-15)
    assert io["Fdf"][2] == pytest.approx(RHO * 0.03 * -4.0, rel=1e-15)
    # zero vectors normalise to (1,0,0) and stay zero
    assert np.all(io["Tdq"] == 0.0)


def test_fluid_position_flat(oracle):
    oc = still_ocean()
    assert oracle.fluid_position(oc, (-1, -1, -2), (1, 1, -0.5)) == abi.OUTSIDE
    assert oracle.fluid_position(oc, (-1, -1, 0.5), (1, 1, 2)) == abi.INSIDE
    assert oracle.fluid_position(oc, (-1, -1, -1), (1, 1, 1)) == abi.CROSSING_SURFACE
    # depth must be strictly positive (> 0) to count as under water
    assert oracle.fluid_position(oc, (-1, -1, 0.0), (1, 1, 1)) == abi.CROSSING_SURFACE


def test_wave_lookup_reproduces_texels_and_wraps(oracle):
    n, L = 16, 8.0
    rng = np.random.default_rng(3)
    data = rng.normal(size=(n, n)).astype(np.float32)
    waves = {"data": data, "layers": [(0, L)]}
    oc = still_ocean()
    oc.waves = 1
    d = L / n
    for i, j in [(0, 0), (3, 7), (15, 15), (8, 2)]:
        x, y = (i + 0.5) * d, (j + 0.5) * d
        # depth = z - waveHeight, waveHeight = -texel
        assert oracle.depth(oc, waves, x, y, 0.0) == pytest.approx(float(data[j, i]), abs=1e-5)
        assert oracle.depth(oc, waves, x + 3 * L, y - 2 * L, 0.0) == pytest.approx(float(data[j, i]), abs=1e-4)
    # halfway between two texel centres along x: the mean
    x, y = 2.0 * d, 0.5 * d
    assert oracle.depth(oc, waves, x, y, 0.0) == pytest.approx(0.5 * (data[0, 1] + data[0, 2]), abs=1e-5)


def test_fp32_reference_close_to_fp64_on_single_sphere(oracle):
    sc = scenarios.single_sphere(steps=300)
    io32, io64 = scenarios.new_wrenches(300), scenarios.new_wrenches(300)
    oracle.batch(REF32, 4, sc["bodies"], sc["meshes"], sc["ocean"], scenarios.settings(), io32)
    oracle.batch(REF64, 4, sc["bodies"], sc["meshes"], sc["ocean"], scenarios.settings(), io64)
    e = scaled_errors(io32, io64, 0.5)
    crossing = io64["position"] == abi.CROSSING_SURFACE
    for k, v in e.items():
        assert np.median(v[crossing]) < 1e-6, k
        assert np.percentile(v[crossing], 99) < 1e-4, k


def test_translation_invariance(oracle, sphere):
    sc = scenarios.single_sphere(steps=20)
    b = sc["bodies"].copy()
    io1, io2 = scenarios.new_wrenches(20), scenarios.new_wrenches(20)
    oracle.batch(REF64, 2, b, sc["meshes"], sc["ocean"], scenarios.settings(), io1)
    shift = np.array([3.0, -2.0, 0.0])
    for k in ("T_CG", "T_C"):
        b[k]["origin"] += shift
    b["aabb_min"] += shift
    b["aabb_max"] += shift
    oracle.batch(REF64, 2, b, sc["meshes"], sc["ocean"], scenarios.settings(), io2)
    e = scaled_errors(io2, io1, 0.5)
    for k, v in e.items():
        assert np.max(v) < 1e-9, k


def test_wrench_continuous_across_waterline(oracle, sphere):
    zmax = float(sphere[0][:, 2].max())
    res = []
    for eps in (-1e-4, 1e-4):
        b = sphere_body(-(zmax + eps) + 0.3, v=(0.3, 0.1, 0.2))
        io = scenarios.new_wrenches(1)
        oracle.body_forces(REF64, b, sphere, still_ocean(), scenarios.settings(), io)
        res.append(io)
    e = scaled_errors(res[0], res[1], 0.5)
    for k in ("Fb", "Fdq", "Fdf"):
        assert e[k][0] < 1e-2, k


def test_variants_share_branches(oracle):
    """Same classification in every variant for the whole single-sphere run."""
    sc = scenarios.single_sphere(steps=200)
    pos = []
    for v in ALL:
        io = scenarios.new_wrenches(200)
        oracle.batch(v, 2, sc["bodies"], sc["meshes"], sc["ocean"], scenarios.settings(), io)
        pos.append(io["position"].copy())
    for p in pos[1:]:
        assert np.array_equal(p, pos[0])


def test_centred_scene_is_closer_to_fp64(oracle):
    """The reference's FP32 arithmetic on bodies moved to the origin (what
    HYDRO_FRAME_CENTRED evaluates) against the all-FP64 evaluation: the
    rounding no longer grows with the distance from the world origin."""
    from tests.helpers import centred_scene
    sc = scenarios.mixed_batch(n_bodies=400, seed=64, scale_faces=0.1)
    st = scenarios.settings()
    r64 = scenarios.new_wrenches(len(sc["bodies"]))
    oracle.batch(REF64, 8, sc["bodies"], sc["meshes"], sc["ocean"], st, r64)
    out = {}
    for tag, bodies in (("world", sc["bodies"]), ("centred", centred_scene(sc["bodies"]))):
        io = scenarios.new_wrenches(len(bodies))
        oracle.batch(MIRROR32, 8, bodies, sc["meshes"], sc["ocean"], st, io)
        assert np.array_equal(io["position"], r64["position"])
        L = 0.5 * np.linalg.norm(bodies["aabb_max"] - bodies["aabb_min"], axis=1)
        act = r64["position"] == abi.CROSSING_SURFACE
        e = scaled_errors(io, r64, L)
        out[tag] = np.max(np.stack(list(e.values())), axis=0)[act]
    assert np.median(out["centred"]) < 0.25 * np.median(out["world"])
    assert np.percentile(out["centred"], 99) < np.percentile(out["world"], 99)
