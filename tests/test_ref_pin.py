"""The oracle against the reference's own code (no GPU).

oracle/_ref is the reference's hydrodynamics functions (SolidEntity.cpp,
Ocean.cpp, OpenGLRealOcean.cpp, Uniform/Jet/Pipe.cpp, OpenGLDataStructs),
compiled from the reference's source tree by oracle/build_ref.py.  Here the
oracle's REF32 variant -- the restatement every GPU bar is measured against
-- must give the same bits as that code: per body on whole batches, and per
face on single triangles in every depth-sign pattern.  The module is skipped
where the reference's source tree is absent."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import REF32
from oracle.ref import Reference
from stonefish_gb300 import abi, meshes, scenarios
from tests.helpers import body_transform, io_dict

pytestmark = pytest.mark.skipif(not Reference.available(), reason="reference source tree not present")

FIELDS = ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf", "Swet", "Vsub", "position")


@pytest.fixture(scope="module")
def ref():
    return Reference()


def run_both(oracle, ref, sc, settings=None, threads=4):
    st = settings or scenarios.settings()
    n = len(sc["bodies"])
    a = scenarios.new_wrenches(n)
    b = scenarios.new_wrenches(n)
    for io in (a, b):               # non-zero starting values exercise the stale-output rules
        io["Fb"] = 0.5
        io["Vsub"] = 0.25
    ref.batch(threads, sc["bodies"], sc["meshes"], sc["ocean"], st, a, waves=sc.get("waves"))
    oracle.batch(REF32, threads, sc["bodies"], sc["meshes"], sc["ocean"], st, b, waves=sc.get("waves"))
    return a, b


def assert_same(a, b, what):
    for k in FIELDS:
        bad = np.nonzero(np.any((a[k] != b[k]).reshape(len(a), -1), axis=1))[0]
        assert len(bad) == 0, f"{what}: {k} differs on {len(bad)} bodies, first {bad[:4]}"


def with_jet_and_pipe(sc):
    oc = sc["ocean"]
    oc.n_currents = 3
    c = oc.currents[1]
    c.type, c.enabled = abi.CURRENT_JET, 1
    c.point[:] = (-2.0, 0.0, 0.2)
    c.dir[:] = (1.0, 0.0, 0.0)
    c.radius, c.speed = 0.3, 2.0
    p = oc.currents[2]
    p.type, p.enabled = abi.CURRENT_PIPE, 1
    p.point[:] = (0.0, -2.0, 0.1)
    p.dir[:] = (0.0, 1.0, 0.0)
    p.radius, p.radius2, p.length, p.speed, p.gamma = 0.5, 1.0, 5.0, 1.5, 0.7
    return sc


CASES = {
    "sphere_1000_states": lambda: (scenarios.single_sphere(1000, seed=0), None),
    "sphere_inside": lambda: (scenarios.single_sphere(400, seed=11, depth=(0.5, 1.5)), None),
    "sphere_no_damping": lambda: (scenarios.single_sphere(200, seed=12), scenarios.settings(damping=False)),
    "sphere_no_buoyancy": lambda: (scenarios.single_sphere(200, seed=13), scenarios.settings(buoyancy=False)),
    "mixed_batch_512": lambda: (scenarios.mixed_batch(512, seed=14, scale_faces=0.1), None),
    "torpedoes_on_waves": lambda: (scenarios.torpedo_waves(96, seed=15, faces=3000, grid_n=256), None),
    "jet_and_pipe_currents": lambda: (with_jet_and_pipe(scenarios.single_sphere(200, seed=16)), None),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_ref32_equals_reference_per_body(oracle, ref, case):
    sc, st = CASES[case]()
    a, b = run_both(oracle, ref, sc, st)
    assert_same(a, b, case)
    assert len(np.unique(a["position"])) >= 2 or case == "sphere_inside"


def test_mode_gate_and_null_mesh(oracle, ref):
    sc = scenarios.single_sphere(60, seed=17)
    b = sc["bodies"]
    b["mode"][0::4] = abi.MODE_SURFACE
    b["mode"][1::4] = abi.MODE_FLOATING
    b["buoyancy"][2::4] = 0
    b["mesh"][3::8] = abi.NO_MESH
    x, y = run_both(oracle, ref, sc)
    assert_same(x, y, "mode gate")
    assert np.all(x["position"][0::4] == abi.SKIPPED)


def single_face_body(z, v=(0.3, -0.2, 0.1), w=(0.1, 0.2, -0.3)):
    xyz = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 1.0, 0.0]], dtype=np.float32)
    xyz[:, 2] = z
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    body = scenarios.fill_bodies(1, np.eye(3)[None], np.zeros((1, 3)), np.array([v], float),
                                 np.array([w], float), np.ones((1, 3)), 1.0, 1.0, (1, 1, 1), (.1, .1, .1), 0)
    return (xyz, faces), body


def surface_both(oracle, ref, mesh, body, ocean, settings, waves=None):
    T = body_transform(body)
    TC = body_transform(body, "T_C")
    a, b = io_dict(), io_dict()
    ref.surface_forces(settings, mesh, ocean, T, TC, body["v"][0], body["omega"][0], a, waves=waves)
    oracle.surface_forces(REF32, settings, mesh, ocean, T, TC, body["v"][0], body["omega"][0], b, waves=waves)
    return a, b


def test_single_face_every_depth_sign_pattern(oracle, ref):
    """Each corner above, on or below the surface: the 27 cases of the
    waterline clip (SolidEntity.cpp:1360-1647), bit for bit."""
    oc = scenarios.flat_ocean((0.2, 0.1, -0.3))
    levels = (-0.3, 0.0, 0.25)
    for za in levels:
        for zb in levels:
            for zc in levels:
                mesh, body = single_face_body((za, zb, zc))
                a, b = surface_both(oracle, ref, mesh, body, oc, scenarios.settings())
                for k in a:
                    assert np.array_equal(a[k], b[k]), ((za, zb, zc), k, a[k], b[k])


def test_random_faces_straddling_flat_and_waves(oracle, ref):
    rng = np.random.default_rng(18)
    waves = scenarios.wave_grid(n=128, n_waves=16, seed=19)
    for trial in range(600):
        use_waves = trial % 2 == 1
        oc = scenarios.flat_ocean(tuple(rng.uniform(-0.5, 0.5, 3)))
        oc.waves = int(use_waves)
        xyz = rng.uniform(-1.0, 1.0, (3, 3)).astype(np.float32)
        xyz[:, 2] = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        if trial % 7 == 0:                       # slivers near the degenerate-area threshold
            xyz[2] = xyz[0] + np.float32(1e-4) * (xyz[1] - xyz[0])
        faces = np.array([[0, 1, 2]], dtype=np.uint32)
        q = scenarios.random_quaternions(rng, 1)
        R = scenarios.quat_to_matrix(q)
        pos = np.array([[rng.uniform(0, 12.8), rng.uniform(0, 12.8), rng.uniform(-0.3, 0.3)]])
        body = scenarios.fill_bodies(1, R, pos, rng.uniform(-1, 1, (1, 3)), rng.uniform(-0.5, 0.5, (1, 3)),
                                     np.ones((1, 3)), 1.0, 1.0, (1, 1, 1), (.1, .1, .1), 0)
        a, b = surface_both(oracle, ref, (xyz, faces), body, oc, scenarios.settings(),
                            waves=waves if use_waves else None)
        for k in a:
            assert np.array_equal(a[k], b[k]), (trial, k, a[k], b[k])


def test_submerged_static_and_correction(oracle, ref):
    rng = np.random.default_rng(20)
    mesh = meshes.build_icosphere(0.5, 2)
    oc = scenarios.flat_ocean((0.2, 0.0, 0.0))
    for _ in range(50):
        q = scenarios.random_quaternions(rng, 1)
        R = scenarios.quat_to_matrix(q)
        body = scenarios.fill_bodies(1, R, np.array([[0.3, -0.2, 2.0]]), rng.uniform(-1, 1, (1, 3)),
                                     rng.uniform(-0.5, 0.5, (1, 3)), np.full((1, 3), 0.5), 1.0, 1.0,
                                     tuple(rng.uniform(0.2, 1.0, 3)), tuple(rng.uniform(0.01, 0.2, 3)), 0)
        T = body_transform(body)
        a, b = io_dict(), io_dict()
        ref.submerged_forces(mesh, oc, T, T, body["v"][0], body["omega"][0], a)
        oracle.submerged_forces(REF32, mesh, oc, T, T, body["v"][0], body["omega"][0], b)
        for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
            assert np.array_equal(a[k], b[k]), k
        ref.correct_forces(oc, a, body["Cd"][0], body["Cf"][0], body["R_O"][0])
        oracle.correct_forces(oc, b, body["Cd"][0], body["Cf"][0], body["R_O"][0])
        for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
            assert np.array_equal(a[k], b[k]), k


def test_null_mesh_statics(oracle, ref):
    oc = scenarios.flat_ocean()
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    for st in (scenarios.settings(), scenarios.settings(damping=False), scenarios.settings(buoyancy=False)):
        a, b = io_dict(), io_dict()
        for d in (a, b):
            for k in d:
                d[k][:] = 7.0
        ref.surface_forces(st, None, oc, T, T, np.ones(3), np.ones(3), a)
        oracle.surface_forces(REF32, st, None, oc, T, T, np.ones(3), np.ones(3), b)
        for k in a:
            assert np.array_equal(a[k], b[k]), k


def test_depth_and_fluid_position_on_waves(oracle, ref):
    rng = np.random.default_rng(21)
    waves = scenarios.wave_grid(n=64, n_waves=8, seed=22)
    oc = scenarios.flat_ocean()
    oc.waves = 1
    for _ in range(2000):
        x, y = rng.uniform(-20.0, 20.0, 2)
        z = rng.uniform(-1.0, 1.0)
        assert np.float32(ref.depth(oc, waves, x, y, z)) == np.float32(oracle.depth(oc, waves, x, y, z))
    for _ in range(300):
        lo = rng.uniform(-3, 3, 3)
        hi = lo + rng.uniform(0.0, 1.5, 3)
        assert ref.fluid_position(oc, lo, hi, waves) == oracle.fluid_position(oc, lo, hi, waves)


def test_aerodynamic_forces_and_correction(oracle, ref):
    rng = np.random.default_rng(23)
    mesh = meshes.build_box((0.3, 0.2, 0.5), 1)
    atm = abi.Atmosphere()
    atm.density = 1.2
    atm.n_winds = 1
    atm.winds[0].type, atm.winds[0].enabled = abi.CURRENT_UNIFORM, 1
    atm.winds[0].vel[:] = (3.0, -1.0, 0.5)
    for _ in range(40):
        q = scenarios.random_quaternions(rng, 1)
        R = scenarios.quat_to_matrix(q)
        body = scenarios.fill_bodies(1, R, rng.uniform(-5, 5, (1, 3)), rng.uniform(-4, 4, (1, 3)),
                                     rng.uniform(-1, 1, (1, 3)), np.ones((1, 3)), 1.0, 1.0, (1, 1, 1),
                                     (.1, .1, .1), 0)
        T = body_transform(body)
        Fa, Ta = ref.aero_forces(mesh, atm, T, T, body["v"][0], body["omega"][0])
        Fo, To = oracle.aero_forces(REF32, mesh, atm, T, T, body["v"][0], body["omega"][0])
        assert np.array_equal(Fa, Fo) and np.array_equal(Ta, To)
        for kind in (abi.APPROX_AUTO, abi.APPROX_SPHERE, abi.APPROX_CYLINDER, abi.APPROX_ELLIPSOID):
            p = abi.AeroParams()
            p.approx_type = kind
            Rh = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
            for i in range(9):
                p.R_CG2H[i] = float(Rh.reshape(-1)[i])
            for i in range(3):
                p.approx_params[i] = float(rng.uniform(0.1, 1.0))
            assert all(np.array_equal(x, y) for x, y in zip(ref.aero_correct(p, Fa, Ta),
                                                              oracle.aero_correct(p, Fa, Ta)))


def test_reference_buoyancy_of_a_submerged_sphere_mesh(ref):
    """An absolute check of the reference's own code: a fully submerged
    icosphere through the surface loop gives Vsub = the mesh's volume and
    Fb = -rho g V (Archimedes)."""
    mesh = meshes.build_icosphere(0.5, 3)
    T = abi.Transform()
    for i in (0, 4, 8):
        T.basis[i] = 1.0
    T.origin[2] = 3.0
    a = io_dict()
    oc = scenarios.flat_ocean(None)
    ref.surface_forces(scenarios.settings(), mesh, oc, T, T, np.zeros(3), np.zeros(3), a)
    V = meshes.mesh_volume(*mesh)
    assert a["Vsub"][0] == pytest.approx(V, rel=5e-5)
    assert a["Fb"][2] == pytest.approx(-V * oc.density * oc.gravity, rel=5e-5)
    assert V == pytest.approx(4 / 3 * math.pi * 0.125, rel=1e-6)


# ------------------------------------------------------ compound, cable
def _transform(R, o):
    t = abi.Transform()
    for i in range(9):
        t.basis[i] = float(np.asarray(R).reshape(-1)[i])
    for i in range(3):
        t.origin[i] = float(o[i])
    return t


def test_compound_equals_reference(oracle, ref):
    """Compound::ComputeHydrodynamicForces (Compound.cpp:291-436) from the
    reference's code against the oracle: compounds whose origin, part origins
    and part mesh frames are general transforms (the part frames formed by
    the reference's own products), external and internal parts, parts out of
    the fluid computation, a part without a mesh; INSIDE, OUTSIDE, CROSSING."""
    from oracle.ref import REF_PART_DTYPE
    rng = np.random.default_rng(41)
    mesh_list = [meshes.capped_cylinder_for_faces(0.2, 1.2, 600), meshes.build_box((0.5, 0.08, 0.06), 2),
                 meshes.build_box((0.3, 0.1, 0.05), 1), meshes.build_icosphere(0.15, 2)]
    positions = set()
    for c in range(60):
        n_parts = int(rng.integers(1, 6))
        R = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
        cg = np.array([rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-1.2, 1.2)])
        Ro = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
        T_O = _transform(Ro @ R, cg + rng.uniform(-0.05, 0.05, 3))
        comp = np.zeros(1, dtype=abi.BODY_DTYPE)
        comp["T_CG"]["basis"] = R.reshape(9)
        comp["T_CG"]["origin"] = cg
        comp["v"] = rng.uniform(-1, 1, 3)
        comp["omega"] = rng.uniform(-0.5, 0.5, 3)
        comp["volume"], comp["surface"] = 0.12, 1.7
        comp["P_CB"] = rng.uniform(-0.05, 0.05, 3)
        comp["aabb_min"] = cg - 0.9
        comp["aabb_max"] = cg + 0.9
        comp["mode"] = abi.MODE_SUBMERGED if c % 9 else abi.MODE_FLOATING
        comp["buoyancy"] = int(c % 7 != 3)
        rp = np.zeros(n_parts, dtype=REF_PART_DTYPE)
        op = np.zeros(n_parts, dtype=abi.COMPOUND_PART_DTYPE)
        for i in range(n_parts):
            o = _transform(scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0], rng.uniform(-0.4, 0.4, 3))
            o2c = _transform(scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0],
                             rng.uniform(-0.05, 0.05, 3))
            for name, t in (("origin", o), ("O2C", o2c)):
                rp[i][name]["basis"] = t.basis[:]
                rp[i][name]["origin"] = t.origin[:]
            mesh = int(rng.integers(0, 4)) if (c + i) % 11 else abi.NO_MESH
            mode = [abi.MODE_SUBMERGED, abi.MODE_FLOATING, abi.MODE_SUBMERGED, abi.MODE_DISABLED][int(rng.integers(0, 4))]
            cd, cf = rng.uniform(0.2, 1.0, 3), rng.uniform(0.01, 0.1, 3)
            external = int(i == 0 or rng.uniform() < 0.7)
            for arr in (rp, op):
                arr[i]["Cd"], arr[i]["Cf"], arr[i]["mesh"], arr[i]["mode"] = cd, cf, mesh, mode
                arr[i]["external"] = external
            rp[i]["buoyancy"] = op[i]["buoyant"] = int(rng.uniform() < 0.85)
            tc, ro = ref.compound_part_frames(T_O, o, o2c)
            op[i]["T_C"]["basis"] = tc.basis[:]
            op[i]["T_C"]["origin"] = tc.origin[:]
            op[i]["R_O"] = ro
        io_r = scenarios.new_wrenches(1)
        io_o = scenarios.new_wrenches(1)
        for io in (io_r, io_o):
            io["Fb"], io["Vsub"] = 0.5, 0.25
        ref.compound_forces(comp, T_O, rp, mesh_list, scenarios.flat_ocean(), scenarios.settings(), io_r)
        part_meshes = [None if p["mesh"] == abi.NO_MESH else mesh_list[int(p["mesh"])] for p in op]
        oracle.compound_forces(REF32, comp, op, part_meshes, scenarios.flat_ocean(), scenarios.settings(), io_o)
        assert_same(io_r, io_o, f"compound {c}")
        positions.add(int(io_r["position"][0]))
    assert {abi.INSIDE, abi.OUTSIDE, abi.CROSSING_SURFACE} <= positions


@pytest.mark.parametrize("seed", [6, 7])
def test_cables_equal_reference(oracle, ref, seed):
    """CableEntity::ComputeHydrodynamicForces (CableEntity.cpp:240-376) from
    the reference's code against the oracle, every submersion case."""
    cs = scenarios.cable_set(48, seed=seed)
    for st in (scenarios.settings(), scenarios.settings(damping=False), scenarios.settings(buoyancy=False)):
        a = np.zeros(len(cs["x"]), dtype=abi.CABLE_FORCES_DTYPE)
        b = np.zeros(len(cs["x"]), dtype=abi.CABLE_FORCES_DTYPE)
        a["Fb"] = b["Fb"] = 0.75           # untouched where the mode gate skips a cable
        ref.cable_forces(cs["cables"], cs["x"], cs["v"], cs["ocean"], st, a)
        oracle.cable_forces(cs["cables"], cs["x"], cs["v"], cs["ocean"], st, b)
        for k in ("Fb", "Fdq", "Fdf"):
            assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("state,passes", [(3.0, 8), (1.0, 7), (6.0, 8)])
def test_fft_ocean_tables_equal_reference(built_library, ref, state, passes):
    """The FFT ocean's host tables against the reference's OpenGLOcean code:
    the wave spectrum (GenerateWavesSpectrum with its seeded generator) and
    the butterfly table, each value as the reference's RGBA16F textures hold
    it (binary16, round to nearest even)."""
    p = abi.FftOceanParams()
    built = abi.load_library()
    built.hydro_fft_ocean_params_for_state(C.c_float(state), C.byref(p))
    p.passes = passes
    s12, s34, idx, w = abi.fft_ocean_tables(p)
    r12, r34 = ref.fft_spectrum(p)
    assert np.array_equal(s12, r12.astype(np.float16).astype(np.float32))
    assert np.array_equal(s34, r34.astype(np.float16).astype(np.float32))
    assert np.count_nonzero(r12) > 0.4 * r12.size
    n = 1 << passes
    bt = ref.fft_butterfly(n, passes)
    j = np.rint(bt[:, :, 0:2].astype(np.float64) * n - 0.5).astype(np.int32)
    assert np.array_equal(bt[:, :, 0:2], ((j + 0.5) / n).astype(np.float32))
    assert np.array_equal(idx, j)
    assert np.array_equal(w, bt[:, :, 2:4].astype(np.float16).astype(np.float32))
