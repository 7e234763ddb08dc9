"""Mesh ingest, mass properties and coefficient setup against the reference's
own code (no GPU).

Where the reference's source tree is present, oracle/_ref holds its LoadOBJ
(with the vendored rapidobj), OpenGLContent::Refine,
ComputePhysicalProperties and SolidEntity::ComputeFluidDynamicsApprox; the
library's host parse (hydro_obj_parse), the oracle's properties and the
library's hydro_fluid_approx are compared with them here.  The committed
fixture tests/golden/ref_ingest.npz carries the reference's outputs on
synthetic meshes, so the fixture tests run everywhere."""
import math
import os

import numpy as np
import pytest

from oracle.ref import Reference, source_root
from stonefish_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ingest.npz")
MESHES = ("sphere", "box", "cylinder_x", "cylinder_y", "bumpy")
APPROX_KEYS = ("params", "R_CG2H", "origin_CG2H", "added_mass", "added_inertia", "Cd", "Cf")
HAVE_REF = Reference.available()
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference source tree not present")


def transform(R, o):
    t = abi.Transform()
    for i in range(9):
        t.basis[i] = float(np.asarray(R).reshape(-1)[i])
    for i in range(3):
        t.origin[i] = float(o[i])
    return t


def fixture():
    z = np.load(GOLDEN)
    out = {}
    for n in MESHES:
        out[n] = {k: z[f"{n}_{k}"] for k in ("xyz", "faces", "props", "frames", "approx")}
    return out


def reference_data_dir():
    root = source_root()
    return None if root is None else os.path.join(root, "Tests", "Data")


# ------------------------------------------------- against the fixture
@pytest.mark.parametrize("name", MESHES)
def test_fluid_approx_matches_reference_fixture(built_library, name):
    """hydro_fluid_approx against the reference's ComputeFluidDynamicsApprox
    outputs stored in the fixture (bit for bit where no transcendental
    function enters; cos/sin/log/pow may differ in the last bit between C
    libraries)."""
    g = fixture()[name]
    rows = iter(g["approx"])
    for fr in g["frames"]:
        t1, t2 = transform(fr[0:9], fr[9:12]), transform(fr[12:21], fr[21:24])
        pcb = fr[24:27]
        for _ in range(4):
            r = next(rows)
            ap = int(r[0])
            a = abi.fluid_approx(g["xyz"], ap, t1, t2, pcb, 1025.0)
            assert a["type"] == int(r[1]) and len(a["params"]) == int(r[2])
            want = {"params": r[3:3 + int(r[2])], "R_CG2H": r[6:15].reshape(3, 3), "origin_CG2H": r[15:18],
                    "added_mass": r[18:21], "added_inertia": r[21:24], "Cd": r[24:27], "Cf": r[27:30]}
            for k in APPROX_KEYS:
                np.testing.assert_allclose(a[k], want[k], rtol=1e-14, atol=1e-15, err_msg=(name, ap, k))


@pytest.mark.parametrize("name", MESHES)
def test_oracle_properties_match_reference_fixture(oracle, name):
    g = fixture()[name]
    for row, th in zip(g["props"], (-1.0, 0.01)):
        p = oracle.mesh_properties((g["xyz"], g["faces"]), th, 900.0)
        assert p["mass"] == row[0] and p["volume"] == row[1] and p["surface"] == row[2], (name, th)
        assert np.array_equal(p["CG"], row[3:6]), (name, th)
        assert math.isclose(p["trace"], row[6:9].sum(), rel_tol=1e-12)


def test_fluid_approx_reads_the_reference_vertex_layouts(built_library):
    """The same vertices as packed xyz (12 B), as the reference's Vertex
    (24 B: position, normal) and TexturableVertex (44 B: position, normal, uv,
    tangent) arrays, OpenGLDataStructs.h:120-155."""
    g = fixture()["bumpy"]
    xyz = g["xyz"]
    t1 = transform(np.eye(3), (0.01, -0.02, 0.03))
    t2 = transform(np.eye(3), (0.0, 0.0, 0.0))
    base = abi.fluid_approx(xyz, abi.APPROX_ELLIPSOID, t1, t2, (0.0, 0.0, 0.01))
    for floats in (6, 11):
        aos = np.random.default_rng(floats).standard_normal((len(xyz), floats)).astype(np.float32)
        aos[:, :3] = xyz
        a = abi.fluid_approx(aos, abi.APPROX_ELLIPSOID, t1, t2, (0.0, 0.0, 0.01), vertex_stride=4 * floats)
        for k in APPROX_KEYS:
            assert np.array_equal(a[k], base[k]), (floats, k)


def test_fluid_approx_argument_errors(built_library):
    t = transform(np.eye(3), (0, 0, 0))
    one = np.zeros((1, 3), np.float32)
    with pytest.raises(abi.HydroError):
        abi.fluid_approx(one, abi.APPROX_SPHERE, t, t, (0, 0, 0))
    with pytest.raises(abi.HydroError):
        abi.fluid_approx(np.zeros((4, 3), np.float32), 9, t, t, (0, 0, 0))


# ------------------------------------------ against the reference's code
@needs_ref
def test_reference_code_reproduces_its_hull_numbers():
    """hull_hydro.obj as the reference's fluid-dynamics test builds it
    (Polyhedron: LoadOBJ at scale 1, Refine(3), solid ComputePhysicalProperties;
    FluidDynamicsTestManager.cpp:111, :207-209): volume 0.096699 and
    inertia / density (0.001080, 0.014772, 0.014772), to the printed digits."""
    ref = Reference()
    xyz, faces, _ = ref.load_obj(os.path.join(reference_data_dir(), "hull_hydro.obj"), 1.0, 3.0)
    p = ref.mesh_properties((xyz, faces), -1.0, 900.0)
    assert abs(p["volume"] - 0.096699) < 5e-7
    np.testing.assert_allclose(np.sort(p["Ipri"]) / 900.0, [0.001080, 0.014772, 0.014772], rtol=0, atol=5e-7)


@needs_ref
def test_library_parse_gives_the_hull_numbers(oracle):
    """The same hull through the library's OBJ parse and Refine
    (hydro_obj_parse) and the oracle's properties."""
    with open(os.path.join(reference_data_dir(), "hull_hydro.obj"), encoding="utf-8") as fh:
        xyz, faces = abi.obj_parse(fh.read(), 1.0, 3.0)
    p = oracle.mesh_properties((xyz, faces), -1.0, 900.0)
    assert abs(p["volume"] - 0.096699) < 5e-7
    assert abs(p["trace"] / 900.0 - (0.001080 + 2 * 0.014772)) < 1.5e-6


def _reference_objs():
    d = reference_data_dir() if HAVE_REF else None
    if d is None or not os.path.isdir(d):
        return []
    return sorted(f for f in os.listdir(d) if f.endswith(".obj"))


@needs_ref
@pytest.mark.parametrize("scale", [1.0, 2.0])
def test_library_parse_equals_reference_loadobj(scale):
    """Every OBJ of the reference's test data: the library's faces carry the
    same three positions, in the same order, as the faces of the reference's
    LoadOBJ (and Refine(3) for the hydrodynamic hulls).  The reference's copies
    of vertices that carry several normals change vertex numbers, not face
    positions.  Two files name a material library that is not shipped;
    rapidobj rejects them, and the library, which reads geometry only, parses
    them."""
    ref = Reference()
    names = _reference_objs()
    assert len(names) >= 20
    compared = 0
    for name in names:
        path = os.path.join(reference_data_dir(), name)
        th = 3.0 if ("hydro" in name or "phy" in name) else 0.0
        try:
            rx, rf, _ = ref.load_obj(path, scale, th)
        except OSError as e:
            assert "Material not found" in str(e), (name, str(e))
            continue
        with open(path, encoding="utf-8", errors="replace") as fh:
            gx, gf = abi.obj_parse(fh.read(), scale, th)
        assert rf.shape == gf.shape, name
        assert np.array_equal(rx[rf.astype(np.int64)], gx[gf.astype(np.int64)]), name
        compared += 1
    assert compared >= 20


@needs_ref
def test_obj_without_normals_ignores_scale(tmp_path):
    """LoadOBJ scales positions only for files with normals: without "vn"
    lines it copies the unscaled positions back (GeometryFileUtil.cpp:253-254)."""
    ref = Reference()
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 1 3 2\nf 1 2 4\nf 1 4 3\nf 2 3 4\n"
    path = tmp_path / "tetra.obj"
    path.write_text(text)
    for scale in (1.0, 2.5):
        rx, rf, _ = ref.load_obj(str(path), scale, 0.0)
        gx, gf = abi.obj_parse(text, scale, 0.0)
        assert np.array_equal(rx[rf.astype(np.int64)], gx[gf.astype(np.int64)])
        assert float(gx.max()) == 1.0


@needs_ref
def test_properties_and_approx_equal_reference_on_the_hull(oracle):
    ref = Reference()
    xyz, faces, _ = ref.load_obj(os.path.join(reference_data_dir(), "hull_hydro.obj"), 1.0, 3.0)
    for th in (-1.0, 0.004):
        a = ref.mesh_properties((xyz, faces), th, 900.0)
        b = oracle.mesh_properties((xyz, faces), th, 900.0)
        assert a["mass"] == b["mass"] and a["volume"] == b["volume"] and a["surface"] == b["surface"]
        assert np.array_equal(a["CG"], b["CG"])
    rng = np.random.default_rng(31)
    from stonefish_gb300 import scenarios
    for trial in range(4):
        R1 = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
        R2 = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
        t1, t2 = transform(R1, rng.uniform(-0.1, 0.1, 3)), transform(R2, rng.uniform(-0.1, 0.1, 3))
        pcb = rng.uniform(-0.02, 0.02, 3)
        for ap in (abi.APPROX_AUTO, abi.APPROX_SPHERE, abi.APPROX_CYLINDER, abi.APPROX_ELLIPSOID):
            a = ref.fluid_approx((xyz, faces), ap, t1, t2, pcb, 1025.0)
            b = abi.fluid_approx(xyz, ap, t1, t2, pcb, 1025.0)
            assert a["type"] == b["type"]
            for k in APPROX_KEYS:
                assert np.array_equal(a[k], b[k]), (trial, ap, k)


@needs_ref
def test_submerged_hull_volume_through_the_surface_loop(oracle):
    """hull_hydro.obj wholly under water through the CROSSING branch's face
    loop (ComputeHydrodynamicForcesSurface): the reference's code and the
    oracle's REF32 give the same Vsub bit for bit, equal to the hull's volume
    0.096699 (FluidDynamicsTestManager.cpp:207), and Fb = -rho g Vsub."""
    from oracle import REF32
    from tests.helpers import io_dict
    from stonefish_gb300 import scenarios
    ref = Reference()
    xyz, faces, _ = ref.load_obj(os.path.join(reference_data_dir(), "hull_hydro.obj"), 1.0, 3.0)
    mesh = (xyz, faces)
    rng = np.random.default_rng(5)
    oc = scenarios.flat_ocean(None)
    for trial in range(3):
        R = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0]
        T = transform(R, (rng.uniform(-2, 2), rng.uniform(-2, 2), 2.0 + trial))
        a, b = io_dict(), io_dict()
        ref.surface_forces(scenarios.settings(), mesh, oc, T, T, np.zeros(3), np.zeros(3), a)
        oracle.surface_forces(REF32, scenarios.settings(), mesh, oc, T, T, np.zeros(3), np.zeros(3), b)
        for k in a:
            assert np.array_equal(a[k], b[k]), (trial, k)
        assert abs(a["Vsub"][0] - 0.096699) < 5e-6, a["Vsub"][0]
        np.testing.assert_allclose(np.linalg.norm(a["Fb"]), a["Vsub"][0] * oc.density * oc.gravity, rtol=1e-6)
