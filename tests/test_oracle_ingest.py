"""Mesh ingest on the CPU: the library's OBJ parser and refinement
(hydro_obj_parse, host code) against the Python restatement, and the mass
properties oracle (ComputePhysicalProperties, GeometryFileUtil.cpp:335-566)
against closed forms."""
import math
import os

import numpy as np
import pytest

from oracle import obj as ref_obj
from oracle.ref import source_root
from stonefish_gb300 import abi, meshes

RHO = 1000.0


def test_parse_triangulates_like_rapidobj_and_skips_other_statements(built_library):
    text = "\n".join([
        "# comment", "mtllib x.mtl", "o quad", "v 0 0 0", "v 1 0 0", "v 1 1 0", "v 0 1 0", "vt 0 0", "vn 0 0 1",
        "g g1", "usemtl m", "s off", "f 1/1/1 2/1/1 3/1/1 4/1/1",
        "o pent", "v 0 0 1", "v 1 0 1", "v 1.5 0.5 1", "v 1 1 1", "v 0 1 1", "f -5 -4 -3 -2 -1",
    ]) + "\n"
    xyz, faces = abi.obj_parse(text, scale=2.0)
    rx, rf = ref_obj.parse_obj(text, scale=2.0)
    # the square's diagonals are equal, so it is cut along 1-3; the pentagon
    # is ear-sliced and each triangle's first two corners swapped
    assert faces.tolist() == [[0, 1, 3], [1, 2, 3], [8, 7, 4], [5, 4, 6], [7, 6, 4]]
    np.testing.assert_array_equal(faces, rf)
    np.testing.assert_array_equal(xyz, rx)
    assert xyz[6].tolist() == [3.0, 1.0, 2.0]


def _polygon_obj(pts):
    lines = [f"v {x:.9g} {y:.9g} {z:.9g}" for x, y, z in pts]
    return "\n".join(lines + ["f " + " ".join(str(i + 1) for i in range(len(pts)))]) + "\n"


def _ring(n, r_out, r_in=None, plane="xy", seed=None):
    a = np.linspace(0, 2 * np.pi, n, endpoint=False)
    r = np.full(n, r_out) if r_in is None else np.where(np.arange(n) % 2 == 0, r_out, r_in)
    if seed is not None:
        r = r * np.random.default_rng(seed).uniform(0.6, 1.0, n)
    u, v = r * np.cos(a), r * np.sin(a)
    w = 0.05 * np.sin(3 * a)                          # slightly non-planar
    return {"xy": np.stack([u, v, w], 1), "xz": np.stack([u, w, v], 1), "yz": np.stack([w, u, v], 1)}[plane]


POLYGONS = {
    "quad_short_02": [(0, 0, 0), (2, 0, 0), (2.1, 1, 0), (0, 1, 0)],
    "quad_short_13": [(0, 0, 0), (1, 0, 0), (1.5, 1.2, 0), (-0.3, 1, 0)],
    "hexagon_xz": _ring(6, 1.0, plane="xz"),
    "circle_100_yz": _ring(100, 2.0, plane="yz"),           # > 80 points: the reference hashes
    "star_10": _ring(10, 1.0, 0.4),
    "star_reversed": _ring(14, 1.0, 0.35)[::-1],
    "random_star_255": _ring(255, 1.0, 0.5, seed=4),
    "L_shape": [(0, 0, 0), (2, 0, 0), (2, 1, 0), (1, 1, 0), (1, 3, 0), (0, 3, 0)],
    "collinear_points": [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0), (3, 1, 0), (1.5, 1, 0), (0, 1, 0)],
    "repeated_point": [(0, 0, 0), (1, 0, 0), (1, 0, 0), (1, 1, 0), (0.5, 1.5, 0), (0, 1, 0)],
    "bowtie": [(0, 0, 0), (2, 2, 0), (2, 0, 0), (0, 2, 0), (-1, 1, 0)],
}


def _tri_area(xyz, f):
    a, b, c = (xyz[i].astype(np.float64) for i in f)
    return 0.5 * np.linalg.norm(np.cross(b - a, c - a))


@pytest.mark.parametrize("name", list(POLYGONS))
def test_polygon_triangulation_matches_restatement(built_library, name):
    pts = np.asarray(POLYGONS[name], dtype=np.float32)
    text = _polygon_obj(pts)
    gx, gf = abi.obj_parse(text)
    px, pf = ref_obj.parse_obj(text)
    np.testing.assert_array_equal(gf, pf)
    np.testing.assert_array_equal(gx, px)
    assert set(gf.ravel().tolist()) <= set(range(len(pts)))
    if name not in ("bowtie", "repeated_point", "collinear_points"):
        assert len(gf) == len(pts) - 2
    if name.startswith(("hexagon", "circle", "star", "random", "L_")):
        # simple polygons: the triangles tile the polygon (projected area kept)
        drop = {"xz": 1, "yz": 0}.get(name.rsplit("_", 1)[-1], 2)
        q = np.delete(pts.astype(np.float64), drop, axis=1)
        poly_area = 0.5 * abs(np.sum(q[:, 0] * np.roll(q[:, 1], -1) - np.roll(q[:, 0], -1) * q[:, 1]))
        tri = np.delete(gx.astype(np.float64), drop, axis=1)[gf.astype(np.int64)]
        d1, d2 = tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]
        assert math.isclose(0.5 * np.abs(d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0]).sum(), poly_area, rel_tol=1e-5)


def test_degenerate_polygon_is_rejected(built_library):
    text = _polygon_obj([(0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 3, 3), (4, 4, 4)])
    with pytest.raises(abi.HydroError):
        abi.obj_parse(text)
    with pytest.raises(ValueError):
        ref_obj.parse_obj(text)


def test_parse_crlf_and_tabs(built_library):
    text = "v\t0 0 0\r\nv 1 0 0\r\n  v 0 1 0\r\nf\t1 2 3\r\n"
    xyz, faces = abi.obj_parse(text)
    assert xyz.shape == (3, 3) and faces.tolist() == [[0, 1, 2]]


@pytest.mark.parametrize("text", [
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 0\n",       # index 0
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n",       # out of range
    "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 -4 2\n",      # negative out of range
    "v 0 0 0\nv 1 0 0\nf 1 2\n",                  # fewer than 3 vertices
    "v 0 0 0\n" * 3 + "f" + " 1" * 256 + "\n",     # more than 255 vertices
    "v 0 0 0\nv 1 0\n",                           # bad vertex
    "v 0 0 0\nv 1 0 0\nv 0 1 0\n",                # no faces
    "",
])
def test_parse_rejects_malformed_input(built_library, text):
    with pytest.raises(abi.HydroError) as e:
        abi.obj_parse(text)
    assert e.value.status == abi.HYDRO_ERR_INVALID_ARG


def test_parse_capacity_too_small_is_an_error(built_library):
    import ctypes as C
    lib = abi.load_library()
    b = b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    nv, nf = C.c_uint32(), C.c_uint32()
    xyz = np.zeros((2, 3), np.float32)
    faces = np.zeros((1, 3), np.uint32)
    st = lib.hydro_obj_parse(b, len(b), 1.0, 0.0, xyz.ctypes.data, 2, faces.ctypes.data, 1, C.byref(nv),
                             C.byref(nf))
    assert st == abi.HYDRO_ERR_INVALID_ARG and nv.value == 3 and nf.value == 1


@pytest.mark.parametrize("quads", [False, True])
def test_refine_matches_restatement_bit_for_bit(built_library, quads):
    # a box with long thin side faces and one large face: Refine splits the
    # faces above 3x the mean area, recomputes the mean, and repeats
    xyz, faces = meshes.build_box([2.0, 0.3, 0.15], 2)
    xyz = np.concatenate([xyz, np.float32([[0, 0, 5], [6.0, 0, 5], [0, 4.5, 5.3]])])
    faces = np.concatenate([faces, np.uint32([[len(xyz) - 3, len(xyz) - 2, len(xyz) - 1]])])
    text = ref_obj.to_obj(xyz, faces, quads=quads)
    gx, gf = abi.obj_parse(text, 1.0, 3.0)
    px, pf = ref_obj.parse_obj(text)
    rx, rf = ref_obj.refine(px, pf, 3.0)
    assert len(gf) > len(faces)
    np.testing.assert_array_equal(gf, rf)
    np.testing.assert_array_equal(gx, rx)
    # refinement keeps the surface (midpoint splits are exact in area up to rounding)
    assert math.isclose(meshes.mesh_area(gx, gf), meshes.mesh_area(px, pf), rel_tol=1e-6)
    # no face is left above threshold x the final mean
    areas = np.array([ref_obj.face_area(gx, f) for f in gf], dtype=np.float32)
    assert areas.max() <= np.float32(3.0) * max(ref_obj.average_area(gx, gf), np.float32(1e-4))


def test_refine_threshold_zero_leaves_the_mesh(built_library):
    xyz, faces = meshes.build_icosphere(1.0, 1)
    gx, gf = abi.obj_parse(ref_obj.to_obj(xyz, faces), 1.0, 0.0)
    np.testing.assert_array_equal(gf, faces)
    np.testing.assert_array_equal(gx, xyz)


def _pyramid_shell_trace(a, t, rho):
    # the reference's shell inertia: solids of the faces offset by +-t/2 along
    # their normals, each face a pyramid from the centre (square base a x a,
    # height h): integral of r^2 = a^2 h^3 / 5 + a^4 h / 30
    def s(h):
        return a * a * h ** 3 / 5 + a ** 4 * h / 30
    return 2 * rho * 6 * (s((a + t) / 2) - s((a - t) / 2))


def test_oracle_solid_cube(oracle):
    xyz, faces = meshes.build_box([0.5, 0.5, 0.5], 2)
    p = oracle.mesh_properties((xyz + np.float32([3, -1, 2]), faces), 0.0, RHO)
    assert math.isclose(p["volume"], 1.0, rel_tol=1e-12)
    assert math.isclose(p["mass"], RHO, rel_tol=1e-12)
    assert math.isclose(p["surface"], 6.0, rel_tol=1e-12)
    np.testing.assert_allclose(p["CG"], [3, -1, 2], atol=1e-12)
    assert math.isclose(p["trace"], 3 * RHO / 6, rel_tol=1e-12)


def test_oracle_shell_cube(oracle):
    t = 0.01
    xyz, faces = meshes.build_box([0.5, 0.5, 0.5], 2)
    p = oracle.mesh_properties((xyz, faces), t, RHO)
    assert math.isclose(p["volume"], 6 * t, rel_tol=1e-12)
    assert math.isclose(p["mass"], 6 * t * RHO, rel_tol=1e-12)
    np.testing.assert_allclose(p["CG"], 0, atol=1e-12)
    assert math.isclose(p["trace"], _pyramid_shell_trace(1.0, t, RHO), rel_tol=1e-9)


def test_oracle_sphere(oracle):
    xyz, faces = meshes.build_icosphere(1.0, 4)
    p = oracle.mesh_properties((xyz, faces), 0.0, RHO)
    m = 4 / 3 * math.pi * RHO
    assert math.isclose(p["volume"] * RHO, p["mass"], rel_tol=1e-14)
    assert math.isclose(p["mass"], m, rel_tol=1e-3)
    assert math.isclose(p["trace"], 3 * 0.4 * m, rel_tol=1e-3)
    assert math.isclose(p["surface"], meshes.mesh_area(xyz, faces), rel_tol=1e-9)


def _reference_data():
    root = source_root()
    return None if root is None else os.path.join(root, "Tests", "Data")


REFERENCE_DATA = _reference_data()


def _reference_objs():
    if REFERENCE_DATA is None or not os.path.isdir(REFERENCE_DATA):
        return []
    return sorted(f for f in os.listdir(REFERENCE_DATA) if f.endswith(".obj"))


@pytest.mark.skipif(not _reference_objs(), reason="the reference's test meshes are not on this machine")
@pytest.mark.parametrize("name", _reference_objs() or ["none"])
def test_reference_meshes_parse_like_restatement(built_library, oracle, name):
    """Every OBJ the reference's test scenarios load: the library's parse
    (and, for the hydrodynamic hulls, Refine with Polyhedron's threshold 3)
    equals the restatement, and the oracle's mass properties are finite."""
    with open(os.path.join(REFERENCE_DATA, name), encoding="utf-8", errors="replace") as fh:
        text = fh.read()
    gx, gf = abi.obj_parse(text, 1.0, 0.0)
    px, pf = ref_obj.parse_obj(text)
    np.testing.assert_array_equal(gf, pf)
    np.testing.assert_array_equal(gx, px)
    if "hydro" in name or "phy" in name:
        rx, rf = abi.obj_parse(text, 1.0, 3.0)
        qx, qf = ref_obj.refine(px, pf, 3.0)
        np.testing.assert_array_equal(rf, qf)
        np.testing.assert_array_equal(rx, qx)
        p = oracle.mesh_properties((rx, rf), 0.0, RHO)
        assert np.isfinite([p["mass"], p["volume"], p["surface"], p["trace"], *p["CG"]]).all()
