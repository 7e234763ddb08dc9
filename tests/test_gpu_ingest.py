"""GPU mass properties of uploaded meshes (hydro_mesh_compute_properties,
ComputePhysicalProperties at GeometryFileUtil.cpp:335-566) against the
oracle's serial FP64 sums (within 1e-12: only the summation order differs),
the principal axes against an eigen-decomposition of the inertia tensor
restated here in numpy, and hydro_mesh_upload_obj against hydro_obj_parse +
hydro_mesh_upload."""
import math
import os

import numpy as np
import pytest

from oracle import obj as ref_obj
from stonefish_gb300 import abi, meshes

pytestmark = pytest.mark.gpu

RHO = 1027.0


def _rotation(seed):
    q = np.random.default_rng(seed).normal(size=4)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _p_sums(v1, v2, v3):
    V6 = np.einsum("ij,ij->i", v1, np.cross(v2, v3))
    sq = lambda k: v1[:, k] ** 2 + v2[:, k] ** 2 + v3[:, k] ** 2 + v1[:, k] * v2[:, k] + v1[:, k] * v3[:, k] + \
        v2[:, k] * v3[:, k]
    pr = lambda j, k: 2 * (v1[:, j] * v1[:, k] + v2[:, j] * v2[:, k] + v3[:, j] * v3[:, k]) + v1[:, j] * v2[:, k] + \
        v1[:, k] * v2[:, j] + v1[:, j] * v3[:, k] + v1[:, k] * v3[:, j] + v2[:, j] * v3[:, k] + v2[:, k] * v3[:, j]
    P = [2 * sq(0), 2 * sq(1), 2 * sq(2), pr(0, 1), pr(0, 2), pr(1, 2)]
    return np.array([np.sum(V6 * p) for p in P])


def _tensor(P, rho):
    xx, yy, zz, xy, xz, yz = P * rho / 120.0
    return np.array([[yy + zz, -xy, -xz], [-xy, xx + zz, -yz], [-xz, -yz, xx + yy]])


def inertia_tensor(xyz, faces, cg, thickness, rho):
    v = xyz.astype(np.float64)[faces.astype(np.int64)] - cg
    if thickness > 0:
        n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
        u = n / np.linalg.norm(n, axis=1, keepdims=True)
        o = v + u[:, None, :] * thickness / 2
        i = v - u[:, None, :] * thickness / 2
        return _tensor(_p_sums(o[:, 0], o[:, 1], o[:, 2]), rho) - _tensor(_p_sums(i[:, 0], i[:, 1], i[:, 2]), rho)
    return _tensor(_p_sums(v[:, 0], v[:, 1], v[:, 2]), rho)


def shapes():
    R = _rotation(3).astype(np.float32)
    box = meshes.build_box([1.2, 0.4, 0.25], 3)
    hull = meshes.capped_cylinder_for_faces(0.3, 2.0, 200_000)
    return {
        "box_axis_aligned": box,
        "box_rotated_offset": ((box[0] @ R.T + np.float32([4.0, -2.0, 1.5])).astype(np.float32), box[1]),
        "sphere": meshes.build_icosphere(0.8, 4),
        "hull_multi_tile": ((hull[0] @ R.T).astype(np.float32), hull[1]),
    }


@pytest.mark.parametrize("thickness", [0.0, 0.004])
@pytest.mark.parametrize("name", list(shapes().keys()))
def test_properties_match_oracle(oracle, hctx, name, thickness):
    xyz, faces = shapes()[name]
    mid = hctx.upload_mesh(xyz, faces)
    g = hctx.mesh_properties(mid, thickness, RHO)
    r = oracle.mesh_properties((xyz, faces), thickness, RHO)
    for k in ("mass", "volume", "surface"):
        assert math.isclose(g[k], r[k], rel_tol=1e-12), (k, g[k], r[k])
    ext = np.abs(xyz).max()
    np.testing.assert_allclose(g["CG"], r["CG"], rtol=0, atol=1e-12 * ext)
    assert math.isclose(g["Ipri"].sum(), r["trace"], rel_tol=1e-9), (g["Ipri"], r["trace"])

    # principal axes: Ipri are the eigenvalues of the tensor, Irot's columns
    # the axes (orthonormal, right-handed)
    I = inertia_tensor(xyz, faces, g["CG"], thickness, RHO)
    lam = np.linalg.eigvalsh(I)
    scale = lam.max()
    np.testing.assert_allclose(np.sort(g["Ipri"]), lam, rtol=0, atol=1e-7 * scale)
    Rm = g["Irot"]
    np.testing.assert_allclose(Rm.T @ Rm, np.eye(3), atol=1e-6)
    assert np.linalg.det(Rm) > 0
    np.testing.assert_allclose(I @ Rm, Rm * g["Ipri"][None, :], rtol=0, atol=1e-6 * scale)
    if name == "box_axis_aligned":
        np.testing.assert_array_equal(Rm, np.eye(3))
        np.testing.assert_allclose(g["Ipri"], np.diag(I), rtol=1e-12)


def test_upload_obj_equals_parse_then_upload(hctx):
    xyz, faces = meshes.build_box([1.5, 0.5, 0.5], 1)
    xyz = np.concatenate([xyz, np.float32([[0, 0, 3], [5, 0, 3], [0, 4, 3.2]])])
    faces = np.concatenate([faces, np.uint32([[len(xyz) - 3, len(xyz) - 2, len(xyz) - 1]])])
    text = ref_obj.to_obj(xyz, faces, quads=True)
    px, pf = abi.obj_parse(text, 0.5, 3.0)
    a = hctx.upload_obj(text, 0.5, 3.0)
    b = hctx.upload_mesh(px, pf)
    assert hctx.mesh_info(a)[:2] == (len(px), len(pf)) == hctx.mesh_info(b)[:2]
    pa, pb = hctx.mesh_properties(a, 0.0, RHO), hctx.mesh_properties(b, 0.0, RHO)
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k])


def test_upload_obj_rejects_malformed_text(hctx):
    with pytest.raises(abi.HydroError) as e:
        hctx.upload_obj("v 0 0 0\nf 1 2 3\n")
    assert e.value.status == abi.HYDRO_ERR_INVALID_ARG


def test_properties_unknown_mesh(hctx):
    with pytest.raises(abi.HydroError) as e:
        hctx.mesh_properties(10 ** 6)
    assert e.value.status == abi.HYDRO_ERR_NOT_FOUND


@pytest.mark.parametrize("name", ["sphere", "box", "cylinder_x", "cylinder_y", "bumpy"])
def test_properties_match_reference_fixture(hctx, name):
    """hydro_mesh_compute_properties against the reference's own
    ComputePhysicalProperties (tests/golden/ref_ingest.npz, made by the
    reference's code compiled from its source): the GPU's FP64 face sums
    differ from the reference's serial sums only in order."""
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ingest.npz"))
    xyz, faces = z[f"{name}_xyz"], z[f"{name}_faces"]
    mid = hctx.upload_mesh(xyz, faces)
    ext = float(np.abs(xyz).max())
    for row, th in zip(z[f"{name}_props"], (-1.0, 0.01)):
        g = hctx.mesh_properties(mid, th, 900.0)
        for k, v in (("mass", row[0]), ("volume", row[1]), ("surface", row[2])):
            assert math.isclose(g[k], v, rel_tol=1e-12), (name, th, k, g[k], v)
        np.testing.assert_allclose(g["CG"], row[3:6], rtol=0, atol=1e-12 * ext)
        ipri = row[6:9]
        np.testing.assert_allclose(np.sort(g["Ipri"]), np.sort(ipri), rtol=1e-9, atol=1e-12 * ipri.max())
        lam = np.sort(ipri)
        if np.min(np.diff(lam)) > 1e-3 * lam.max():     # distinct moments: the axes are defined
            R_ref = row[9:18].reshape(3, 3)
            for j in range(3):
                col = g["Irot"][:, j]
                jr = int(np.argmin(np.abs(ipri - g["Ipri"][j])))
                assert abs(abs(float(col @ R_ref[:, jr])) - 1.0) < 1e-6, (name, th, j)
