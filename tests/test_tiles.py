"""Mesh tiling (host code, no GPU): the compact-patch tiles that
hydro_mesh_upload stores, checked through hydro_debug_tile_order.

Every face lands in exactly one tile, a tile holds at most HYDRO_TILE_FACES
faces and 448 distinct vertices, tiles are spatially compact, and the
tiling does not depend on the mesh's face order: a shuffled mesh gets as
few vertices per face and as compact tiles as the builder's own order."""
import numpy as np
import pytest

from stonefish_gb300 import abi, meshes

MAX_VERTS = 448


def _check(faces, nv):
    order, starts = abi.tile_order(faces, nv)
    assert starts[0] == 0 and starts[-1] == len(faces)
    assert np.array_equal(np.sort(order), np.arange(len(faces)))
    verts = 0
    for a, b in zip(starts[:-1], starts[1:]):
        assert 0 < b - a <= abi.TILE_FACES
        n = len(np.unique(faces[order[a:b]]))
        assert n <= MAX_VERTS
        verts += n
    return order, starts, verts / len(faces)


def _compactness(xyz, faces, order, starts):
    """Mean tile box diagonal over the diagonal a patch of HYDRO_TILE_FACES
    faces would have if the mesh box diagonal scaled with the square root of
    the face count (about 1 to 3 for compact patches)."""
    full = np.linalg.norm(xyz.max(0) - xyz.min(0))
    d = []
    for a, b in zip(starts[:-1], starts[1:]):
        p = xyz[np.unique(faces[order[a:b]])]
        d.append(np.linalg.norm(p.max(0) - p.min(0)))
    return float(np.mean(d)) / (full * np.sqrt(abi.TILE_FACES / len(faces)))


def _mesh(name):
    if name == "icosphere":
        return meshes.build_icosphere(0.5, 5)
    if name == "cylinder":
        return meshes.capped_cylinder_for_faces(0.25, 2.0, 20000)
    if name == "small_box":
        return meshes.build_box((0.3, 0.2, 0.4), 2)
    return meshes.build_box((0.3, 0.2, 0.4), 5)


@pytest.mark.parametrize("mesh", ["icosphere", "cylinder", "box", "small_box"])
def test_tiles_cover_faces_within_limits(built_library, mesh):
    xyz, fc = _mesh(mesh)
    order, starts, vpf = _check(fc, len(xyz))
    n_min = int(np.ceil(len(fc) / abi.TILE_FACES))
    assert len(starts) - 1 <= int(n_min * 1.1) + 2, (len(starts) - 1, n_min)
    if mesh == "small_box":
        # 192 faces on six separately indexed sides share one tile
        assert len(starts) == 2
        return
    # a closed surface has about half as many vertices as faces; tile borders add some
    assert vpf < 0.65, vpf
    assert _compactness(xyz, fc, order, starts) < 3.5


@pytest.mark.parametrize("mesh", ["icosphere", "cylinder", "box"])
def test_tiling_independent_of_face_order(built_library, mesh):
    """A mesh whose faces arrive in random order gets tiles about as good as
    the generator's order: greedy tiling in face order would give about three
    new vertices per face and tiles spread over the whole surface."""
    xyz, fc = _mesh(mesh)
    shuffled = fc[np.random.default_rng(4).permutation(len(fc))]
    o1, s1, v1 = _check(fc, len(xyz))
    o2, s2, v2 = _check(shuffled, len(xyz))
    assert v2 < v1 * 1.05, (v1, v2)
    c2 = _compactness(xyz, shuffled, o2, s2)
    assert c2 < 3.5 and c2 < 2.0 * _compactness(xyz, fc, o1, s1), c2


def test_degenerate_faces_and_bad_indices(built_library):
    xyz, fc = meshes.build_icosphere(0.5, 2)
    fc = fc.copy()
    fc[5] = (fc[5][0], fc[5][0], fc[5][1])        # a repeated vertex
    _check(fc, len(xyz))
    bad = fc.copy()
    bad[3, 1] = len(xyz)
    with pytest.raises(abi.HydroError) as e:
        abi.tile_order(bad, len(xyz))
    assert e.value.status == abi.HYDRO_ERR_INDEX_RANGE
