"""Mesh builders: face/vertex counts of the reference's builders and closed,
outward-facing surfaces (no GPU)."""
import math

import numpy as np
import pytest

from stonefish_gb300 import meshes


def edge_counts(xyz, faces):
    """Each undirected geometric edge (vertices matched by position to 1e-6 m)
    must occur exactly twice.  The cylinder's seam vertices differ by
    sin(2*pi) in float32 (OpenGLContent.cpp:2125-2131), hence the rounding."""
    q = np.round(np.asarray(xyz, dtype=np.float64) * 1e6).astype(np.int64)
    key = {}
    canon = np.array([key.setdefault(tuple(p), i) for i, p in enumerate(map(tuple, q))])
    f = canon[faces.astype(np.int64)]
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    e.sort(axis=1)
    _, c = np.unique(e, axis=0, return_counts=True)
    return c


@pytest.mark.parametrize("s", [0, 1, 2, 3])
def test_icosphere_counts_and_volume(s):
    xyz, faces = meshes.build_icosphere(0.5, s)
    assert faces.shape == (20 * 4 ** s, 3)
    assert xyz.shape == (10 * 4 ** s + 2, 3)
    assert meshes.mesh_volume(xyz, faces) == pytest.approx(4 / 3 * math.pi * 0.125, rel=1e-6)
    assert np.all(edge_counts(xyz, faces) == 2)


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_box_counts_closed_volume(k):
    xyz, faces = meshes.build_box((0.3, 0.2, 0.1), k)
    assert faces.shape == (12 * 4 ** k, 3)
    assert meshes.mesh_volume(xyz, faces) == pytest.approx(8 * 0.3 * 0.2 * 0.1, rel=1e-6)
    assert np.all(edge_counts(xyz, faces) == 2)


@pytest.mark.parametrize("slices", [8, 32])
def test_cylinder_counts_closed(slices):
    xyz, faces = meshes.build_cylinder(0.2, 1.0, slices)
    assert faces.shape == (64 * slices, 3)
    # volume-corrected radius (OpenGLContent.cpp:2117-2119): volume close to pi r^2 h
    assert meshes.mesh_volume(xyz, faces) == pytest.approx(math.pi * 0.04 * 1.0, rel=2e-3)
    assert np.all(edge_counts(xyz, faces) == 2)


@pytest.mark.parametrize("nf", [500, 8000, 20000])
def test_capped_cylinder(nf):
    xyz, faces = meshes.capped_cylinder_for_faces(0.25, 2.0, nf)
    assert abs(len(faces) - nf) / nf < 0.05
    assert np.all(edge_counts(xyz, faces) == 2)
    v = meshes.mesh_volume(xyz, faces)
    assert v > 0
    assert v == pytest.approx(meshes.capped_cylinder_volume(0.25, 2.0), rel=0.05)
