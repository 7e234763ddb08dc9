"""Physics-mesh builders for the hydrodynamics path.

These restate the rules of Stonefish's primitive mesh builders so that the
synthetic workloads have the face counts and vertex layouts the reference
produces:

* ``build_icosphere``  -- ``OpenGLContent::BuildSphere``
  (Library/src/graphics/OpenGLContent.cpp:1948-2108): icosahedron, ``s``
  ico-subdivisions (new vertex = normalize(a + b), ``vertex4EdgeIco``
  :2700-2731), then a uniform scale so that the mesh volume equals the
  analytic sphere volume.  20*4**s faces, 10*4**s + 2 vertices.
* ``build_box``        -- ``OpenGLContent::BuildBox`` (:1690-1946): 24
  vertices (4 per side), 12 faces, ``k`` midpoint subdivisions
  (``vertex4Edge`` :2733-2785).  12*4**k faces.
* ``build_cylinder``   -- ``OpenGLContent::BuildCylinder`` (:2110-2196):
  volume-corrected radius, side strip plus two cap fans, two midpoint
  subdivisions.  64*slices faces.
* ``subdivide``        -- ``OpenGLContent::Subdivide`` (:2787-2831).

``build_capped_cylinder`` (a cylinder with hemispherical caps, the torpedo
hull of the wave and batch workloads) has no reference builder; it is a
closed latitude/longitude mesh with 2*segments*rings faces.

Arithmetic that the reference does in float (glm) is done in float32 here in
the same order; the one transcendental step of the sphere rescale is done in
float64 and rounded once, so that the builders give the same bits on x86 and
Arm hosts.  All builders return ``(xyz float32 [V,3], faces uint32 [F,3])``
with outward-facing counter-clockwise faces.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def _normalize32(v: np.ndarray) -> np.ndarray:
    """glm::normalize on float32: v * (1 / sqrt(dot(v, v)))."""
    d = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]
    inv = f32(1.0) / np.sqrt(d, dtype=np.float32)
    return (v * inv).astype(np.float32)


def subdivide(xyz: np.ndarray, faces: np.ndarray, ico: bool) -> tuple[np.ndarray, np.ndarray]:
    """One pass of OpenGLContent::Subdivide (OpenGLContent.cpp:2787-2831).

    Each face (v0, v1, v2) with edge midpoints m0=(v0,v1), m1=(v1,v2),
    m2=(v2,v0) becomes (v0,m0,m2), (v1,m1,m0), (v2,m2,m1), (m0,m1,m2).  A
    midpoint vertex is appended the first time its (sorted) edge is met.
    """
    verts = [row for row in np.asarray(xyz, dtype=np.float32)]
    lookup: dict[tuple[int, int], int] = {}
    new_faces = np.empty((len(faces) * 4, 3), dtype=np.uint32)

    def mid(a: int, b: int) -> int:
        key = (a, b) if a <= b else (b, a)
        idx = lookup.get(key)
        if idx is None:
            idx = len(verts)
            lookup[key] = idx
            s = (verts[a] + verts[b]).astype(np.float32)
            verts.append(_normalize32(s) if ico else (s / f32(2.0)).astype(np.float32))
        return idx

    for i, (a, b, c) in enumerate(np.asarray(faces, dtype=np.int64)):
        m0 = mid(int(a), int(b))
        m1 = mid(int(b), int(c))
        m2 = mid(int(c), int(a))
        new_faces[4 * i + 0] = (a, m0, m2)
        new_faces[4 * i + 1] = (b, m1, m0)
        new_faces[4 * i + 2] = (c, m2, m1)
        new_faces[4 * i + 3] = (m0, m1, m2)
    return np.stack(verts).astype(np.float32), new_faces


def mesh_volume(xyz: np.ndarray, faces: np.ndarray) -> float:
    """Signed volume, sum of v1.(v2 x v3)/6 in float64 (OpenGLContent.cpp:2071-2087)."""
    p = np.asarray(xyz, dtype=np.float64)[np.asarray(faces, dtype=np.int64)]
    v1, v2, v3 = p[:, 0], p[:, 1], p[:, 2]
    c = np.stack([v2[:, 1] * v3[:, 2] - v2[:, 2] * v3[:, 1],
                  v2[:, 2] * v3[:, 0] - v2[:, 0] * v3[:, 2],
                  v2[:, 0] * v3[:, 1] - v2[:, 1] * v3[:, 0]], axis=1)
    return float(np.sum(v1[:, 0] * c[:, 0] + v1[:, 1] * c[:, 1] + v1[:, 2] * c[:, 2]) / 6.0)


def mesh_area(xyz: np.ndarray, faces: np.ndarray) -> float:
    p = np.asarray(xyz, dtype=np.float64)[np.asarray(faces, dtype=np.int64)]
    return float(0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1).sum())


_ICO_FACES = np.array([
    (0, 4, 1), (0, 9, 4), (9, 5, 4), (4, 5, 8), (4, 8, 1),
    (8, 10, 1), (8, 3, 10), (5, 3, 8), (5, 2, 3), (2, 7, 3),
    (7, 10, 3), (7, 6, 10), (7, 11, 6), (11, 0, 6), (0, 1, 6),
    (6, 1, 10), (9, 0, 11), (9, 11, 2), (9, 2, 5), (7, 2, 11)], dtype=np.uint32)


def build_icosphere(radius: float, subdivisions: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """OpenGLContent::BuildSphere (OpenGLContent.cpp:1948-2108)."""
    X = f32(-.525731112119133606)
    Z = f32(-.850650808352039932)
    N = f32(0.0)
    xyz = np.array([(-X, N, Z), (X, N, Z), (-X, N, -Z), (X, N, -Z),
                    (N, Z, X), (N, Z, -X), (N, -Z, X), (N, -Z, -X),
                    (Z, X, N), (-Z, X, N), (Z, -X, N), (-Z, -X, N)], dtype=np.float32)
    faces = _ICO_FACES.copy()
    for _ in range(subdivisions):
        xyz, faces = subdivide(xyz, faces, ico=True)
    vol = mesh_volume(xyz, faces)
    ratio = (4.0 / 3.0 * math.pi * radius * radius * radius) / vol
    scale = f32(float(f32(ratio)) ** (1.0 / 3.0))
    return (xyz * scale).astype(np.float32), faces


def build_box(half_extents, subdivisions: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """OpenGLContent::BuildBox (OpenGLContent.cpp:1690-1946), positions only."""
    hx, hy, hz = (f32(h) for h in half_extents)
    v1 = (-hx, -hy, -hz); v2 = (-hx, hy, -hz); v3 = (hx, hy, -hz); v4 = (hx, -hy, -hz)
    v5 = (hx, hy, hz); v6 = (hx, -hy, hz); v7 = (-hx, -hy, hz); v8 = (-hx, hy, hz)
    sides = [(v1, v2, v3, v4), (v4, v3, v5, v6), (v7, v8, v2, v1),
             (v6, v5, v8, v7), (v5, v3, v2, v8), (v4, v6, v7, v1)]
    xyz = np.array([p for side in sides for p in side], dtype=np.float32)
    faces = []
    for s in range(6):
        b = 4 * s
        faces += [(b, b + 1, b + 2), (b, b + 2, b + 3)]
    faces = np.array(faces, dtype=np.uint32)
    for _ in range(subdivisions):
        xyz, faces = subdivide(xyz, faces, ico=False)
    return xyz, faces


def build_cylinder(radius: float, height: float, slices: int) -> tuple[np.ndarray, np.ndarray]:
    """OpenGLContent::BuildCylinder (OpenGLContent.cpp:2110-2196), positions only."""
    half = f32(height) / f32(2.0)
    r = f32(radius)
    dphi = f32(2.0) * f32(math.pi) / f32(slices)
    r = np.sqrt(dphi * r * r / np.sin(dphi, dtype=np.float32), dtype=np.float32)
    verts = []
    ang = [f32(float(f32(i) / f32(slices)) * math.pi * 2.0) for i in range(slices + 1)]
    s = [np.sin(a, dtype=np.float32) for a in ang]
    c = [np.cos(a, dtype=np.float32) for a in ang]
    for i in range(slices + 1):
        verts.append((s[i] * r, -c[i] * r, half))
        verts.append((s[i] * r, -c[i] * r, -half))
    faces = []
    for i in range(slices):
        faces.append((2 * i, 2 * i + 1, 2 * i + 2))
        faces.append((2 * i + 1, 2 * i + 3, 2 * i + 2))
    verts.append((f32(0), f32(0), half))
    center = len(verts) - 1
    for i in range(slices + 1):
        verts.append((s[i] * r, -c[i] * r, half))
    for i in range(slices):
        faces.append((center, center + i + 1, center + i + 2))
    verts.append((f32(0), f32(0), -half))
    center = len(verts) - 1
    for i in range(slices + 1):
        verts.append((s[i] * r, -c[i] * r, -half))
    for i in range(slices):
        faces.append((center, center + i + 2, center + i + 1))
    xyz = np.array(verts, dtype=np.float32)
    faces = np.array(faces, dtype=np.uint32)
    for _ in range(2):
        xyz, faces = subdivide(xyz, faces, ico=False)
    return xyz, faces


def build_capped_cylinder(radius: float, length: float, segments: int, rings: int,
                          axis: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Closed torpedo hull: a cylinder of ``length`` (the straight part) and
    ``radius`` with a hemispherical cap at each end, centred at the origin
    with its axis along ``axis`` (0 = x, the vehicle's forward axis).

    ``rings`` latitude circles (split between the caps and the straight part
    in proportion to their meridian lengths) and ``segments`` points per
    circle give 2*segments*rings faces.
    """
    if rings < 3 or segments < 3:
        raise ValueError("need rings >= 3 and segments >= 3")
    r = float(radius)
    L = float(length)
    cap_arc = 0.5 * math.pi * r
    total = 2.0 * cap_arc + L
    # meridian positions of the rings, uniformly spaced in arc length
    s = (np.arange(rings, dtype=np.float64) + 0.5) / rings * total
    ax = np.empty(rings)
    rad = np.empty(rings)
    for k, sk in enumerate(s):
        if sk < cap_arc:                      # back cap
            th = sk / r
            ax[k] = -0.5 * L - r * math.cos(th)
            rad[k] = r * math.sin(th)
        elif sk > cap_arc + L:                # front cap
            th = (total - sk) / r
            ax[k] = 0.5 * L + r * math.cos(th)
            rad[k] = r * math.sin(th)
        else:
            ax[k] = -0.5 * L + (sk - cap_arc)
            rad[k] = r
    phi = np.arange(segments, dtype=np.float64) / segments * 2.0 * math.pi
    pts = [(-0.5 * L - r, 0.0, 0.0)]
    for k in range(rings):
        for j in range(segments):
            pts.append((ax[k], rad[k] * math.cos(phi[j]), rad[k] * math.sin(phi[j])))
    pts.append((0.5 * L + r, 0.0, 0.0))
    xyz = np.array(pts, dtype=np.float64)
    n_last = len(pts) - 1
    faces = []
    ring = lambda k, j: 1 + k * segments + (j % segments)  # noqa: E731
    for j in range(segments):                       # back pole fan
        faces.append((0, ring(0, j + 1), ring(0, j)))
    for k in range(rings - 1):
        for j in range(segments):
            a, b = ring(k, j), ring(k, j + 1)
            c, d = ring(k + 1, j), ring(k + 1, j + 1)
            faces.append((a, b, d))
            faces.append((a, d, c))
    for j in range(segments):                       # front pole fan
        faces.append((n_last, ring(rings - 1, j), ring(rings - 1, j + 1)))
    faces = np.array(faces, dtype=np.uint32)
    # the local frame above has the hull along x; permute for other axes
    perm = {0: [0, 1, 2], 1: [2, 0, 1], 2: [1, 2, 0]}[axis]
    xyz = xyz[:, perm]
    if mesh_volume(xyz, faces) < 0:
        faces = faces[:, [0, 2, 1]].copy()
    return xyz.astype(np.float32), faces


def capped_cylinder_for_faces(radius: float, length: float, n_faces: int,
                              axis: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """A capped cylinder with close to ``n_faces`` faces (2*segments*rings)."""
    half = max(n_faces // 2, 9)
    segments = max(3, int(round(math.sqrt(half * 0.8))))
    rings = max(3, int(round(half / segments)))
    return build_capped_cylinder(radius, length, segments, rings, axis)


def capped_cylinder_volume(radius: float, length: float) -> float:
    return math.pi * radius * radius * length + 4.0 / 3.0 * math.pi * radius ** 3


def capped_cylinder_surface(radius: float, length: float) -> float:
    return 2.0 * math.pi * radius * length + 4.0 * math.pi * radius * radius
