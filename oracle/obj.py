"""CPU restatement of the physics-mesh ingest (test infrastructure only):
the physics part of LoadOBJ (Library/src/utils/GeometryFileUtil.cpp:52-283:
positions times scale -- only when the file has normals, :253-254 copies the
unscaled positions back otherwise -- all shapes fused), the triangulation LoadOBJ asks of
rapidobj (rapidobj::Triangulate, 3rdparty/rapidobj.hpp:7338-7503: quads cut
along the shorter diagonal, larger polygons ear-sliced by mapbox earcut
v2.2.4, rapidobj.hpp:358-1160, in the axis plane of largest projected area,
each triangle's first two corners swapped), and OpenGLContent::Refine
(Library/src/graphics/OpenGLContent.cpp:2833-2895) with the FP32 face areas
of PlainMesh::ComputeFaceArea (Library/include/graphics/OpenGLDataStructs.h:219-224).

The ear slicer follows mapbox earcut.hpp v2.2.4 step for step; its licence:

    ISC License

    Copyright (c) 2015, Mapbox

    Permission to use, copy, modify, and/or distribute this software for any
    purpose with or without fee is hereby granted, provided that the above
    copyright notice and this permission notice appear in all copies.

    THE SOFTWARE IS PROVIDED "AS IS" AND THE AUTHOR DISCLAIMS ALL WARRANTIES
    WITH REGARD TO THIS SOFTWARE INCLUDING ALL IMPLIED WARRANTIES OF
    MERCHANTABILITY AND FITNESS. IN NO EVENT SHALL THE AUTHOR BE LIABLE FOR ANY
    SPECIAL, DIRECT, INDIRECT, OR CONSEQUENTIAL DAMAGES OR ANY DAMAGES
    WHATSOEVER RESULTING FROM LOSS OF USE, DATA OR PROFITS, WHETHER IN AN ACTION
    OF CONTRACT, NEGLIGENCE OR OTHER TORTIOUS ACTION, ARISING OUT OF OR IN
    CONNECTION WITH THE USE OR PERFORMANCE OF THIS SOFTWARE."""
from __future__ import annotations

import numpy as np

f32 = np.float32


class _Node:
    __slots__ = ("i", "x", "y", "prev", "next")

    def __init__(self, i, x, y):
        self.i, self.x, self.y = i, x, y
        self.prev = self.next = self


class _Slicer:
    """Ear slicing of one simple ring in doubles (the published earcut
    algorithm without holes; its z-order hash only speeds up the search)."""

    def __init__(self):
        self.tri = []

    @staticmethod
    def area(p, q, r):
        return (q.y - p.y) * (r.x - q.x) - (q.x - p.x) * (r.y - q.y)

    @staticmethod
    def equals(a, b):
        return a.x == b.x and a.y == b.y

    @staticmethod
    def unlink(p):
        p.next.prev = p.prev
        p.prev.next = p.next

    @staticmethod
    def insert(i, x, y, last):
        p = _Node(i, x, y)
        if last is not None:
            p.next, p.prev = last.next, last
            last.next.prev = p
            last.next = p
        return p

    def run(self, xs, ys):
        n = len(xs)
        s = 0.0
        j = n - 1
        for i in range(n):
            s += (xs[j] - xs[i]) * (ys[i] + ys[j])
            j = i
        last = None
        order = range(n) if s > 0 else range(n - 1, -1, -1)
        for i in order:
            last = self.insert(i, xs[i], ys[i], last)
        if last is not None and self.equals(last, last.next):
            self.unlink(last)
            last = last.next
        if last is None or last.prev is last.next:
            return
        self.slice(last, 0)

    def in_triangle(self, a, b, c, p):
        return ((c.x - p.x) * (a.y - p.y) >= (a.x - p.x) * (c.y - p.y)
                and (a.x - p.x) * (b.y - p.y) >= (b.x - p.x) * (a.y - p.y)
                and (b.x - p.x) * (c.y - p.y) >= (c.x - p.x) * (b.y - p.y))

    def is_ear(self, e):
        a, c = e.prev, e.next
        if self.area(a, e, c) >= 0:
            return False
        p = c.next
        while p is not a:
            if self.in_triangle(a, e, c, p) and self.area(p.prev, p, p.next) >= 0:
                return False
            p = p.next
        return True

    def filter(self, start, end=None):
        end = end or start
        p = start
        while True:
            again = False
            if self.equals(p, p.next) or self.area(p.prev, p, p.next) == 0:
                self.unlink(p)
                p = end = p.prev
                if p is p.next:
                    break
                again = True
            else:
                p = p.next
            if not (again or p is not end):
                break
        return end

    @staticmethod
    def sgn(v):
        return (v > 0) - (v < 0)

    @staticmethod
    def on_segment(p, q, r):
        return min(p.x, r.x) <= q.x <= max(p.x, r.x) and min(p.y, r.y) <= q.y <= max(p.y, r.y)

    def intersects(self, p1, q1, p2, q2):
        o1, o2 = self.sgn(self.area(p1, q1, p2)), self.sgn(self.area(p1, q1, q2))
        o3, o4 = self.sgn(self.area(p2, q2, p1)), self.sgn(self.area(p2, q2, q1))
        if o1 != o2 and o3 != o4:
            return True
        return ((o1 == 0 and self.on_segment(p1, p2, q1)) or (o2 == 0 and self.on_segment(p1, q2, q1))
                or (o3 == 0 and self.on_segment(p2, p1, q2)) or (o4 == 0 and self.on_segment(p2, q1, q2)))

    def locally_inside(self, a, b):
        if self.area(a.prev, a, a.next) < 0:
            return self.area(a, b, a.next) >= 0 and self.area(a, a.prev, b) >= 0
        return self.area(a, b, a.prev) < 0 or self.area(a, a.next, b) < 0

    def middle_inside(self, a, b):
        mx, my = (a.x + b.x) / 2, (a.y + b.y) / 2
        inside, p = False, a
        while True:
            q = p.next
            if (p.y > my) != (q.y > my) and q.y != p.y and mx < (q.x - p.x) * (my - p.y) / (q.y - p.y) + p.x:
                inside = not inside
            p = q
            if p is a:
                return inside

    def crosses_ring(self, a, b):
        p = a
        while True:
            if (p.i != a.i and p.next.i != a.i and p.i != b.i and p.next.i != b.i
                    and self.intersects(p, p.next, a, b)):
                return True
            p = p.next
            if p is a:
                return False

    def valid_diagonal(self, a, b):
        return (a.next.i != b.i and a.prev.i != b.i and not self.crosses_ring(a, b)
                and ((self.locally_inside(a, b) and self.locally_inside(b, a) and self.middle_inside(a, b)
                      and (self.area(a.prev, a, b.prev) != 0.0 or self.area(a, b.prev, b) != 0.0))
                     or (self.equals(a, b) and self.area(a.prev, a, a.next) > 0
                         and self.area(b.prev, b, b.next) > 0)))

    def cure(self, start):
        p = start
        while True:
            a, b = p.prev, p.next.next
            if (not self.equals(a, b) and self.intersects(a, p, p.next, b) and self.locally_inside(a, b)
                    and self.locally_inside(b, a)):
                self.tri += [a.i, p.i, b.i]
                self.unlink(p)
                self.unlink(p.next)
                p = start = b
            p = p.next
            if p is start:
                return self.filter(p)

    def split(self, start):
        a = start
        while True:
            b = a.next.next
            while b is not a.prev:
                if a.i != b.i and self.valid_diagonal(a, b):
                    a2, b2 = _Node(a.i, a.x, a.y), _Node(b.i, b.x, b.y)
                    an, bp = a.next, b.prev
                    a.next, b.prev = b, a
                    a2.next, an.prev = an, a2
                    b2.next, a2.prev = a2, b2
                    bp.next, b2.prev = b2, bp
                    a = self.filter(a, a.next)
                    c = self.filter(b2, b2.next)
                    self.slice(a, 0)
                    self.slice(c, 0)
                    return
                b = b.next
            a = a.next
            if a is start:
                return

    def slice(self, ear, npass):
        stop = ear
        while ear.prev is not ear.next:
            prev, nxt = ear.prev, ear.next
            if self.is_ear(ear):
                self.tri += [prev.i, ear.i, nxt.i]
                self.unlink(ear)
                ear = stop = nxt.next
                continue
            ear = nxt
            if ear is stop:
                if npass == 0:
                    self.slice(self.filter(ear), 1)
                elif npass == 1:
                    self.slice(self.cure(self.filter(ear)), 2)
                else:
                    self.split(ear)
                break


def _projected_area(x, y):
    a = f32(0)
    n = len(x)
    for i in range(1, n):
        a = f32(a + (x[i] - x[i - 1]) * ((y[i - 1] + y[i]) / f32(2)))
    a = f32(a + (x[0] - x[n - 1]) * ((y[0] + y[n - 1]) / f32(2)))
    return abs(a)


def triangulate(raw: np.ndarray, poly: list[int]) -> list[tuple[int, int, int]]:
    """One OBJ polygon (indices into raw float32 positions) to triangles."""
    n = len(poly)
    if n == 3:
        return [tuple(poly)]
    P = [raw[i] for i in poly]
    if n == 4:
        e = P[0] - P[2]
        f = P[1] - P[3]
        d02 = f32(f32(e[0] * e[0] + e[1] * e[1]) + e[2] * e[2])
        d13 = f32(f32(f[0] * f[0] + f[1] * f[1]) + f[2] * f[2])
        c = d02 < d13
        return [(poly[0], poly[1], poly[2] if c else poly[3]), (poly[0] if c else poly[1], poly[2], poly[3])]
    xs, ys, zs = ([p[k] for p in P] for k in range(3))
    ax, ay, az = _projected_area(ys, zs), _projected_area(xs, zs), _projected_area(xs, ys)
    if max(ax, ay, az) < np.finfo(np.float32).tiny:
        raise ValueError("degenerate polygon")
    if ax > ay:
        u, w = (ys, zs) if ax > az else (xs, ys)
    else:
        u, w = (xs, zs) if ay > az else (xs, ys)
    s = _Slicer()
    s.run([float(v) for v in u], [float(v) for v in w])
    if not s.tri:
        raise ValueError("polygon cannot be triangulated")
    t = s.tri
    return [(poly[t[k + 1]], poly[t[k]], poly[t[k + 2]]) for k in range(0, len(t), 3)]


def parse_obj(text: str, scale: float = 1.0):
    raw, polys = [], []
    has_normals = False
    for line in text.splitlines():
        tok = line.split()
        if not tok:
            continue
        if tok[0] == "vn":
            has_normals = True
        if tok[0] == "v":
            raw.append([f32(float(t)) for t in tok[1:4]])
        elif tok[0] == "f":
            idx = []
            for t in tok[1:]:
                i = int(t.split("/")[0])
                idx.append(i - 1 if i > 0 else len(raw) + i)
            polys.append(idx)
    raw = np.array(raw, dtype=np.float32).reshape(-1, 3)
    faces = [f for p in polys for f in triangulate(raw, p)]
    if not has_normals:
        scale = 1.0
    return (f32(scale) * raw).astype(np.float32), np.array(faces, dtype=np.uint32).reshape(-1, 3)


def face_area(xyz, f) -> np.float32:
    a, b, c = xyz[f[0]], xyz[f[1]], xyz[f[2]]
    u = [b[k] - a[k] for k in range(3)]
    v = [c[k] - a[k] for k in range(3)]
    n = [u[1] * v[2] - v[1] * u[2], u[2] * v[0] - v[2] * u[0], u[0] * v[1] - v[0] * u[1]]
    return np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]) / f32(2)


def average_area(xyz, faces) -> np.float32:
    a = f32(0)
    for f in faces:
        a = f32(a + face_area(xyz, f))
    return f32(a / f32(len(faces)))


def refine(xyz: np.ndarray, faces: np.ndarray, threshold: float = 3.0):
    xyz = [np.asarray(p, dtype=np.float32) for p in xyz]
    faces = [tuple(int(i) for i in f) for f in faces]
    thr = f32(threshold)
    avg = max(average_area(xyz, faces), f32(0.01) * f32(0.01))
    while True:
        out, n_sub = [], 0
        for f in faces:
            if face_area(xyz, f) > thr * avg:
                mid = []
                for e in range(3):
                    a, b = xyz[f[e]], xyz[f[(e + 1) % 3]]
                    mid.append(len(xyz))
                    xyz.append(((a + b) / f32(2)).astype(np.float32))
                out += [(f[0], mid[0], mid[2]), (f[1], mid[1], mid[0]), (f[2], mid[2], mid[1]),
                        (mid[0], mid[1], mid[2])]
                n_sub += 1
            else:
                out.append(f)
        if n_sub == 0:
            break
        faces = out
        avg = max(average_area(xyz, faces), f32(0.01) * f32(0.01))
    return np.array(xyz, dtype=np.float32), np.array(faces, dtype=np.uint32)


def to_obj(xyz: np.ndarray, faces: np.ndarray, quads: bool = False) -> str:
    """OBJ text of a triangle mesh; with quads=True pairs of consecutive
    triangles that share an edge are written as one quad (so the parser's
    triangulation is exercised) where their union is the fan of the quad."""
    lines = ["# generated", "o mesh"] + [f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}" for p in xyz]
    i = 0
    while i < len(faces):
        a = faces[i]
        if quads and i + 1 < len(faces):
            b = faces[i + 1]
            if a[0] == b[0] and a[2] == b[1]:        # (p0,p1,p2) + (p0,p2,p3) = fan of p0 p1 p2 p3
                lines.append(f"f {a[0] + 1}/1/1 {a[1] + 1}/1/1 {a[2] + 1}/1/1 {b[2] + 1}/1/1")
                i += 2
                continue
        lines.append(f"f {a[0] + 1} {a[1] + 1} {a[2] + 1}")
        i += 1
    return "\n".join(lines) + "\n"
