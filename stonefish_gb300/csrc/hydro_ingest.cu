// hydro_ingest.cu -- physics-mesh ingest: OBJ text to a triangle mesh
// (the part of LoadOBJ, Library/src/utils/GeometryFileUtil.cpp:52-230, that
// the physics uses: positions scaled, polygons triangulated, all shapes
// fused), the refinement Polyhedron applies to it (OpenGLContent::Refine,
// Library/src/graphics/OpenGLContent.cpp:2833-2895), and the mass
// properties of a device mesh (ComputePhysicalProperties,
// GeometryFileUtil.cpp:335-566) with the per-face sums on the GPU.
//
// Host code parses and refines (the reference does both on the CPU at load
// time); the face sums run as one CTA per mesh tile with a fixed-order
// FP64 tree reduction, and the tile partials are added on the host in tile
// order.  The principal axes follow the reference's closed form.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hydro_internal.h"

namespace sfh {

// ------------------------------------------------------------------ OBJ
// LoadOBJ reads the file through rapidobj (3rdparty/rapidobj.hpp, vendored
// by the reference) and triangulates with rapidobj::Triangulate
// (rapidobj.hpp:7338-7503): triangles are kept, a quad is cut along its
// shorter diagonal, larger polygons (at most 255 vertices) go through the
// earcut ear slicer (mapbox earcut.hpp v2.2.4, rapidobj.hpp:358-1160) in the
// axis plane where the polygon's projected area is largest.  Both rules work
// on the positions as written in the file; the scale is applied afterwards
// (GeometryFileUtil.cpp:161-166), and only to a file that has normals: for a
// file without "vn" statements LoadOBJ copies the unscaled positions over the
// scaled ones (GeometryFileUtil.cpp:253-254), so such a mesh keeps the
// file's size whatever the scale.  LoadOBJ splits vertices that carry
// several normals or texture coordinates (GeometryFileUtil.cpp:100-228);
// those copies share the position, so the physics mesh here indexes the
// position list directly.
namespace {

constexpr size_t kMaxPolygon = 255;

// Ear slicing of one simple ring (no holes), in double precision, with the
// three fallback passes of the published algorithm: filter collinear and
// repeated points, cure local self-intersections, split along a valid
// diagonal.  The z-order hash the original uses above 80 points only
// narrows the point-in-ear search and does not change which ears are cut.
// The steps follow mapbox earcut.hpp v2.2.4 function for function (the
// triangles must be the ones rapidobj produces), under its licence:
//
//   ISC License
//
//   Copyright (c) 2015, Mapbox
//
//   Permission to use, copy, modify, and/or distribute this software for any
//   purpose with or without fee is hereby granted, provided that the above
//   copyright notice and this permission notice appear in all copies.
//
//   THE SOFTWARE IS PROVIDED "AS IS" AND THE AUTHOR DISCLAIMS ALL WARRANTIES
//   WITH REGARD TO THIS SOFTWARE INCLUDING ALL IMPLIED WARRANTIES OF
//   MERCHANTABILITY AND FITNESS. IN NO EVENT SHALL THE AUTHOR BE LIABLE FOR
//   ANY SPECIAL, DIRECT, INDIRECT, OR CONSEQUENTIAL DAMAGES OR ANY DAMAGES
//   WHATSOEVER RESULTING FROM LOSS OF USE, DATA OR PROFITS, WHETHER IN AN
//   ACTION OF CONTRACT, NEGLIGENCE OR OTHER TORTIOUS ACTION, ARISING OUT OF OR
//   IN CONNECTION WITH THE USE OR PERFORMANCE OF THIS SOFTWARE.
class EarSlicer {
public:
    std::vector<uint32_t> tri;   // polygon-local indices, three per triangle

    void run(const std::vector<double>& px, const std::vector<double>& py)
    {
        tri.clear();
        nodes_.clear();
        const size_t len = px.size();
        double sum = 0.0;
        for (size_t i = 0, j = len - 1; i < len; j = i++) sum += (px[j] - px[i]) * (py[i] + py[j]);
        int last = -1;
        if (sum > 0) {                                   // clockwise already
            for (size_t i = 0; i < len; ++i) last = insert((uint32_t)i, px[i], py[i], last);
        } else {
            for (size_t i = len; i-- > 0;) last = insert((uint32_t)i, px[i], py[i], last);
        }
        if (last >= 0 && equals(last, nx(last))) {
            unlink(last);
            last = nx(last);
        }
        if (last < 0 || pv(last) == nx(last)) return;
        slice(last, 0);
    }

private:
    struct Node {
        uint32_t i;
        double x, y;
        int prev, next;
    };
    std::vector<Node> nodes_;

    int nx(int p) const { return nodes_[p].next; }
    int pv(int p) const { return nodes_[p].prev; }

    int insert(uint32_t i, double x, double y, int last)
    {
        const int p = (int)nodes_.size();
        nodes_.push_back({i, x, y, p, p});
        if (last >= 0) {
            nodes_[p].next = nodes_[last].next;
            nodes_[p].prev = last;
            nodes_[nodes_[last].next].prev = p;
            nodes_[last].next = p;
        }
        return p;
    }
    void unlink(int p)
    {
        nodes_[nodes_[p].next].prev = nodes_[p].prev;
        nodes_[nodes_[p].prev].next = nodes_[p].next;
    }
    double area(int p, int q, int r) const
    {
        const Node &P = nodes_[p], &Q = nodes_[q], &R = nodes_[r];
        return (Q.y - P.y) * (R.x - Q.x) - (Q.x - P.x) * (R.y - Q.y);
    }
    bool equals(int a, int b) const { return nodes_[a].x == nodes_[b].x && nodes_[a].y == nodes_[b].y; }
    static int sgn(double v) { return (0.0 < v) - (v < 0.0); }
    void emit(int a, int b, int c)
    {
        tri.push_back(nodes_[a].i);
        tri.push_back(nodes_[b].i);
        tri.push_back(nodes_[c].i);
    }

    bool in_triangle(int a, int b, int c, int p) const
    {
        const double ax = nodes_[a].x, ay = nodes_[a].y, bx = nodes_[b].x, by = nodes_[b].y;
        const double cx = nodes_[c].x, cy = nodes_[c].y, x = nodes_[p].x, y = nodes_[p].y;
        return (cx - x) * (ay - y) >= (ax - x) * (cy - y) && (ax - x) * (by - y) >= (bx - x) * (ay - y) &&
               (bx - x) * (cy - y) >= (cx - x) * (by - y);
    }
    bool on_segment(int p, int q, int r) const
    {
        const Node &P = nodes_[p], &Q = nodes_[q], &R = nodes_[r];
        return Q.x <= std::max(P.x, R.x) && Q.x >= std::min(P.x, R.x) && Q.y <= std::max(P.y, R.y) &&
               Q.y >= std::min(P.y, R.y);
    }
    bool intersects(int p1, int q1, int p2, int q2) const
    {
        const int o1 = sgn(area(p1, q1, p2)), o2 = sgn(area(p1, q1, q2));
        const int o3 = sgn(area(p2, q2, p1)), o4 = sgn(area(p2, q2, q1));
        if (o1 != o2 && o3 != o4) return true;
        return (o1 == 0 && on_segment(p1, p2, q1)) || (o2 == 0 && on_segment(p1, q2, q1)) ||
               (o3 == 0 && on_segment(p2, p1, q2)) || (o4 == 0 && on_segment(p2, q1, q2));
    }
    bool locally_inside(int a, int b) const
    {
        return area(pv(a), a, nx(a)) < 0 ? area(a, b, nx(a)) >= 0 && area(a, pv(a), b) >= 0
                                         : area(a, b, pv(a)) < 0 || area(a, nx(a), b) < 0;
    }
    bool middle_inside(int a, int b) const
    {
        const double mx = (nodes_[a].x + nodes_[b].x) / 2, my = (nodes_[a].y + nodes_[b].y) / 2;
        bool inside = false;
        int p = a;
        do {
            const Node &P = nodes_[p], &Q = nodes_[nx(p)];
            if (((P.y > my) != (Q.y > my)) && Q.y != P.y && (mx < (Q.x - P.x) * (my - P.y) / (Q.y - P.y) + P.x))
                inside = !inside;
            p = nx(p);
        } while (p != a);
        return inside;
    }
    bool crosses_ring(int a, int b) const
    {
        const uint32_t ia = nodes_[a].i, ib = nodes_[b].i;
        int p = a;
        do {
            const uint32_t ip = nodes_[p].i, iq = nodes_[nx(p)].i;
            if (ip != ia && iq != ia && ip != ib && iq != ib && intersects(p, nx(p), a, b)) return true;
            p = nx(p);
        } while (p != a);
        return false;
    }
    bool valid_diagonal(int a, int b) const
    {
        return nodes_[nx(a)].i != nodes_[b].i && nodes_[pv(a)].i != nodes_[b].i && !crosses_ring(a, b) &&
               ((locally_inside(a, b) && locally_inside(b, a) && middle_inside(a, b) &&
                 (area(pv(a), a, pv(b)) != 0.0 || area(a, pv(b), b) != 0.0)) ||
                (equals(a, b) && area(pv(a), a, nx(a)) > 0 && area(pv(b), b, nx(b)) > 0));
    }
    bool is_ear(int e) const
    {
        const int a = pv(e), c = nx(e);
        if (area(a, e, c) >= 0) return false;            // reflex
        for (int p = nx(c); p != a; p = nx(p))
            if (in_triangle(a, e, c, p) && area(pv(p), p, nx(p)) >= 0) return false;
        return true;
    }
    int filter(int start, int end = -1)
    {
        if (end < 0) end = start;
        int p = start;
        bool again;
        do {
            again = false;
            if (equals(p, nx(p)) || area(pv(p), p, nx(p)) == 0) {
                unlink(p);
                p = end = pv(p);
                if (p == nx(p)) break;
                again = true;
            } else {
                p = nx(p);
            }
        } while (again || p != end);
        return end;
    }
    int cure(int start)
    {
        int p = start;
        do {
            const int a = pv(p), b = nx(nx(p));
            if (!equals(a, b) && intersects(a, p, nx(p), b) && locally_inside(a, b) && locally_inside(b, a)) {
                emit(a, p, b);
                unlink(p);
                unlink(nx(p));
                p = start = b;
            }
            p = nx(p);
        } while (p != start);
        return filter(p);
    }
    int split_ring(int a, int b)
    {
        const int a2 = (int)nodes_.size();
        nodes_.push_back({nodes_[a].i, nodes_[a].x, nodes_[a].y, -1, -1});
        const int b2 = (int)nodes_.size();
        nodes_.push_back({nodes_[b].i, nodes_[b].x, nodes_[b].y, -1, -1});
        const int an = nx(a), bp = pv(b);
        nodes_[a].next = b;
        nodes_[b].prev = a;
        nodes_[a2].next = an;
        nodes_[an].prev = a2;
        nodes_[b2].next = a2;
        nodes_[a2].prev = b2;
        nodes_[bp].next = b2;
        nodes_[b2].prev = bp;
        return b2;
    }
    void split(int start)
    {
        int a = start;
        do {
            for (int b = nx(nx(a)); b != pv(a); b = nx(b)) {
                if (nodes_[a].i != nodes_[b].i && valid_diagonal(a, b)) {
                    int c = split_ring(a, b);
                    a = filter(a, nx(a));
                    c = filter(c, nx(c));
                    slice(a, 0);
                    slice(c, 0);
                    return;
                }
            }
            a = nx(a);
        } while (a != start);
    }
    void slice(int ear, int pass)
    {
        int stop = ear;
        while (pv(ear) != nx(ear)) {
            const int prev = pv(ear), next = nx(ear);
            if (is_ear(ear)) {
                emit(prev, ear, next);
                unlink(ear);
                ear = stop = nx(next);                   // skipping one vertex gives fewer slivers
                continue;
            }
            ear = next;
            if (ear == stop) {
                if (pass == 0) slice(filter(ear), 1);
                else if (pass == 1) slice(cure(filter(ear)), 2);
                else split(ear);
                break;
            }
        }
    }
};

// |shoelace area| of a projected polygon in FP32, trapezoids in vertex order
float projected_area(const float* x, const float* y, size_t n)
{
    float a = 0.f;
    for (size_t i = 1; i != n; ++i) a += (x[i] - x[i - 1]) * ((y[i - 1] + y[i]) / 2);
    a += (x[0] - x[n - 1]) * ((y[0] + y[n - 1]) / 2);
    return std::fabs(a);
}

bool triangulate(const std::vector<float>& raw, const long* poly, size_t n, std::vector<uint32_t>& faces,
                 EarSlicer& slicer)
{
    auto P = [&](long v, int k) { return raw[3 * (size_t)v + k]; };
    if (n == 3) {
        for (size_t k = 0; k < 3; ++k) faces.push_back((uint32_t)poly[k]);
        return true;
    }
    if (n == 4) {
        float d02 = 0.f, d13 = 0.f;
        {
            const float ex = P(poly[0], 0) - P(poly[2], 0), ey = P(poly[0], 1) - P(poly[2], 1),
                        ez = P(poly[0], 2) - P(poly[2], 2);
            const float fx = P(poly[1], 0) - P(poly[3], 0), fy = P(poly[1], 1) - P(poly[3], 1),
                        fz = P(poly[1], 2) - P(poly[3], 2);
            d02 = ex * ex + ey * ey + ez * ez;
            d13 = fx * fx + fy * fy + fz * fz;
        }
        const bool cut02 = d02 < d13;
        const long t[6] = {poly[0], poly[1], cut02 ? poly[2] : poly[3], cut02 ? poly[0] : poly[1], poly[2], poly[3]};
        for (long v : t) faces.push_back((uint32_t)v);
        return true;
    }
    float xs[kMaxPolygon], ys[kMaxPolygon], zs[kMaxPolygon];
    for (size_t k = 0; k < n; ++k) {
        xs[k] = P(poly[k], 0);
        ys[k] = P(poly[k], 1);
        zs[k] = P(poly[k], 2);
    }
    const float ax = projected_area(ys, zs, n), ay = projected_area(xs, zs, n), az = projected_area(xs, ys, n);
    if (std::max(ax, std::max(ay, az)) < FLT_MIN) return false;
    const float *u, *w;
    if (ax > ay) {
        if (ax > az) u = ys, w = zs;
        else u = xs, w = ys;
    } else {
        if (ay > az) u = xs, w = zs;
        else u = xs, w = ys;
    }
    std::vector<double> px(u, u + n), py(w, w + n);
    slicer.run(px, py);
    if (slicer.tri.empty() || slicer.tri.size() % 3) return false;
    for (size_t k = 0; k < slicer.tri.size(); k += 3) {          // the caller flips each triangle
        faces.push_back((uint32_t)poly[slicer.tri[k + 1]]);
        faces.push_back((uint32_t)poly[slicer.tri[k]]);
        faces.push_back((uint32_t)poly[slicer.tri[k + 2]]);
    }
    return true;
}

}  // namespace

// "v x y z ..." and "f i[/t][/n] ..." lines; 1-based or negative (relative
// to the vertices read so far) indices; whether any "vn" line is present.
// Other statements (vt, o, g, s, usemtl, mtllib, l, p, comments) carry
// nothing the physics uses (material libraries are not read: the reference's
// loader rejects a file whose material library is missing, this one reads
// its geometry).  Returns
// false, with a message, on malformed input or a polygon the triangulation
// rejects.
bool parse_obj(const char* text, size_t len, float scale, std::vector<float>& xyz, std::vector<uint32_t>& faces,
               std::string& err)
{
    xyz.clear();
    faces.clear();
    std::vector<long> corners;                 // every face's resolved indices
    std::vector<std::pair<size_t, size_t>> polys;  // (first corner, line)
    size_t pos = 0, line_no = 0;
    bool has_normals = false;
    while (pos < len) {
        size_t end = pos;
        while (end < len && text[end] != '\n' && text[end] != '\r') ++end;
        std::string line(text + pos, end - pos);
        pos = end + 1;
        ++line_no;
        size_t i = 0;
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
        if (i + 1 >= line.size()) continue;
        if (line[i] == 'v' && line[i + 1] == 'n' && i + 2 < line.size() && (line[i + 2] == ' ' || line[i + 2] == '\t'))
            has_normals = true;
        if (line[i] == 'v' && (line[i + 1] == ' ' || line[i + 1] == '\t')) {
            const char* s = line.c_str() + i + 1;
            char* e = nullptr;
            for (int k = 0; k < 3; ++k) {
                const float v = strtof(s, &e);
                if (e == s) {
                    err = "line " + std::to_string(line_no) + ": bad vertex";
                    return false;
                }
                xyz.push_back(v);
                s = e;
            }
        } else if (line[i] == 'f' && (line[i + 1] == ' ' || line[i + 1] == '\t')) {
            const size_t first = corners.size();
            const char* s = line.c_str() + i + 1;
            while (*s) {
                while (*s == ' ' || *s == '\t') ++s;
                if (!*s) break;
                char* e = nullptr;
                const long idx = strtol(s, &e, 10);
                if (e == s || idx == 0) {
                    err = "line " + std::to_string(line_no) + ": bad face index";
                    return false;
                }
                corners.push_back(idx > 0 ? idx - 1 : (long)(xyz.size() / 3) + idx);
                s = e;
                while (*s && *s != ' ' && *s != '\t') ++s;   // skip /t/n
            }
            const size_t n = corners.size() - first;
            if (n < 3 || n > kMaxPolygon) {
                err = "line " + std::to_string(line_no) + ": face with " + std::to_string(n) + " vertices";
                return false;
            }
            polys.push_back({first, line_no});
        }
    }
    const long nv = (long)(xyz.size() / 3);
    for (long c : corners)
        if (c < 0 || c >= nv) {
            err = "face index out of range";
            return false;
        }
    EarSlicer slicer;
    for (size_t p = 0; p < polys.size(); ++p) {
        const size_t first = polys[p].first, last = p + 1 < polys.size() ? polys[p + 1].first : corners.size();
        if (!triangulate(xyz, &corners[first], last - first, faces, slicer)) {
            err = "line " + std::to_string(polys[p].second) + ": polygon cannot be triangulated";
            return false;
        }
    }
    if (faces.empty()) {
        err = "no faces";
        return false;
    }
    if (has_normals)
        for (float& v : xyz) v = scale * v;
    return true;
}

// ---------------------------------------------------------------- Refine
namespace {

struct f3 {
    float x, y, z;
};

f3 vpos(const std::vector<float>& xyz, uint32_t i) { return {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}; }

// PlainMesh::ComputeFaceArea (OpenGLDataStructs.h:219-224): glm, FP32
float face_area(const std::vector<float>& xyz, const uint32_t* f)
{
    const f3 a = vpos(xyz, f[0]), b = vpos(xyz, f[1]), c = vpos(xyz, f[2]);
    const f3 u = {b.x - a.x, b.y - a.y, b.z - a.z}, v = {c.x - a.x, c.y - a.y, c.z - a.z};
    const f3 n = {u.y * v.z - v.y * u.z, u.z * v.x - v.z * u.x, u.x * v.y - v.x * u.y};
    return std::sqrt((n.x * n.x + n.y * n.y) + n.z * n.z) / 2.f;
}

// OpenGLContent::ComputeAverageFaceArea (OpenGLContent.cpp:2779-2785)
float average_area(const std::vector<float>& xyz, const std::vector<uint32_t>& faces)
{
    float a = 0.f;
    for (size_t i = 0; i < faces.size() / 3; ++i) a += face_area(xyz, &faces[3 * i]);
    return a / (float)(faces.size() / 3);
}

}  // namespace

void refine_mesh(std::vector<float>& xyz, std::vector<uint32_t>& faces, float threshold)
{
    const float min_area = 0.01f * 0.01f;
    float avg = std::max(average_area(xyz, faces), min_area);
    for (;;) {
        std::vector<uint32_t> out;
        size_t n_sub = 0;
        for (size_t i = 0; i < faces.size() / 3; ++i) {
            const uint32_t* f = &faces[3 * i];
            if (face_area(xyz, f) > threshold * avg) {
                // the edge lookup is local to the face: every subdivided face
                // gets its own three midpoint vertices (OpenGLContent.cpp:2850-2854)
                uint32_t mid[3];
                for (int e = 0; e < 3; ++e) {
                    const f3 a = vpos(xyz, f[e]), b = vpos(xyz, f[(e + 1) % 3]);
                    mid[e] = (uint32_t)(xyz.size() / 3);
                    xyz.push_back((a.x + b.x) / 2.f);
                    xyz.push_back((a.y + b.y) / 2.f);
                    xyz.push_back((a.z + b.z) / 2.f);
                }
                const uint32_t nf[12] = {f[0], mid[0], mid[2], f[1], mid[1], mid[0],
                                         f[2], mid[2], mid[1], mid[0], mid[1], mid[2]};
                out.insert(out.end(), nf, nf + 12);
                ++n_sub;
            } else {
                out.insert(out.end(), f, f + 3);
            }
        }
        if (n_sub == 0) break;
        faces.swap(out);
        avg = std::max(average_area(xyz, faces), min_area);
    }
}

// ------------------------------------------------------- mass properties
// Per-face terms (GeometryFileUtil.cpp:343-420): pass 0 gives surface,
// CG-weighted volume and volume; pass 1 (vertices relative to the CG) gives
// the six P sums of the inertia tensor.
constexpr int kPropThreads = 128;

__device__ __forceinline__ void d3sub(double* r, const double* a, const double* b)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}

__device__ __forceinline__ void d3cross(double* r, const double* a, const double* b)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ double d3dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

__device__ __forceinline__ double d3len(const double* a) { return sqrt(d3dot(a, a)); }

__device__ void p_terms(const double* v1, const double* v2, const double* v3, double* P)
{
    double c[3];
    d3cross(c, v2, v3);
    const double V6 = d3dot(v1, c);
#define SQ(k) (v1[k] * v1[k] + v2[k] * v2[k] + v3[k] * v3[k] + v1[k] * v2[k] + v1[k] * v3[k] + v2[k] * v3[k])
#define PR(j, k) (2 * (v1[j] * v1[k] + v2[j] * v2[k] + v3[j] * v3[k]) + v1[j] * v2[k] + v1[k] * v2[j] + \
                  v1[j] * v3[k] + v1[k] * v3[j] + v2[j] * v3[k] + v2[k] * v3[j])
    P[0] = V6 * 2 * SQ(0);
    P[1] = V6 * 2 * SQ(1);
    P[2] = V6 * 2 * SQ(2);
    P[3] = V6 * PR(0, 1);
    P[4] = V6 * PR(0, 2);
    P[5] = V6 * PR(1, 2);
#undef SQ
#undef PR
}

// One CTA per tile; out[tile][12]: pass 0 uses 0..4 (surface, CG*V x3,
// volume), pass 1 uses 0..5 (outer P sums) and 6..11 (inner, shells).
__global__ void mesh_props_kernel(const TileDesc* __restrict__ tiles, uint32_t first_tile, int pass, double thickness,
                                  double3 cg, double* __restrict__ out)
{
    __shared__ double red[12][kPropThreads];
    const TileDesc td = tiles[first_tile + blockIdx.x];
    const int nv = td.nv, nvp = (nv + 3) & ~3;
    const float* x = reinterpret_cast<const float*>(td.block);
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(x + 3 * nvp);
    double acc[12];
    for (int k = 0; k < 12; ++k) acc[k] = 0.0;
    const double C[3] = {cg.x, cg.y, cg.z};
    for (int f = threadIdx.x; f < td.nf; f += kPropThreads) {
        const uint32_t w = idx[f];
        const uint32_t i[3] = {w & 511u, (w >> 9) & 511u, w >> 18};
        double v[3][3];
        for (int a = 0; a < 3; ++a) {
            v[a][0] = (double)x[i[a]];
            v[a][1] = (double)x[nvp + i[a]];
            v[a][2] = (double)x[2 * nvp + i[a]];
        }
        double e1[3], e2[3], n[3];
        d3sub(e1, v[1], v[0]);
        d3sub(e2, v[2], v[0]);
        d3cross(n, e1, e2);
        if (pass == 0) {
            const double A = d3len(n) / 2.0;
            if (thickness > 0.0) {                                   // shell (:343-367)
                const double V = A * thickness;
                acc[0] += A;
                // btVector3 / s multiplies by 1 / s
                for (int k = 0; k < 3; ++k) acc[1 + k] += ((v[0][k] + v[1][k]) + v[2][k]) * (1.0 / 3.0) * V;
                acc[4] += V;
            } else {                                                 // solid (:369-394)
                acc[0] += A;
                double c[3];
                d3cross(c, v[1], v[2]);
                const double V6 = d3dot(v[0], c);
                for (int k = 0; k < 3; ++k) acc[1 + k] += ((v[0][k] + v[1][k]) + v[2][k]) * 0.25 * V6;
                acc[4] += V6;
            }
        } else {
            if (thickness > 0.0) {                                   // :400-488
                const double il = 1.0 / d3len(n);                   // btVector3::normalize
                const double u[3] = {n[0] * il, n[1] * il, n[2] * il};
                double o[3][3], in[3][3], P[6];
                for (int a = 0; a < 3; ++a)
                    for (int k = 0; k < 3; ++k) {
                        o[a][k] = v[a][k] + u[k] * thickness / 2.0 - C[k];
                        in[a][k] = v[a][k] - u[k] * thickness / 2.0 - C[k];
                    }
                p_terms(o[0], o[1], o[2], P);
                for (int k = 0; k < 6; ++k) acc[k] += P[k];
                p_terms(in[0], in[1], in[2], P);
                for (int k = 0; k < 6; ++k) acc[6 + k] += P[k];
            } else {                                                 // :490-520
                double r[3][3], P[6];
                for (int a = 0; a < 3; ++a)
                    for (int k = 0; k < 3; ++k) r[a][k] = v[a][k] - C[k];
                p_terms(r[0], r[1], r[2], P);
                for (int k = 0; k < 6; ++k) acc[k] += P[k];
            }
        }
    }
    for (int k = 0; k < 12; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = kPropThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 12; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 12) out[(size_t)blockIdx.x * 12 + threadIdx.x] = red[threadIdx.x][0];
}

cudaError_t launch_mesh_props(const TileDesc* tiles, uint32_t first_tile, uint32_t n_tiles, int pass, double thickness,
                              double3 cg, double* out, cudaStream_t s)
{
    if (n_tiles == 0) return cudaSuccess;
    mesh_props_kernel<<<n_tiles, kPropThreads, 0, s>>>(tiles, first_tile, pass, thickness, cg, out);
    return cudaGetLastError();
}

// --------------------------------------------------- principal axes (host)
namespace {

struct M3 {
    double m[3][3];
};

double det3(const M3& a)
{
    return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) -
           a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]) +
           a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}

void cross3(const double* a, const double* b, double* r)
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

double len2(const double* a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }

// FindInertialAxis (GeometryFileUtil.cpp:576-606)
void inertial_axis(const M3& I, double value, double* axis)
{
    M3 L = I;
    for (int k = 0; k < 3; ++k) L.m[k][k] -= value;
    double c[3][3];
    cross3(L.m[0], L.m[1], c[0]);
    cross3(L.m[0], L.m[2], c[1]);
    cross3(L.m[1], L.m[2], c[2]);
    int best;
    if (len2(c[0]) >= len2(c[1])) best = len2(c[0]) >= len2(c[2]) ? 0 : 2;
    else best = len2(c[1]) >= len2(c[2]) ? 1 : 2;
    const double il = 1.0 / std::sqrt(len2(c[best]));              // normalized(): times 1 / length
    for (int k = 0; k < 3; ++k) axis[k] = c[best][k] * il;
}

// IsDiagonal (GeometryFileUtil.cpp:608-625)
bool is_diagonal(const M3& A)
{
    const double mn = std::min(std::min(std::fabs(A.m[0][0]), std::fabs(A.m[1][1])), std::fabs(A.m[2][2]));
    const double d = mn / 1e6;
    return std::fabs(A.m[0][1]) < d && std::fabs(A.m[0][2]) < d && std::fabs(A.m[1][0]) < d &&
           std::fabs(A.m[1][2]) < d && std::fabs(A.m[2][0]) < d && std::fabs(A.m[2][1]) < d;
}

}  // namespace

// Mass, inertia tensor and principal axes from the summed terms
// (GeometryFileUtil.cpp:395-566).
void finish_properties(double thickness, double density, const double* s0, const double* s1,
                       hydro_mesh_properties* out)
{
    double volume = s0[4];
    double cg[3] = {s0[1], s0[2], s0[3]};
    if (volume > 0.0) {
        const double iv = 1.0 / volume;                              // btVector3 /= multiplies by 1 / s
        for (int k = 0; k < 3; ++k) cg[k] *= iv;
    } else {
        cg[0] = cg[1] = cg[2] = 0.0;
    }
    if (!(thickness > 0.0)) volume /= 6.0;
    out->volume = volume;
    out->surface = s0[0];
    for (int k = 0; k < 3; ++k) out->CG[k] = cg[k];
    out->mass = volume * density;
    auto tensor = [&](const double* P) {
        const double k = density / 120.0;
        const double xx = P[0] * k, yy = P[1] * k, zz = P[2] * k, xy = P[3] * k, xz = P[4] * k, yz = P[5] * k;
        M3 I = {{{yy + zz, -xy, -xz}, {-xy, xx + zz, -yz}, {-xz, -yz, xx + yy}}};
        return I;
    };
    M3 I = tensor(s1);
    if (thickness > 0.0) {
        const M3 Ii = tensor(s1 + 6);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) I.m[r][c] -= Ii.m[r][c];
    }
    out->Ipri[0] = I.m[0][0];
    out->Ipri[1] = I.m[1][1];
    out->Ipri[2] = I.m[2][2];
    for (int k = 0; k < 9; ++k) out->Irot[k] = (k % 4 == 0) ? 1.0 : 0.0;
    if (!is_diagonal(I)) {                                           // :524-554
        const double T = I.m[0][0] + I.m[1][1] + I.m[2][2];
        const double II = I.m[0][0] * I.m[1][1] + I.m[0][0] * I.m[2][2] + I.m[1][1] * I.m[2][2] -
                          I.m[0][1] * I.m[0][1] - I.m[0][2] * I.m[0][2] - I.m[1][2] * I.m[1][2];
        const double U = std::sqrt(T * T - 3.0 * II) / 3.0;
        double ac = (-2.0 * T * T * T + 9.0 * T * II - 27.0 * det3(I)) / (54.0 * U * U * U);
        ac = std::min(1.0, std::max(-1.0, ac));                      // btAcos clamps
        const double theta = std::acos(ac);
        const double pi = 3.14159265358979323846;
        const double A = T / 3.0 - 2.0 * U * std::cos(theta / 3.0);
        const double B = T / 3.0 - 2.0 * U * std::cos(theta / 3.0 - 2.0 * pi / 3.0);
        const double Cc = T / 3.0 - 2.0 * U * std::cos(theta / 3.0 + 2.0 * pi / 3.0);
        out->Ipri[0] = A;
        out->Ipri[1] = B;
        out->Ipri[2] = Cc;
        double a1[3], a2[3], a3[3];
        inertial_axis(I, A, a1);
        inertial_axis(I, B, a2);
        cross3(a1, a2, a3);
        cross3(a3, a1, a2);
        const double R[9] = {a1[0], a2[0], a3[0], a1[1], a2[1], a3[1], a1[2], a2[2], a3[2]};
        for (int k = 0; k < 9; ++k) out->Irot[k] = R[k];
    }
}

}  // namespace sfh
