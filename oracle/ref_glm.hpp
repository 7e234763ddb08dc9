/*
 * ref_glm.hpp -- the few glm types and functions that Stonefish's hydrodynamics
 * path calls, restated from glm's published semantics (glm >= 0.9.9, MIT
 * licence; the reference names it as a system dependency, README
 * "libglm-dev >= 0.9.9.0", and does not vendor it).
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/build_ref.py to compile the
 * reference's own hydrodynamics functions on the CPU.  Nothing in the
 * library includes it.
 *
 * Semantics kept (glm's scalar code path, no SIMD: Stonefish does not define
 * GLM_FORCE_INTRINSICS):
 *   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z     (component product, then x+y+z)
 *   cross(a, b)  = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
 *   length2(v)   = dot(v, v);  length(v) = sqrt(dot(v, v))
 *   normalize(v) = v * (1 / sqrt(dot(v, v)))
 *   mat4 * vec4  = (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w), column by column
 *   vec / s      = per-component division;  s * vec = per-component s*v_i
 *   vec3::length() is the component count 3 (glm's length_t), not the norm.
 */
#ifndef REF_GLM_HPP
#define REF_GLM_HPP

#include <cmath>

namespace glm {

typedef int length_t;

struct vec3;

struct vec4 {
    float x, y, z, w;
    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    inline vec4(const vec3& v, float d);
    float& operator[](length_t i) { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
    float operator[](length_t i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
};

inline vec4 operator*(const vec4& a, const vec4& b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

struct vec3 {
    float x, y, z;
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}
    static constexpr length_t length() { return 3; }
    float& operator[](length_t i) { return i == 0 ? x : i == 1 ? y : z; }
    float operator[](length_t i) const { return i == 0 ? x : i == 1 ? y : z; }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
    bool operator==(const vec3& o) const { return x == o.x && y == o.y && z == o.z; }
};

inline vec4::vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}

struct vec2 {
    float x, y;
    vec2() : x(0.f), y(0.f) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const vec3& v) : x(v.x), y(v.y) {}  /* glm converts vec3 -> vec2 implicitly */
    bool operator==(const vec2& o) const { return x == o.x && y == o.y; }
};
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
/* vec3 * length_t (the aerodynamic term's vn * vn.length()): the integer is
 * converted to float first. */
inline vec3 operator*(const vec3& a, length_t n) { return a * static_cast<float>(n); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

inline float dot(const vec3& a, const vec3& b)
{
    vec3 t = a * b;
    return t.x + t.y + t.z;
}
inline vec3 cross(const vec3& a, const vec3& b)
{
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length2(const vec3& v) { return dot(v, v); }
inline float sqrt(float s) { return std::sqrt(s); }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v * (1.f / std::sqrt(dot(v, v))); }

struct mat4 {
    vec4 c[4];
    mat4() {}
    mat4(float x0, float y0, float z0, float w0, float x1, float y1, float z1, float w1,
         float x2, float y2, float z2, float w2, float x3, float y3, float z3, float w3)
    {
        c[0] = vec4(x0, y0, z0, w0);
        c[1] = vec4(x1, y1, z1, w1);
        c[2] = vec4(x2, y2, z2, w2);
        c[3] = vec4(x3, y3, z3, w3);
    }
    vec4& operator[](length_t i) { return c[i]; }
    const vec4& operator[](length_t i) const { return c[i]; }
};

inline vec4 operator*(const mat4& m, const vec4& v)
{
    vec4 add0 = m[0] * vec4(v[0]) + m[1] * vec4(v[1]);
    vec4 add1 = m[2] * vec4(v[2]) + m[3] * vec4(v[3]);
    return add0 + add1;
}

}  // namespace glm

#endif
