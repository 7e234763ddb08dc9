// hydro_approx.cu -- per-body coefficient setup of the hydrodynamics path:
// SolidEntity::ComputeFluidDynamicsApprox (Library/src/entities/SolidEntity.cpp:
// 698-718) and the three proxy shapes it fits to the physics mesh, sphere
// (:720-758), cylinder (:760-847) and axis-aligned ellipsoid (:849-1025, with
// LambKFactor :1027-1039).  They give the form and skin-friction
// coefficients fdCd / fdCf that CorrectHydrodynamicForces applies every step
// (hydro_body.Cd / Cf), the proxy frame T_CG2H that the aerodynamic
// correction reads, and the added mass and inertia of the body.
//
// Host code: the reference runs this once per body when the body is built,
// on the CPU; it is FP64 throughout.  The vector and matrix arithmetic keeps
// the operation order of the reference's Bullet types (BT_USE_DOUBLE_PRECISION,
// no SIMD), so the results are the reference's bits:
//   a.dot(b)          = (a.x*b.x + a.y*b.y) + a.z*b.z
//   T * p             = (row_r . p) + origin_r
//   M * v             = (row_0 . v, row_1 . v, row_2 . v)
//   (A * B)[i][j]     = (B[0][j]*A[i][0] + B[1][j]*A[i][1]) + B[2][j]*A[i][2]
//   M.inverse()       = cofactors times 1/det, det = row_0 . cofactors
//   v /= s            = v * (1/s)
//   Quaternion(yaw, pitch, roll) with BT_EULER_DEFAULT_ZYX, then the rotation
//   matrix of a quaternion with s = 2/|q|^2.
// The ellipsoid fit (minimum-volume enclosing axis-aligned ellipsoid,
// Kumar & Yildirim, J Optim Theory Appl 136 (2008) 211-228) evaluates the
// weighted sums u_j and v_j once per iteration instead of once per point:
// each is the same sum over the same points in the same order, so the
// result is unchanged and the fit costs O(N) per iteration instead of O(N^2).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "hydro_internal.h"

namespace {

struct V3 {
    double x, y, z;
    double operator[](int i) const { return i == 0 ? x : i == 1 ? y : z; }
};

inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline bool same(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

struct M3 {
    double m[3][3];
    V3 row(int r) const { return {m[r][0], m[r][1], m[r][2]}; }
};

M3 identity()
{
    M3 r{};
    r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0;
    return r;
}

M3 from_rows(const double* b)
{
    M3 r;
    for (int i = 0; i < 9; ++i) r.m[i / 3][i % 3] = b[i];
    return r;
}

V3 mul(const M3& a, V3 v) { return {dot(a.row(0), v), dot(a.row(1), v), dot(a.row(2), v)}; }

M3 mul(const M3& a, const M3& b)
{
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = b.m[0][j] * a.m[i][0] + b.m[1][j] * a.m[i][1] + b.m[2][j] * a.m[i][2];
    return r;
}

double cofac(const M3& a, int r1, int c1, int r2, int c2) { return a.m[r1][c1] * a.m[r2][c2] - a.m[r1][c2] * a.m[r2][c1]; }

M3 inverse(const M3& a)
{
    V3 co{cofac(a, 1, 1, 2, 2), cofac(a, 1, 2, 2, 0), cofac(a, 1, 0, 2, 1)};
    double s = 1.0 / dot(a.row(0), co);
    M3 r;
    r.m[0][0] = co.x * s;
    r.m[0][1] = cofac(a, 0, 2, 2, 1) * s;
    r.m[0][2] = cofac(a, 0, 1, 1, 2) * s;
    r.m[1][0] = co.y * s;
    r.m[1][1] = cofac(a, 0, 0, 2, 2) * s;
    r.m[1][2] = cofac(a, 0, 2, 1, 0) * s;
    r.m[2][0] = co.z * s;
    r.m[2][1] = cofac(a, 0, 1, 2, 0) * s;
    r.m[2][2] = cofac(a, 0, 0, 1, 1) * s;
    return r;
}

// Rotation of the quaternion built from Euler angles (yaw about z, pitch
// about y, roll about x), as Quaternion(yaw, pitch, roll) does with
// BT_EULER_DEFAULT_ZYX, then turned into a basis.
M3 euler_zyx_basis(double yaw, double pitch, double roll)
{
    const double hy = yaw * 0.5, hp = pitch * 0.5, hr = roll * 0.5;
    const double cy = std::cos(hy), sy = std::sin(hy), cp = std::cos(hp), sp = std::sin(hp);
    const double cr = std::cos(hr), sr = std::sin(hr);
    const double qx = sr * cp * cy - cr * sp * sy;
    const double qy = cr * sp * cy + sr * cp * sy;
    const double qz = cr * cp * sy - sr * sp * cy;
    const double qw = cr * cp * cy + sr * sp * sy;
    const double d = qx * qx + qy * qy + qz * qz + qw * qw;
    const double s = 2.0 / d;
    const double xs = qx * s, ys = qy * s, zs = qz * s;
    const double wx = qw * xs, wy = qw * ys, wz = qw * zs;
    const double xx = qx * xs, xy = qx * ys, xz = qx * zs;
    const double yy = qy * ys, yz = qy * zs, zz = qz * zs;
    M3 r;
    r.m[0][0] = 1.0 - (yy + zz);
    r.m[0][1] = xy - wz;
    r.m[0][2] = xz + wy;
    r.m[1][0] = xy + wz;
    r.m[1][1] = 1.0 - (xx + zz);
    r.m[1][2] = yz - wx;
    r.m[2][0] = xz - wy;
    r.m[2][1] = yz + wx;
    r.m[2][2] = 1.0 - (xx + yy);
    return r;
}

struct Fit {
    int type;
    int n_params;
    double params[3];
    M3 R_CG2H;
    V3 added_mass, added_inertia, Cd;
};

// Sphere: radius^2 of the farthest vertex (the reference keeps the squared
// radius in the added-mass formula, :737-746).
Fit sphere(const std::vector<V3>& x, double rho)
{
    double r = 0.0;
    for (const V3& p : x) {
        const double rc = dot(p, p);
        if (rc > r) r = rc;
    }
    Fit f{};
    f.type = HYDRO_APPROX_SPHERE;
    f.n_params = 1;
    f.params[0] = std::sqrt(r);
    const double m = 2.0 * M_PI * rho * r * r * r / 3.0;
    f.added_mass = {m, m, m};
    f.added_inertia = {0.0, 0.0, 0.0};
    f.R_CG2H = identity();
    f.Cd = {1.0, 1.0, 1.0};
    return f;
}

Fit cylinder(const std::vector<V3>& x, double rho, const M3& R_CG2O)
{
    double r[3] = {0.0, 0.0, 0.0};
    for (const V3& p : x) {
        double d = std::sqrt(p.y * p.y + p.z * p.z);
        r[0] = d > r[0] ? d : r[0];
        d = std::sqrt(p.x * p.x + p.z * p.z);
        r[1] = d > r[1] ? d : r[1];
        d = std::sqrt(p.x * p.x + p.y * p.y);
        r[2] = d > r[2] ? d : r[2];
    }
    int axis;
    if (r[0] <= r[1] && r[0] <= r[2])
        axis = 0;
    else if (r[1] <= r[0] && r[1] <= r[2])
        axis = 1;
    else
        axis = 2;
    double l_2 = 0.0;
    for (const V3& p : x) {
        const double d = std::fabs(p[axis]);
        l_2 = d > l_2 ? d : l_2;
    }
    Fit f{};
    f.type = HYDRO_APPROX_CYLINDER;
    f.n_params = 2;
    f.params[0] = r[axis];
    f.params[1] = l_2 * 2.0;
    if (axis == 0)
        f.R_CG2H = euler_zyx_basis(0.0, M_PI_2, 0.0);
    else if (axis == 1)
        f.R_CG2H = euler_zyx_basis(0.0, 0.0, M_PI_2);
    else
        f.R_CG2H = identity();
    const double p0 = f.params[0], p1 = f.params[1];
    const double m1 = rho * M_PI * p0 * p0;
    const double m2 = rho * M_PI * p0 * p0 * p1;
    const double I1 = 0.0;
    const double I2 = 1.0 / 12.0 * M_PI * rho * p1 * p1 * std::pow(p0, 3.0);
    f.added_mass = vabs(mul(f.R_CG2H, V3{m2, m2, m1}));
    f.added_inertia = vabs(mul(f.R_CG2H, V3{I2, I2, I1}));
    f.Cd = vabs(mul(mul(inverse(R_CG2O), f.R_CG2H), V3{0.5, 0.5, 1.0}));
    return f;
}

double lamb_k_factor(double r1, double r2)
{
    const double e = 1.0 - r2 * r2 / r1;
    const double elog = (1.0 + e) / (1.0 - e);
    if (elog > 0.0) {
        const double alpha0 = 2.0 * (1.0 - e * e) / (e * e) * (0.5 * std::log((1.0 + e) / (1.0 - e)) - e);
        return alpha0 / (2.0 - alpha0);
    }
    return 1.0;
}

Fit ellipsoid(const std::vector<V3>& x, double rho, const M3& R_CG2O)
{
    const size_t n = x.size();
    // Initial core set: per axis the first smallest and the last largest
    // coordinate (std::minmax_element's rule).
    V3 x0[6];
    for (int k = 0; k < 3; ++k) {
        size_t lo = 0, hi = 0;
        for (size_t i = 1; i < n; ++i) {
            if (x[i][k] < x[lo][k]) lo = i;
            if (!(x[i][k] < x[hi][k])) hi = i;
        }
        x0[2 * k] = x[lo];
        x0[2 * k + 1] = x[hi];
    }
    std::vector<double> sigma(n, 0.0);
    for (size_t i = 0; i < n; ++i)
        for (const V3& c : x0)
            if (same(c, x[i])) {
                sigma[i] = 1.0 / 6.0;
                break;
            }
    double u[3], v[3];
    auto sums = [&]() {
        for (int j = 0; j < 3; ++j) {
            double su = 0.0, sv = 0.0;
            for (size_t i = 0; i < n; ++i) {
                su += sigma[i] * x[i][j] * x[i][j];
                sv += sigma[i] * x[i][j];
            }
            u[j] = su;
            v[j] = sv;
        }
    };
    auto lambda = [&](size_t i) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s += (x[i][j] - v[j]) * (x[i][j] - v[j]) / (3 * (u[j] - v[j] * v[j]));
        return s;
    };
    auto argmax = [&]() {       // first index of the largest lambda
        size_t best = 0;
        double bv = lambda(0);
        for (size_t i = 1; i < n; ++i) {
            const double l = lambda(i);
            if (bv < l) {
                bv = l;
                best = i;
            }
        }
        return best;
    };
    sums();
    size_t i_star = argmax();
    double epsilon = lambda(i_star) - 1.0;
    const double epsilon_tol = std::pow(1.0 + 0.2, 2.0 / 3.0) - 1.0;
    const size_t max_iter = 10;
    size_t k = 0;
    while (epsilon > epsilon_tol && k < max_iter) {
        const double beta = epsilon / (double(3 + 1) * (1.0 + epsilon));
        for (size_t i = 0; i < n; ++i) sigma[i] = (1.0 - beta) * sigma[i];
        sigma[i_star] += beta;
        sums();
        i_star = argmax();
        epsilon = lambda(i_star) - 1.0;
        ++k;
    }
    V3 d;
    if (k == 0) {
        const V3 c{(x0[0].x + x0[1].x) / 2.0, (x0[2].y + x0[3].y) / 2.0, (x0[4].z + x0[5].z) / 2.0};
        d = {std::fabs(x0[0].x - c.x), std::fabs(x0[2].y - c.y), std::fabs(x0[4].z - c.z)};
    } else {
        double dd[3];
        for (int j = 0; j < 3; ++j) {
            dd[j] = 1.0 / (3.0 * (u[j] - v[j] * v[j]));
            dd[j] = 1.0 / std::sqrt(dd[j]);
        }
        d = {dd[0], dd[1], dd[2]};
    }
    Fit f{};
    f.type = HYDRO_APPROX_ELLIPSOID;
    f.n_params = 3;
    f.params[0] = d.x;
    f.params[1] = d.y;
    f.params[2] = d.z;
    const double r12 = (d.y + d.z) / 2.0;
    f.added_mass = {lamb_k_factor(d.x, r12) * 4.0 / 3.0 * M_PI * rho * d.x * r12 * r12,
                    4.0 / 3.0 * M_PI * rho * d.z * d.z * d.x, 4.0 / 3.0 * M_PI * rho * d.y * d.y * d.x};
    f.added_inertia = {0.0, 1.0 / 12.0 * M_PI * rho * d.y * d.y * std::pow(d.x, 3.0),
                       1.0 / 12.0 * M_PI * rho * d.z * d.z * std::pow(d.x, 3.0)};
    f.R_CG2H = identity();
    V3 cd{1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
    const double max_cd = std::max(std::max(cd.x, cd.y), cd.z);
    cd = scale(cd, 1.0 / max_cd);
    f.Cd = vabs(mul(inverse(R_CG2O), cd));
    return f;
}

}  // namespace

extern "C" hydro_status hydro_fluid_approx(const void* vertex_data, size_t vertex_stride, uint32_t n_vertices,
                                           int32_t approx_type, const hydro_transform* T_CG2C,
                                           const hydro_transform* T_CG2O, const double P_CB[3], double density,
                                           hydro_fluid_approx_result* out)
{
    if (vertex_data == nullptr || T_CG2C == nullptr || T_CG2O == nullptr || P_CB == nullptr || out == nullptr ||
        vertex_stride < 3 * sizeof(float) || n_vertices < 2 || approx_type < HYDRO_APPROX_AUTO ||
        approx_type > HYDRO_APPROX_ELLIPSOID || !(density > 0.0))
        return HYDRO_ERR_INVALID_ARG;
    // Points in the CG frame about the centre of buoyancy: T_CG2C * p - P_CB
    // (getMeshVertices, SolidEntity.cpp:683-696, then :724-725).
    const M3 R = from_rows(T_CG2C->basis);
    const V3 o{T_CG2C->origin[0], T_CG2C->origin[1], T_CG2C->origin[2]};
    const V3 cb{P_CB[0], P_CB[1], P_CB[2]};
    std::vector<V3> x(n_vertices);
    const unsigned char* base = static_cast<const unsigned char*>(vertex_data);
    for (uint32_t i = 0; i < n_vertices; ++i) {
        float p[3];
        std::memcpy(p, base + (size_t)i * vertex_stride, sizeof(p));
        const V3 q{(double)p[0], (double)p[1], (double)p[2]};
        const V3 t{dot(q, R.row(0)) + o.x, dot(q, R.row(1)) + o.y, dot(q, R.row(2)) + o.z};
        x[i] = sub(t, cb);
    }
    const M3 R_CG2O = from_rows(T_CG2O->basis);
    Fit f;
    if (approx_type == HYDRO_APPROX_SPHERE)
        f = sphere(x, density);
    else if (approx_type == HYDRO_APPROX_CYLINDER)
        f = cylinder(x, density, R_CG2O);
    else
        f = ellipsoid(x, density, R_CG2O);
    out->approx_type = f.type;
    out->n_params = f.n_params;
    for (int i = 0; i < 3; ++i) out->params[i] = i < f.n_params ? f.params[i] : 0.0;
    for (int i = 0; i < 9; ++i) out->T_CG2H.basis[i] = f.R_CG2H.m[i / 3][i % 3];
    out->T_CG2H.origin[0] = cb.x;
    out->T_CG2H.origin[1] = cb.y;
    out->T_CG2H.origin[2] = cb.z;
    const V3* src[4] = {&f.added_mass, &f.added_inertia, &f.Cd, nullptr};
    double* dst[3] = {out->added_mass, out->added_inertia, out->Cd};
    for (int k = 0; k < 3; ++k) {
        dst[k][0] = src[k]->x;
        dst[k][1] = src[k]->y;
        dst[k][2] = src[k]->z;
    }
    const V3 cf = scale(f.Cd, 0.1);  // Scalar(0.1) * Cd
    out->Cf[0] = cf.x;
    out->Cf[1] = cf.y;
    out->Cf[2] = cf.z;
    return HYDRO_OK;
}
