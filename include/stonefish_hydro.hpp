/*
 * stonefish_hydro.hpp -- header-only C++ layer over stonefish_hydro.h with
 * the call signatures of Stonefish's three static hydrodynamics functions
 * (Library/include/entities/SolidEntity.h:113-153):
 *
 *   ComputeHydrodynamicForcesSurface(settings, mesh, ocean, T_CG, T_C, v, omega,
 *                                    Fb, Tb, Fdq, Tdq, Fdf, Tdf, Swet, Vsub, debug)
 *   ComputeHydrodynamicForcesSubmerged(mesh, ocean, T_CG, T_C, v, omega,
 *                                      Fdq, Tdq, Fdf, Tdf)
 *   CorrectHydrodynamicForces(ocean, Fdq, Tdq, Fdf, Tdf, Cd, Cf, T_O)
 *
 * so that the reference's call sites (SolidEntity.cpp:1822-1848,
 * Compound.cpp:347-429) can call the GPU library unchanged.  The functions
 * are templates over the caller's types, which need only Bullet's accessors:
 *   Transform  getBasis()[r][c] (or getBasis().getRow(r)[c]), getOrigin()[i]
 *   Vector3    operator[](i) const, setValue(x, y, z)
 *   Scalar     assignable from double
 *   Settings   members dampingForces, reallisticBuoyancy (Ocean.h:36-40)
 *   Mesh       getVertexDataPointer(), getVertexSize(), getNumOfVertices(),
 *              getFaceDataPointer(), faces.size() (OpenGLDataStructs.h:170-190)
 * so btTransform / btVector3 / btScalar and the reference's Mesh types work
 * as they are.  The ocean is passed as a hydro_ocean, which the caller fills
 * from its Ocean once per tick (density, gravity, waves, currents).
 *
 * A HydroStatics object owns the link to one hydro_ctx and uploads each
 * mesh on its first use, keyed by the Mesh pointer (the reference's meshes
 * do not change after they are built).  Like the reference, the functions
 * return nothing and never throw: a failing call leaves the outputs as they
 * were, and status() / last_error() report it.  The `debug` Renderable of
 * ComputeHydrodynamicForcesSurface is accepted and left untouched (the
 * reference fills it only under DEBUG_HYDRO).
 */
#ifndef STONEFISH_HYDRO_HPP
#define STONEFISH_HYDRO_HPP

#include <cstdint>
#include <mutex>
#include <unordered_map>

#include "stonefish_hydro.h"

namespace stonefish_gb300 {

/* btTransform -> hydro_transform (basis rows, then origin). */
template <class Transform>
hydro_transform to_hydro(const Transform& T)
{
    hydro_transform t;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t.basis[3 * r + c] = static_cast<double>(T.getBasis()[r][c]);
    for (int i = 0; i < 3; ++i) t.origin[i] = static_cast<double>(T.getOrigin()[i]);
    return t;
}

template <class Vector3>
void to_array(const Vector3& v, double out[3])
{
    for (int i = 0; i < 3; ++i) out[i] = static_cast<double>(v[i]);
}

template <class Vector3>
void from_array(const double in[3], Vector3& v)
{
    v.setValue(in[0], in[1], in[2]);
}

class HydroStatics {
public:
    explicit HydroStatics(hydro_ctx* ctx) : ctx_(ctx) {}

    hydro_status status() const { return status_; }
    const char* last_error() const { return hydro_last_error(ctx_); }
    hydro_ctx* context() const { return ctx_; }

    /* The id of a reference mesh, uploaded on first use; HYDRO_NO_MESH for
     * nullptr or when the upload fails (status() tells which). */
    template <class Mesh>
    hydro_mesh_id mesh_id(const Mesh* mesh)
    {
        if (mesh == nullptr) return HYDRO_NO_MESH;
        std::lock_guard<std::mutex> lk(mu_);
        auto it = ids_.find(static_cast<const void*>(mesh));
        if (it != ids_.end()) return it->second;
        hydro_mesh_id id = HYDRO_NO_MESH;
        status_ = hydro_mesh_upload(ctx_, mesh->getVertexDataPointer(), mesh->getVertexSize(),
                                    static_cast<uint32_t>(mesh->getNumOfVertices()),
                                    static_cast<const uint32_t*>(mesh->getFaceDataPointer()),
                                    static_cast<uint32_t>(mesh->faces.size()), &id);
        if (status_ != HYDRO_OK) return HYDRO_NO_MESH;
        ids_.emplace(static_cast<const void*>(mesh), id);
        return id;
    }

    /* SolidEntity::ComputeHydrodynamicForcesSurface (SolidEntity.cpp:1289-1721). */
    template <class Settings, class Mesh, class Transform, class Vector3, class Scalar, class Renderable>
    void ComputeHydrodynamicForcesSurface(const Settings& settings, const Mesh* mesh, const hydro_ocean* ocn,
                                          const Transform& T_CG, const Transform& T_C, const Vector3& _v,
                                          const Vector3& _omega, Vector3& _Fb, Vector3& _Tb, Vector3& _Fdq,
                                          Vector3& _Tdq, Vector3& _Fdf, Vector3& _Tdf, Scalar& _Swet,
                                          Scalar& _Vsub, Renderable& debug)
    {
        (void)debug;
        const hydro_mesh_id id = mesh_id(mesh);
        if (mesh != nullptr && id == HYDRO_NO_MESH) return;
        const hydro_settings s = {settings.dampingForces ? 1 : 0, settings.reallisticBuoyancy ? 1 : 0};
        const hydro_transform tcg = to_hydro(T_CG), tc = to_hydro(T_C);
        double v[3], w[3], Fb[3], Tb[3], Fdq[3], Tdq[3], Fdf[3], Tdf[3];
        to_array(_v, v);
        to_array(_omega, w);
        to_array(_Fb, Fb);
        to_array(_Tb, Tb);
        to_array(_Fdq, Fdq);
        to_array(_Tdq, Tdq);
        to_array(_Fdf, Fdf);
        to_array(_Tdf, Tdf);
        double swet = static_cast<double>(_Swet), vsub = static_cast<double>(_Vsub);
        status_ = hydro_surface_forces(ctx_, &s, id, ocn, &tcg, &tc, v, w, Fb, Tb, Fdq, Tdq, Fdf, Tdf, &swet, &vsub);
        if (status_ != HYDRO_OK) return;
        from_array(Fb, _Fb);
        from_array(Tb, _Tb);
        from_array(Fdq, _Fdq);
        from_array(Tdq, _Tdq);
        from_array(Fdf, _Fdf);
        from_array(Tdf, _Tdf);
        _Swet = swet;
        _Vsub = vsub;
    }

    /* SolidEntity::ComputeHydrodynamicForcesSubmerged (SolidEntity.cpp:1723-1797). */
    template <class Mesh, class Transform, class Vector3>
    void ComputeHydrodynamicForcesSubmerged(const Mesh* mesh, const hydro_ocean* ocn, const Transform& T_CG,
                                            const Transform& T_C, const Vector3& _v, const Vector3& _omega,
                                            Vector3& _Fdq, Vector3& _Tdq, Vector3& _Fdf, Vector3& _Tdf)
    {
        const hydro_mesh_id id = mesh_id(mesh);
        if (mesh != nullptr && id == HYDRO_NO_MESH) return;
        const hydro_transform tcg = to_hydro(T_CG), tc = to_hydro(T_C);
        double v[3], w[3], Fdq[3], Tdq[3], Fdf[3], Tdf[3];
        to_array(_v, v);
        to_array(_omega, w);
        status_ = hydro_submerged_forces(ctx_, id, ocn, &tcg, &tc, v, w, Fdq, Tdq, Fdf, Tdf);
        if (status_ != HYDRO_OK) return;
        from_array(Fdq, _Fdq);
        from_array(Tdq, _Tdq);
        from_array(Fdf, _Fdf);
        from_array(Tdf, _Tdf);
    }

    /* SolidEntity::CorrectHydrodynamicForces (SolidEntity.cpp:1263-1287). */
    template <class Vector3, class Transform>
    void CorrectHydrodynamicForces(const hydro_ocean* ocn, Vector3& _Fdq, Vector3& _Tdq, Vector3& _Fdf,
                                   Vector3& _Tdf, const Vector3& fdCd, const Vector3& fdCf, const Transform& T_O)
    {
        double Fdq[3], Tdq[3], Fdf[3], Tdf[3], cd[3], cf[3];
        to_array(_Fdq, Fdq);
        to_array(_Tdq, Tdq);
        to_array(_Fdf, Fdf);
        to_array(_Tdf, Tdf);
        to_array(fdCd, cd);
        to_array(fdCf, cf);
        const hydro_transform to = to_hydro(T_O);
        status_ = hydro_correct_forces(ctx_, ocn, Fdq, Tdq, Fdf, Tdf, cd, cf, to.basis);
        if (status_ != HYDRO_OK) return;
        from_array(Fdq, _Fdq);
        from_array(Tdq, _Tdq);
        from_array(Fdf, _Fdf);
        from_array(Tdf, _Tdf);
    }

private:
    hydro_ctx* ctx_;
    hydro_status status_ = HYDRO_OK;
    std::mutex mu_;
    std::unordered_map<const void*, hydro_mesh_id> ids_;
};

}  // namespace stonefish_gb300

#endif
