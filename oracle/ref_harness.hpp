/*
 * ref_harness.hpp -- the minimal Stonefish environment in which the
 * reference's own hydrodynamics functions compile on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.py reads the reference's
 * functions (SolidEntity.cpp:170-208, :671-1040, :1239-1956; Ocean.cpp:77-80,
 * :149-201; Atmosphere.cpp:146-157; Uniform/Jet/Pipe GetVelocityAtPoint;
 * OpenGLRealOcean.cpp:282-331; OpenGLDataStructs.cpp:148-171;
 * GeometryFileUtil.cpp:52-283, :335-620; OpenGLContent.cpp:2733-2897;
 * Compound.cpp:291-436; CableEntity.cpp:218-376; OpenGLOcean.cpp:856-1048)
 * and its type definitions (Entity.h:57-69, Ocean.h:36-40, SolidEntity.h:39-41,
 * OpenGLDataStructs.h:120-310, GeometryFileUtil.h:34-123, CableEntity.h:42-54,
 * OpenGLOcean.h:36-51, SystemUtil.hpp:208-218)
 * out of the
 * reference tree at build time and
 * compiles them between this header's two halves into oracle/_ref/.  Nothing
 * of the reference's text is stored in this repository; this header declares
 * only what those functions use, in place of the reference's headers, which
 * pull in SDL2, GL and glm.
 *
 * The classes below carry the reference's member names, because the
 * extracted member functions use them.  Where the reference reads Bullet
 * state (getCGTransform, getAABB, velocities), the stand-in returns the
 * values the test passes in.
 */
#if defined(REF_HARNESS_PART2) && !defined(REF_HARNESS_PART2_DONE)
#define REF_HARNESS_PART2_DONE
/* ------------------------------------------------------------------ part 2:
 * classes whose declarations need the extracted mesh and settings types. */
namespace sf {

/* Console output and timing used by LoadOBJ (SimulationApp.h:34-37,
 * SystemUtil.hpp).  cInfo is silent; cCritical, which aborts the reference's
 * process, records its message instead (ref_last_error). */
extern thread_local char ref_error_message[512];
inline void cInfo(const char*, ...) {}
inline void cCritical(const char* format, ...)
{
    va_list ap;
    va_start(ap, format);
    vsnprintf(ref_error_message, sizeof(ref_error_message), format, ap);
    va_end(ap);
}
inline int64_t GetTimeInMicroseconds() { return 0; }

Mesh* LoadOBJ(const std::string& path, GLfloat scale);
void ComputePhysicalProperties(const Mesh* mesh, Scalar thickness, Scalar density, Scalar& mass, Vector3& CG,
                               Scalar& volume, Scalar& surface, Vector3& Ipri, Matrix3& Irot);
Vector3 FindInertialAxis(const Matrix3& I, Scalar value);
bool IsDiagonal(const Matrix3& A);
GLuint vertex4Edge(std::map<std::pair<GLuint, GLuint>, GLuint>& lookup, Mesh* mesh, GLuint firstID, GLuint secondID);

class OpenGLContent {
public:
    static GLfloat ComputeAverageFaceArea(Mesh* mesh);
    static void Refine(Mesh* mesh, GLfloat sizeThreshold);
};

struct Renderable {
    std::shared_ptr<std::vector<glm::vec3>> points;
    std::shared_ptr<std::vector<glm::vec3>> getDataAsPoints() const { return points; }
};

class OpenGLRealOcean {
public:
    OceanParams params;
    GLfloat* fftData;
    GLfloat ComputeInterpolatedWaveData(GLfloat x, GLfloat y, GLuint channel);
    GLfloat ComputeWaveHeight(GLfloat x, GLfloat y);
};

/* The host half of the FFT ocean (OpenGLOcean.h): spectrum and butterfly table. */
class OpenGLOcean {
public:
    OceanParams params;
    int bitReverse(int i, int N);
    void computeWeight(int N, int k, float& Wr, float& Wi);
    GLfloat* ComputeButterflyLookupTable(unsigned int size, unsigned int passes);
    float sqr(float x);
    float omega(float k);
    float spectrum(float kx, float ky, bool omnispectrum = false);
    void GetSpectrumSample(int i, int j, float lengthScale, float kMin, float* result);
    void GenerateWavesSpectrum();
};

class VelocityField {
public:
    bool enabled = true;
    virtual ~VelocityField() {}
    bool isEnabled() const { return enabled; }
    virtual Vector3 GetVelocityAtPoint(const Vector3& p) const = 0;
};

class Uniform : public VelocityField {
public:
    Vector3 v;
    Vector3 GetVelocityAtPoint(const Vector3& p) const override;
};

class Jet : public VelocityField {
public:
    Vector3 c, n;
    Scalar r, vout;
    Vector3 GetVelocityAtPoint(const Vector3& p) const override;
};

class Pipe : public VelocityField {
public:
    Vector3 p1, n;
    Scalar l, r1, r2, vin, gamma;
    Vector3 GetVelocityAtPoint(const Vector3& p) const override;
};

struct Fluid {
    Scalar density;
};

class Ocean {
public:
    OpenGLRealOcean* glOcean = nullptr;
    Scalar oceanState = Scalar(0);
    bool currentsEnabled = false;
    std::vector<VelocityField*> currents;
    Fluid liquid;
    Fluid getLiquid() const { return liquid; }
    bool hasWaves() const;
    float GetDepth(const glm::vec3& point);
    Scalar GetDepth(const Vector3& point);
    Vector3 GetFluidVelocity(const Vector3& point) const;
    glm::vec3 GetFluidVelocity(const glm::vec3& point) const;
};

class Atmosphere {
public:
    std::vector<VelocityField*> wind;
    Fluid gas;
    Fluid getGas() const { return gas; }
    Vector3 GetFluidVelocity(const Vector3& point) const;
    glm::vec3 GetFluidVelocity(const glm::vec3& point) const;
};

/* SimulationApp::getApp()->getSimulationManager()->getGravity(). */
class SimulationManager {
public:
    Vector3 gravity = Vector3(0, 0, 9.81);
    Ocean* ocean = nullptr;
    Vector3 getGravity() const { return gravity; }
    Ocean* getOcean() { return ocean; }
};

class SimulationApp {
public:
    SimulationManager manager;
    static SimulationApp* getApp();
    SimulationManager* getSimulationManager() { return &manager; }
};

class SolidEntity {
public:
    /* extracted statics (SolidEntity.h:113-180) */
    static void CorrectHydrodynamicForces(Ocean* ocn, Vector3& _Fdq, Vector3& _Tdq, Vector3& _Fdf, Vector3& _Tdf,
                                          const Vector3& fdCd, const Vector3& fdCf, const Transform& T_O);
    static void ComputeHydrodynamicForcesSurface(const HydrodynamicsSettings& settings, const Mesh* mesh, Ocean* liquid,
                                                 const Transform& T_CG, const Transform& T_C, const Vector3& _v,
                                                 const Vector3& _omega, Vector3& _Fb, Vector3& _Tb, Vector3& _Fdq,
                                                 Vector3& _Tdq, Vector3& _Fdf, Vector3& _Tdf, Scalar& _Swet,
                                                 Scalar& _Vsub, Renderable& debug);
    static void ComputeHydrodynamicForcesSubmerged(const Mesh* mesh, Ocean* liquid, const Transform& T_CG,
                                                   const Transform& T_C, const Vector3& _v, const Vector3& _omega,
                                                   Vector3& _Fdq, Vector3& _Tdq, Vector3& _Fdf, Vector3& _Tdf);
    static void ComputeAerodynamicForces(const Mesh* mesh, Atmosphere* atm, const Transform& T_CG,
                                         const Transform& T_C, const Vector3& _v, const Vector3& _omega,
                                         Vector3& _Fda, Vector3& _Tda);
    /* extracted members */
    bool isBuoyant() const;
    BodyFluidPosition CheckBodyFluidPosition(Ocean* ocn);
    void ComputeHydrodynamicForces(HydrodynamicsSettings settings, Ocean* ocn);
    void ComputeAerodynamicForces(Atmosphere* atm);
    void CorrectAerodynamicForces(Atmosphere* atm, Vector3& _Fda, Vector3& _Tda);
    void ComputeFluidDynamicsApprox(GeometryApproxType t);
    void ComputeSphericalApprox();
    void ComputeCylindricalApprox();
    void ComputeEllipsoidalApprox();
    Scalar LambKFactor(Scalar r1, Scalar r2);
    void SetHydrodynamicCoefficients(const Vector3& Cd, const Vector3& Cf);
    std::vector<Vector3>* getMeshVertices() const;
    PhysicsMode getPhysicsMode() const;
    Transform getO2CTransform() const;
    void getHydrodynamicCoefficients(Vector3& Cd, Vector3& Cf) const;

    /* stand-ins for the Bullet-backed accessors */
    void getAABB(Vector3& min, Vector3& max) { min = aabbMin; max = aabbMax; }
    Vector3 getLinearVelocity() const { return vLin; }
    Vector3 getAngularVelocity() const { return vAng; }
    Transform getCGTransform() const { return tCG; }
    Transform getCTransform() const { return tC; }
    Transform getOTransform() const { return tO; }
    const Mesh* getPhysicsMesh() { return physMesh; }

    Vector3 aabbMin, aabbMax, vLin, vAng;
    Transform tCG, tC, tO;
    const Mesh* physMesh = nullptr;

    /* members with the reference's names (SolidEntity.h:400-448) */
    PhysicsSettings phy;
    Scalar volume = Scalar(0);
    Scalar surface = Scalar(0);
    Vector3 P_CB;
    GeometryApproxType fdApproxType = GeometryApproxType::AUTO;
    std::vector<Scalar> fdApproxParams;
    Vector3 fdCd, fdCf;
    Transform T_CG2H;
    Transform T_CG2C, T_CG2O, T_O2C;
    Vector3 aMass, aI;
    Mesh* phyMesh = nullptr;
    Vector3 Fb, Tb, Fdq, Tdq, Fdf, Tdf, Fda, Tda;
    Scalar Swet = Scalar(0);
    Scalar Vsub = Scalar(0);
    Renderable submerged;
};

/* Compound.h:33-39. */
typedef struct {
    SolidEntity* solid;
    Transform origin;
    bool isExternal;
    bool alwaysVisible;
} CompoundPart;

class Compound : public SolidEntity {
public:
    std::vector<CompoundPart> parts;
    void ComputeHydrodynamicForces(HydrodynamicsSettings settings, Ocean* ocn);
};

/* The node array of the cable's btSoftBody: positions m_x, velocities m_v. */
struct SoftBodyNode {
    Vector3 m_x, m_v;
};
struct SoftBodyNodes {
    std::vector<SoftBodyNode> m_nodes;
};

class CableEntity {
public:
    SoftBodyNodes* cableBody_ = nullptr;
    Scalar radius_ = Scalar(0);
    std::vector<CableNodalForces> nodalForces_;
    PhysicsSettings phy_;
    Scalar circularSegmentArea(Scalar h) const;
    void ComputeHydrodynamicForces(HydrodynamicsSettings settings, Ocean* ocn);
};

}  // namespace sf

#elif !defined(REF_HARNESS_PART1_DONE)
#define REF_HARNESS_PART1_DONE
/* ------------------------------------------------------------------ part 1 */
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <unordered_set>
#include <utility>
#include <vector>

#include "rapidobj.hpp"

#include "LinearMath/btMatrix3x3.h"
#include "LinearMath/btQuaternion.h"
#include "LinearMath/btTransform.h"
#include "LinearMath/btVector3.h"
#include "ref_glm.hpp"

typedef float GLfloat;
typedef unsigned int GLuint;

namespace sf {
typedef btScalar Scalar;
typedef btQuaternion Quaternion;
typedef btVector3 Vector3;
typedef btMatrix3x3 Matrix3;
typedef btTransform Transform;
inline Transform I4() { return Transform::getIdentity(); }
inline Matrix3 I3() { return Matrix3::getIdentity(); }
inline Quaternion IQ() { return Quaternion::getIdentity(); }
inline Vector3 V0() { return Vector3(0, 0, 0); }
}  // namespace sf

#endif
