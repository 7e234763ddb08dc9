"""Builds oracle/_ref/libstonefish_ref.so: the reference's own hydrodynamics
functions, compiled on the CPU from the reference's source tree.

TEST INFRASTRUCTURE ONLY.  The reference as a whole does not build without
SDL2, GL, FreeType and glm, but the functions of its hydrodynamics path use
only glm vector arithmetic, Bullet's LinearMath and rapidobj (both vendored
in the reference, 3rdparty/) and a few members of Ocean, SolidEntity,
OpenGLRealOcean, OpenGLOcean (its host-side spectrum and butterfly table),
OpenGLContent, Compound and CableEntity.  This recipe reads those functions and type definitions out
of the reference's files where they lie, finds each by its signature and
brace matching, and pipes them with ``#line`` markers into g++ between the
two halves of ``oracle/ref_harness.hpp`` (stand-ins for the reference's
headers; glm restated in ``oracle/ref_glm.hpp``), followed by
``oracle/ref_api.inc`` (C entry points).  Nothing is written but the shared
library and a note of the source root: no reference text is stored.

Compiled as the reference's release build is (CMakeLists.txt:18, :53):
``-O3 -DNDEBUG``, C++17, no ``-march``, BT_USE_DOUBLE_PRECISION and
BT_EULER_DEFAULT_ZYX; plus ``-ffp-contract=off`` so that aarch64 gcc does not
contract what x86-64 gcc cannot.

The source root is ``$STONEFISH_REFERENCE`` or, if unset, /root/reference.
When it is absent (as on a machine without the reference) nothing is built
and ``build_ref()`` returns None.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libstonefish_ref.so")
# the same functions compiled with the reference's DEBUG_HYDRO switch, which
# records the outline of every submerged face part the surface loop evaluates
LIB_DEBUG = os.path.join(OUT_DIR, "libstonefish_ref_debug.so")
ROOT_NOTE = os.path.join(OUT_DIR, "source_root.txt")
DEFAULT_ROOT = "/root/reference"

# (file relative to the reference root, signature prefix).  Types first, in
# declaration order, then the functions.  A block runs from the line that
# starts with the prefix (after indentation) to its matching closing brace.
TYPES = [
    ("Library/include/entities/Entity.h", "enum class PhysicsMode"),
    ("Library/include/entities/Entity.h", "struct PhysicsSettings"),
    ("Library/include/entities/forcefields/Ocean.h", "struct HydrodynamicsSettings"),
    ("Library/include/entities/SolidEntity.h", "enum class GeometryApproxType"),
    ("Library/include/entities/SolidEntity.h", "enum class BodyFluidPosition"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct Vertex"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct TexturableVertex"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct Face"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct Mesh"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct PlainMesh"),
    ("Library/include/graphics/OpenGLDataStructs.h", "struct TexturableMesh"),
    ("Library/include/utils/GeometryFileUtil.h", "inline void hashCombine("),
    ("Library/include/utils/GeometryFileUtil.h", "struct IndexedVertex"),
    ("Library/include/utils/GeometryFileUtil.h", "struct IndexedVertexHash"),
    ("Library/include/utils/GeometryFileUtil.h", "struct IndexedTexturableVertex"),
    ("Library/include/utils/GeometryFileUtil.h", "struct IndexedTexturableVertexHash"),
    ("Library/include/entities/CableEntity.h", "struct CableNodalForces"),
    ("Library/include/graphics/OpenGLOcean.h", "struct OceanParams"),
    ("Library/include/utils/SystemUtil.hpp", "inline long lrandom("),
    ("Library/include/utils/SystemUtil.hpp", "inline float frandom("),
]
FUNCTIONS = [
    ("Library/src/graphics/OpenGLDataStructs.cpp", "glm::mat4 glMatrixFromTransform("),
    ("Library/src/graphics/OpenGLDataStructs.cpp", "glm::vec3 glVectorFromVector("),
    ("Library/src/graphics/OpenGLRealOcean.cpp", "GLfloat OpenGLRealOcean::ComputeInterpolatedWaveData("),
    ("Library/src/graphics/OpenGLRealOcean.cpp", "GLfloat OpenGLRealOcean::ComputeWaveHeight("),
    ("Library/src/entities/forcefields/Uniform.cpp", "Vector3 Uniform::GetVelocityAtPoint("),
    ("Library/src/entities/forcefields/Jet.cpp", "Vector3 Jet::GetVelocityAtPoint("),
    ("Library/src/entities/forcefields/Pipe.cpp", "Vector3 Pipe::GetVelocityAtPoint("),
    ("Library/src/entities/forcefields/Ocean.cpp", "bool Ocean::hasWaves()"),
    ("Library/src/entities/forcefields/Ocean.cpp", "float Ocean::GetDepth(const glm::vec3& point)"),
    ("Library/src/entities/forcefields/Ocean.cpp", "Scalar Ocean::GetDepth(const Vector3& point)"),
    ("Library/src/entities/forcefields/Ocean.cpp", "Vector3 Ocean::GetFluidVelocity(const Vector3& point)"),
    ("Library/src/entities/forcefields/Ocean.cpp", "glm::vec3 Ocean::GetFluidVelocity(const glm::vec3& point)"),
    ("Library/src/entities/forcefields/Atmosphere.cpp", "Vector3 Atmosphere::GetFluidVelocity(const Vector3& point)"),
    ("Library/src/entities/forcefields/Atmosphere.cpp", "glm::vec3 Atmosphere::GetFluidVelocity(const glm::vec3& point)"),
    ("Library/src/entities/SolidEntity.cpp", "bool SolidEntity::isBuoyant()"),
    ("Library/src/entities/SolidEntity.cpp", "BodyFluidPosition SolidEntity::CheckBodyFluidPosition("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::CorrectHydrodynamicForces("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeHydrodynamicForcesSurface("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeHydrodynamicForcesSubmerged("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeHydrodynamicForces(HydrodynamicsSettings"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeAerodynamicForces(Atmosphere*"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeAerodynamicForces(const Mesh*"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::CorrectAerodynamicForces("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::SetHydrodynamicCoefficients("),
    ("Library/src/entities/SolidEntity.cpp", "std::vector<Vector3>* SolidEntity::getMeshVertices()"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeFluidDynamicsApprox("),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeSphericalApprox()"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeCylindricalApprox()"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::ComputeEllipsoidalApprox()"),
    ("Library/src/entities/SolidEntity.cpp", "Scalar SolidEntity::LambKFactor("),
    ("Library/src/graphics/OpenGLContent.cpp", "GLuint vertex4Edge(std::map"),
    ("Library/src/graphics/OpenGLContent.cpp", "GLfloat OpenGLContent::ComputeAverageFaceArea("),
    ("Library/src/graphics/OpenGLContent.cpp", "void OpenGLContent::Refine("),
    ("Library/src/utils/GeometryFileUtil.cpp", "Mesh* LoadOBJ("),
    ("Library/src/utils/GeometryFileUtil.cpp", "void ComputePhysicalProperties(const Mesh* mesh, Scalar thickness, Scalar density, Scalar& mass"),
    ("Library/src/utils/GeometryFileUtil.cpp", "Vector3 FindInertialAxis("),
    ("Library/src/utils/GeometryFileUtil.cpp", "bool IsDiagonal("),
    ("Library/src/entities/SolidEntity.cpp", "PhysicsMode SolidEntity::getPhysicsMode()"),
    ("Library/src/entities/SolidEntity.cpp", "Transform SolidEntity::getO2CTransform()"),
    ("Library/src/entities/SolidEntity.cpp", "void SolidEntity::getHydrodynamicCoefficients("),
    ("Library/src/entities/solids/Compound.cpp", "void Compound::ComputeHydrodynamicForces("),
    ("Library/src/entities/CableEntity.cpp", "Scalar CableEntity::circularSegmentArea("),
    ("Library/src/entities/CableEntity.cpp", "void CableEntity::ComputeHydrodynamicForces("),
    ("Library/src/graphics/OpenGLOcean.cpp", "int OpenGLOcean::bitReverse("),
    ("Library/src/graphics/OpenGLOcean.cpp", "void OpenGLOcean::computeWeight("),
    ("Library/src/graphics/OpenGLOcean.cpp", "GLfloat* OpenGLOcean::ComputeButterflyLookupTable("),
    ("Library/src/graphics/OpenGLOcean.cpp", "float OpenGLOcean::sqr("),
    ("Library/src/graphics/OpenGLOcean.cpp", "float OpenGLOcean::omega("),
    ("Library/src/graphics/OpenGLOcean.cpp", "float OpenGLOcean::spectrum("),
    ("Library/src/graphics/OpenGLOcean.cpp", "void OpenGLOcean::GetSpectrumSample("),
    ("Library/src/graphics/OpenGLOcean.cpp", "void OpenGLOcean::GenerateWavesSpectrum()"),
]

CXXFLAGS = ["-O3", "-DNDEBUG", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
            "-DBT_USE_DOUBLE_PRECISION", "-DBT_EULER_DEFAULT_ZYX", "-w"]


def reference_root() -> str | None:
    root = os.environ.get("STONEFISH_REFERENCE", DEFAULT_ROOT)
    ok = os.path.isfile(os.path.join(root, "Library", "src", "entities", "SolidEntity.cpp"))
    return root if ok else None


def _strip_code(line: str, in_block: bool) -> tuple[str, bool]:
    """The line without comments and string/char literals (for brace counting)."""
    out, i, n = [], 0, len(line)
    while i < n:
        if in_block:
            j = line.find("*/", i)
            if j < 0:
                return "".join(out), True
            i, in_block = j + 2, False
            continue
        c = line[i]
        if line.startswith("//", i):
            break
        if line.startswith("/*", i):
            in_block, i = True, i + 2
            continue
        if c in "\"'":
            j = i + 1
            while j < n and line[j] != c:
                j += 2 if line[j] == "\\" else 1
            i = j + 1
            continue
        out.append(c)
        i += 1
    return "".join(out), in_block


def extract(path: str, prefix: str) -> tuple[int, list[str]]:
    """(first line number, lines) of the block that starts with `prefix`."""
    with open(path, encoding="utf-8", errors="replace") as f:
        lines = f.read().split("\n")
    pat = re.compile(r"^\s*" + re.escape(prefix) + (r"\b" if prefix[-1].isalnum() else ""))
    starts = [i for i, l in enumerate(lines) if pat.match(l)]
    if len(starts) != 1:
        raise RuntimeError(f"{path}: {len(starts)} matches for {prefix!r}")
    s = starts[0]
    depth, opened, in_block = 0, False, False
    for i in range(s, len(lines)):
        code, in_block = _strip_code(lines[i], in_block)
        for ch in code:
            if ch == "{":
                depth, opened = depth + 1, True
            elif ch == "}":
                depth -= 1
        if opened and depth == 0:
            return s + 1, lines[s:i + 1]
    raise RuntimeError(f"{path}: unbalanced block for {prefix!r}")


def translation_unit(root: str) -> str:
    parts = ['#include "ref_harness.hpp"', "namespace sf {"]
    for rel, prefix in TYPES:
        first, body = extract(os.path.join(root, rel), prefix)
        parts.append(f'#line {first} "{rel}"')
        parts.extend(body)
        if not body[-1].rstrip().endswith(";"):
            parts.append(";")
    parts.append("}  // namespace sf")
    parts.append("#define REF_HARNESS_PART2 1")
    parts.append('#include "ref_harness.hpp"')
    parts.append("namespace sf {")
    for rel, prefix in FUNCTIONS:
        first, body = extract(os.path.join(root, rel), prefix)
        parts.append(f'#line {first} "{rel}"')
        parts.extend(body)
    parts.append("}  // namespace sf")
    parts.append('#line 1 "oracle/ref_api.inc"')
    parts.append('#include "ref_api.inc"')
    return "\n".join(parts) + "\n"


def _inputs() -> list[str]:
    own = ["build_ref.py", "ref_harness.hpp", "ref_glm.hpp", "ref_api.inc", "hydro_oracle.h"]
    return [os.path.join(HERE, f) for f in own] + [
        os.path.join(os.path.dirname(HERE), "include", "stonefish_hydro.h")]


def build_ref(force: bool = False) -> str | None:
    """Compiles the library if the reference tree is present; returns its path or None."""
    root = reference_root()
    if root is None:
        return LIB if os.path.exists(LIB) else None
    srcs = _inputs() + [os.path.join(root, rel) for rel, _ in TYPES + FUNCTIONS]
    if not force and all(os.path.exists(L) and all(os.path.getmtime(s) <= os.path.getmtime(L) for s in srcs)
                         for L in (LIB, LIB_DEBUG)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tu = translation_unit(root)
    procs = []
    for out, extra in ((LIB, []), (LIB_DEBUG, ["-DDEBUG_HYDRO"])):
        cmd = [os.environ.get("CXX", "g++"), *CXXFLAGS, *extra, "-I", HERE, "-I", os.path.join(root, "3rdparty"),
               "-I", os.path.join(os.path.dirname(HERE), "include"), "-x", "c++", "-", "-o", out]
        p = subprocess.Popen(cmd, stdin=subprocess.PIPE, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        procs.append(p)
        p.stdin.write(tu.encode())
        p.stdin.close()
    for p in procs:
        log = p.stdout.read()
        if p.wait() != 0:
            raise RuntimeError("reference build failed:\n" + log.decode(errors="replace")[-6000:])
    with open(ROOT_NOTE, "w") as f:
        f.write(root + "\n")
    return LIB


if __name__ == "__main__":
    print(build_ref(force="--force" in sys.argv))
