"""The C ABI as a C or C++ caller sees it (no GPU).

Every struct of include/stonefish_hydro.h is checked field by field against
the Python mirror in stonefish_gb300/abi.py by a program compiled with gcc
(C11) and g++ (C++17), both with all warnings as errors; the program links
against the library and calls entry points that need no device.  The
header-only C++ layer include/stonefish_hydro.hpp, which gives the three
static hydrodynamics functions the reference's signatures
(SolidEntity.h:113-153), is compiled with minimal Bullet-like types and,
where the reference's source tree is present, with its vendored LinearMath
(btTransform, btVector3)."""
import ctypes as C
import os
import subprocess

import pytest

from oracle.ref import source_root
from stonefish_gb300 import abi

STRUCTS = {
    "hydro_transform": abi.Transform, "hydro_settings": abi.Settings, "hydro_current": abi.Current,
    "hydro_ocean": abi.Ocean, "hydro_compound_part": abi.CompoundPart, "hydro_mesh_properties": abi.MeshProperties,
    "hydro_fluid_approx_result": abi.FluidApprox, "hydro_fft_ocean_params": abi.FftOceanParams,
    "hydro_cable": abi.Cable, "hydro_cable_node_forces": abi.CableNodeForces, "hydro_atmosphere": abi.Atmosphere,
    "hydro_aero_params": abi.AeroParams, "hydro_aero_wrench": abi.AeroWrench, "hydro_body": abi.Body,
    "hydro_wrench": abi.Wrench, "hydro_rigid_state": abi.RigidState, "hydro_tune_result": abi.TuneResult,
    "hydro_config": abi.Config, "hydro_nn_layer": abi.NnLayer, "hydro_nn_net": abi.NnNet,
}
LIB_DIR = os.path.dirname(abi.LIB_PATH)
WARN = ["-Wall", "-Wextra", "-Werror", "-pedantic"]


def layout_program() -> str:
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "stonefish_hydro.h"', "int main(void) {"]
    for cname, st in STRUCTS.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in st._fields_:
            lines.append(f'  printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    # entry points that need no device
    lines += [
        '  printf("abi %d\\n", hydro_abi_version());',
        '  hydro_config cfg; hydro_config_default(&cfg);',
        '  printf("default_cut %d\\n", (int)cfg.cut_precision);',
        '  printf("status_string %d\\n", hydro_status_string(HYDRO_ERR_TIMEOUT) != NULL);',
        '  hydro_ctx* ctx = NULL;',
        '  printf("create_null %d\\n", (int)hydro_create(NULL, &cfg));',
        '  cfg.device = 1000000;',
        '  hydro_status st = hydro_create(&ctx, &cfg);',
        '  printf("create_bad_device %d %d\\n", (int)st, ctx == NULL);',
        "  return 0;", "}"]
    return "\n".join(lines) + "\n"


def compile_and_run(tmp_path, compiler, std, source, suffix, extra=()):
    src = tmp_path / f"prog{suffix}"
    src.write_text(source)
    exe = tmp_path / f"prog_{compiler}"
    cmd = [compiler, f"-std={std}", *WARN, "-I", abi.INCLUDE_DIR, *extra, str(src), "-o", str(exe),
           "-L", LIB_DIR, "-lstonefish_hydro", f"-Wl,-rpath,{LIB_DIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return dict(line.rsplit(" ", 1) if line.count(" ") == 1 else (line.split(" ", 1)[0], line.split(" ", 1)[1])
                for line in out.stdout.strip().splitlines())


@pytest.mark.parametrize("compiler,std,suffix", [("gcc", "c11", ".c"), ("g++", "c++17", ".cpp")])
def test_header_layout_and_host_calls(built_library, tmp_path, compiler, std, suffix):
    got = compile_and_run(tmp_path, compiler, std, layout_program(), suffix)
    for cname, st in STRUCTS.items():
        assert int(got[cname]) == C.sizeof(st), cname
        for f, _ in st._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(st, f).offset, (cname, f)
    assert int(got["abi"]) == abi.ABI_VERSION
    assert int(got["default_cut"]) == abi.CUT_FP32
    assert int(got["status_string"]) == 1
    assert int(got["create_null"]) == abi.HYDRO_ERR_INVALID_ARG
    status, null_ctx = got["create_bad_device"].split()
    assert int(status) != abi.HYDRO_OK and int(null_ctx) == 1


SHIM_STANDIN = r"""
// Minimal types with Bullet's accessors, standing in for btVector3,
// btMatrix3x3 and btTransform, and a mesh with the reference Mesh's accessors.
#include <vector>
#include <cstdio>
#include "stonefish_hydro.hpp"
struct Vec { double m[4] = {0, 0, 0, 0};
  Vec() {} Vec(double x, double y, double z) { m[0] = x; m[1] = y; m[2] = z; }
  double operator[](int i) const { return m[i]; }
  void setValue(double x, double y, double z) { m[0] = x; m[1] = y; m[2] = z; } };
struct Mat { Vec r[3]; const Vec& operator[](int i) const { return r[i]; } };
struct Tf { Mat b; Vec o; const Mat& getBasis() const { return b; } const Vec& getOrigin() const { return o; } };
struct Settings { bool dampingForces; bool reallisticBuoyancy; };
struct Renderable {};
struct Face { unsigned vertexID[3]; };
struct Vertex { float pos[3]; float normal[3]; };
struct PlainMesh { std::vector<Vertex> vertices; std::vector<Face> faces;
  const void* getVertexDataPointer() const { return vertices.data(); }
  size_t getVertexSize() const { return sizeof(Vertex); }
  size_t getNumOfVertices() const { return vertices.size(); }
  const void* getFaceDataPointer() const { return faces.data(); } };
int main() {
  hydro_config cfg; hydro_config_default(&cfg); cfg.device = 1000000;
  hydro_ctx* ctx = nullptr;
  if (hydro_create(&ctx, &cfg) == HYDRO_OK) return 1;   // no such device: the shim is only instantiated
  stonefish_gb300::HydroStatics hs(ctx);
  Settings s{true, true}; Renderable dbg; Tf T; Vec v, w, Fb, Tb, Fdq, Tdq, Fdf, Tdf, cd(1, 1, 1), cf(.1, .1, .1);
  double Swet = 0, Vsub = 0; hydro_ocean ocean = {};
  const PlainMesh* none = nullptr;
  if (ctx != nullptr) {
    hs.ComputeHydrodynamicForcesSurface(s, none, &ocean, T, T, v, w, Fb, Tb, Fdq, Tdq, Fdf, Tdf, Swet, Vsub, dbg);
    hs.ComputeHydrodynamicForcesSubmerged(none, &ocean, T, T, v, w, Fdq, Tdq, Fdf, Tdf);
    hs.CorrectHydrodynamicForces(&ocean, Fdq, Tdq, Fdf, Tdf, cd, cf, T);
  }
  std::printf("ok %d\n", (int)hs.status());
  return 0;
}
"""


def test_cpp_shim_compiles_with_standin_types(built_library, tmp_path):
    got = compile_and_run(tmp_path, "g++", "c++17", SHIM_STANDIN, ".cpp")
    assert "ok" in got


SHIM_BULLET = r"""
// The shim instantiated with the reference's own Bullet types.
#include "LinearMath/btTransform.h"
#include "LinearMath/btVector3.h"
#include "stonefish_hydro.hpp"
#include <cstdio>
struct HydrodynamicsSettings { bool dampingForces; bool reallisticBuoyancy; };
struct Renderable {};
struct Mesh { const void* getVertexDataPointer() const { return nullptr; } size_t getVertexSize() const { return 24; }
  size_t getNumOfVertices() const { return 0; } const void* getFaceDataPointer() const { return nullptr; }
  struct { size_t size() const { return 0; } } faces; };
int main() {
  hydro_config cfg; hydro_config_default(&cfg); cfg.device = 1000000;
  hydro_ctx* ctx = nullptr;
  if (hydro_create(&ctx, &cfg) == HYDRO_OK) return 1;
  stonefish_gb300::HydroStatics hs(ctx);
  HydrodynamicsSettings s{true, true}; Renderable dbg;
  btTransform T = btTransform::getIdentity(); btVector3 v(0, 0, 0), w(0, 0, 0), Fb, Tb, Fdq, Tdq, Fdf, Tdf;
  btVector3 cd(1, 1, 1), cf(0.1, 0.1, 0.1); btScalar Swet = 0, Vsub = 0; hydro_ocean ocean = {};
  const Mesh* none = nullptr;
  hydro_transform t = stonefish_gb300::to_hydro(T);
  if (t.basis[0] != 1.0 || t.basis[4] != 1.0 || t.basis[8] != 1.0) return 2;
  if (ctx != nullptr) {
    hs.ComputeHydrodynamicForcesSurface(s, none, &ocean, T, T, v, w, Fb, Tb, Fdq, Tdq, Fdf, Tdf, Swet, Vsub, dbg);
    hs.ComputeHydrodynamicForcesSubmerged(none, &ocean, T, T, v, w, Fdq, Tdq, Fdf, Tdf);
    hs.CorrectHydrodynamicForces(&ocean, Fdq, Tdq, Fdf, Tdf, cd, cf, T);
  }
  std::printf("ok %d\n", (int)sizeof(btScalar));
  return 0;
}
"""


@pytest.mark.skipif(source_root() is None, reason="reference source tree not present")
def test_cpp_shim_compiles_with_reference_bullet_types(built_library, tmp_path):
    inc = os.path.join(source_root(), "3rdparty")
    got = compile_and_run(tmp_path, "g++", "c++17", SHIM_BULLET, ".cpp",
                          extra=["-DBT_USE_DOUBLE_PRECISION", "-isystem", inc, "-Wno-pedantic"])
    assert got["ok"] == "8"
