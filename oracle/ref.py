"""ctypes front end of oracle/_ref/libstonefish_ref.so -- test infrastructure.

The library is the reference's own hydrodynamics code (SolidEntity.cpp,
Ocean.cpp, OpenGLRealOcean.cpp, Uniform/Jet/Pipe.cpp, OpenGLDataStructs)
compiled on the CPU by oracle/build_ref.py.  It exists only where the
reference's source tree is present; ``Reference.available()`` says whether
it is.  Argument conventions follow oracle.Oracle so tests can run both on
the same inputs.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from stonefish_gb300 import abi

from .build_ref import LIB, LIB_DEBUG, ROOT_NOTE, build_ref
from .oracle import Oracle, OracleMesh


def source_root() -> str | None:
    """The reference tree the library was built from (None if not built)."""
    if not os.path.exists(ROOT_NOTE):
        return None
    with open(ROOT_NOTE) as f:
        root = f.read().strip()
    return root if os.path.isdir(root) else None


class RefCompoundPart(C.Structure):
    """One part of a compound as the reference holds it (ref_api.inc)."""
    _fields_ = [("origin", abi.Transform), ("O2C", abi.Transform), ("Cd", C.c_double * 3), ("Cf", C.c_double * 3),
                ("mesh", C.c_uint32), ("mode", C.c_int32), ("buoyancy", C.c_int32), ("external", C.c_int32)]


REF_PART_DTYPE = abi._dtype_of(RefCompoundPart)


class Reference:
    """The reference's functions, loaded from oracle/_ref."""

    @staticmethod
    def available() -> bool:
        try:
            return build_ref() is not None and os.path.exists(LIB)
        except RuntimeError:
            return False

    def __init__(self):
        path = build_ref()
        if path is None:
            raise RuntimeError("the reference's source tree is not present: oracle/_ref cannot be built")
        self.lib = L = C.CDLL(path)
        vp, i32, u32, d = C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_double)
        P = C.POINTER
        L.ref_depth.restype = C.c_float
        L.ref_depth.argtypes = [P(abi.Ocean), vp, C.c_float, C.c_float, C.c_float]
        L.ref_fluid_position.restype = i32
        L.ref_fluid_position.argtypes = [P(abi.Ocean), vp, d, d]
        L.ref_body_forces.restype = i32
        L.ref_body_forces.argtypes = [vp, vp, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.ref_surface_forces.restype = i32
        L.ref_surface_forces.argtypes = [P(abi.Settings), vp, P(abi.Ocean), vp, P(abi.Transform),
                                         P(abi.Transform), d, d, d, d, d, d, d, d, d, d]
        L.ref_submerged_forces.restype = i32
        L.ref_submerged_forces.argtypes = [vp, P(abi.Ocean), P(abi.Transform), P(abi.Transform), d, d,
                                           d, d, d, d]
        L.ref_correct_forces.restype = None
        L.ref_correct_forces.argtypes = [P(abi.Ocean), d, d, d, d, d, d, d]
        L.ref_aero_forces.restype = None
        L.ref_aero_forces.argtypes = [vp, P(abi.Atmosphere), P(abi.Transform), P(abi.Transform), d, d, d, d]
        L.ref_aero_correct.restype = None
        L.ref_aero_correct.argtypes = [P(abi.AeroParams), d, d]
        L.ref_batch.restype = C.c_double
        L.ref_batch.argtypes = [i32, vp, u32, vp, u32, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.ref_load_obj.restype = i32
        L.ref_load_obj.argtypes = [C.c_char_p, C.c_float, C.c_float, vp, u32, vp, u32, P(u32), P(u32), P(i32)]
        L.ref_mesh_properties.restype = None
        L.ref_mesh_properties.argtypes = [vp, C.c_double, C.c_double, vp]
        L.ref_last_error.restype = C.c_char_p
        L.ref_last_error.argtypes = []
        L.ref_compound_part_frames.restype = None
        L.ref_compound_part_frames.argtypes = [P(abi.Transform), P(abi.Transform), P(abi.Transform),
                                               P(abi.Transform), d]
        L.ref_compound_forces.restype = i32
        L.ref_compound_forces.argtypes = [vp, P(abi.Transform), vp, u32, vp, u32, P(abi.Ocean), vp,
                                          P(abi.Settings), vp]
        L.ref_cable_forces.restype = i32
        L.ref_cable_forces.argtypes = [vp, u32, vp, vp, u32, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.ref_fluid_approx.restype = None
        L.ref_fluid_approx.argtypes = [vp, i32, P(abi.Transform), P(abi.Transform), d, C.c_double, vp]

    _p = staticmethod(Oracle._p)
    _vec = staticmethod(Oracle._vec)
    make_mesh = staticmethod(Oracle.make_mesh)
    make_waves = staticmethod(Oracle.make_waves)

    def depth(self, ocean, waves, x, y, z) -> float:
        w = self.make_waves(waves)
        return float(self.lib.ref_depth(C.byref(ocean), self._p(w), x, y, z))

    def fluid_position(self, ocean, aabb_min, aabb_max, waves=None) -> int:
        w = self.make_waves(waves)
        a, pa = self._vec(aabb_min)
        b, pb = self._vec(aabb_max)
        return int(self.lib.ref_fluid_position(C.byref(ocean), self._p(w), pa, pb))

    def body_forces(self, body, mesh, ocean, settings, io, waves=None):
        m = None if mesh is None else self.make_mesh(*mesh)
        w = self.make_waves(waves)
        rc = self.lib.ref_body_forces(body.ctypes.data, self._p(m), C.byref(ocean), self._p(w),
                                      C.byref(settings), io.ctypes.data)
        if rc != 0:
            raise ValueError("wave data not expressible as the reference's two-layer texture")
        return io

    def batch(self, threads, bodies, meshes, ocean, settings, io, waves=None) -> float:
        oms = (OracleMesh * max(1, len(meshes)))()
        keep = []
        for i, (xyz, faces) in enumerate(meshes):
            m = self.make_mesh(xyz, faces)
            keep.append(m)
            oms[i] = m
        w = self.make_waves(waves)
        t = float(self.lib.ref_batch(threads, bodies.ctypes.data, len(bodies), C.cast(oms, C.c_void_p),
                                     len(meshes), C.byref(ocean), self._p(w), C.byref(settings),
                                     io.ctypes.data))
        if t < 0:
            raise ValueError("wave data not expressible as the reference's two-layer texture")
        return t

    def surface_forces(self, settings, mesh, ocean, T_CG, T_C, v, omega, io, waves=None):
        m = None if mesh is None else self.make_mesh(*mesh)
        w = self.make_waves(waves)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in
                ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf", "Swet", "Vsub")]
        self.lib.ref_surface_forces(C.byref(settings), self._p(m), C.byref(ocean), self._p(w), C.byref(T_CG),
                                    C.byref(T_C), pv, pw, *ptrs)
        return io

    def surface_outline(self, settings, mesh, ocean, T_CG, T_C, v, omega, waves=None) -> np.ndarray:
        """The points the reference's DEBUG_HYDRO build records in
        ComputeHydrodynamicForcesSurface (float32 [n, 3], two per segment)."""
        if not hasattr(self, "dbg"):
            self.dbg = C.CDLL(LIB_DEBUG)
            P = C.POINTER
            d = C.POINTER(C.c_double)
            self.dbg.ref_surface_outline.restype = C.c_int32
            self.dbg.ref_surface_outline.argtypes = [P(abi.Settings), C.c_void_p, P(abi.Ocean), C.c_void_p,
                                                     P(abi.Transform), P(abi.Transform), d, d, C.c_void_p,
                                                     C.c_uint32, P(C.c_uint32)]
        m = None if mesh is None else self.make_mesh(*mesh)
        w = self.make_waves(waves)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        n = C.c_uint32(0)
        args = (C.byref(settings), self._p(m), C.byref(ocean), self._p(w), C.byref(T_CG), C.byref(T_C), pv, pw)
        if self.dbg.ref_surface_outline(*args, None, 0, C.byref(n)):
            raise ValueError("wave data not expressible as the reference's two-layer texture")
        pts = np.zeros((n.value, 3), dtype=np.float32)
        self.dbg.ref_surface_outline(*args, pts.ctypes.data, n.value, C.byref(n))
        return pts

    def submerged_forces(self, mesh, ocean, T_CG, T_C, v, omega, io):
        m = None if mesh is None else self.make_mesh(*mesh)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self.lib.ref_submerged_forces(self._p(m), C.byref(ocean), C.byref(T_CG), C.byref(T_C), pv, pw, *ptrs)
        return io

    def correct_forces(self, ocean, io, Cd, Cf, R_O):
        cd, pcd = self._vec(Cd)
        cf, pcf = self._vec(Cf)
        ro, pro = self._vec(R_O)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self.lib.ref_correct_forces(C.byref(ocean), *ptrs, pcd, pcf, pro)
        return io

    def aero_forces(self, mesh, atm, T_CG, T_C, v, omega):
        m = None if mesh is None else self.make_mesh(*mesh)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        F = np.zeros(3)
        T = np.zeros(3)
        self.lib.ref_aero_forces(self._p(m), C.byref(atm), C.byref(T_CG), C.byref(T_C), pv, pw,
                                 F.ctypes.data_as(C.POINTER(C.c_double)), T.ctypes.data_as(C.POINTER(C.c_double)))
        return F, T

    def aero_correct(self, params, Fda, Tda):
        F = np.array(Fda, dtype=np.float64)
        T = np.array(Tda, dtype=np.float64)
        self.lib.ref_aero_correct(C.byref(params), F.ctypes.data_as(C.POINTER(C.c_double)),
                                  T.ctypes.data_as(C.POINTER(C.c_double)))
        return F, T

    def load_obj(self, path: str, scale: float = 1.0, refine: float = 0.0):
        """LoadOBJ (+ Refine when refine > 0): (xyz float32 [V,3], faces uint32 [F,3], texturable)."""
        nv, nf, tex = C.c_uint32(0), C.c_uint32(0), C.c_int32(0)
        b = path.encode()
        if self.lib.ref_load_obj(b, scale, refine, None, 0, None, 0, C.byref(nv), C.byref(nf), C.byref(tex)):
            raise OSError(f"the reference's LoadOBJ failed on {path}: {self.lib.ref_last_error().decode()}")
        xyz = np.zeros((nv.value, 3), dtype=np.float32)
        faces = np.zeros((nf.value, 3), dtype=np.uint32)
        self.lib.ref_load_obj(b, scale, refine, xyz.ctypes.data, nv.value, faces.ctypes.data, nf.value,
                              C.byref(nv), C.byref(nf), C.byref(tex))
        return xyz, faces, bool(tex.value)

    def mesh_properties(self, mesh, thickness: float, density: float) -> dict:
        """ComputePhysicalProperties: mass, volume, surface, CG, Ipri, Irot."""
        m = self.make_mesh(*mesh)
        out = np.zeros(18)
        self.lib.ref_mesh_properties(self._p(m), thickness, density, out.ctypes.data)
        return {"mass": out[0], "volume": out[1], "surface": out[2], "CG": out[3:6].copy(),
                "Ipri": out[6:9].copy(), "Irot": out[9:18].reshape(3, 3).copy()}

    def fluid_approx(self, mesh, approx: int, T_CG2C, T_CG2O, P_CB, density: float = -1.0) -> dict:
        """ComputeFluidDynamicsApprox for a body with this physics mesh;
        density < 0 = no ocean (the reference then takes 1000)."""
        m = self.make_mesh(*mesh)
        pc, ppc = self._vec(P_CB)
        out = np.zeros(31)
        self.lib.ref_fluid_approx(self._p(m), approx, C.byref(T_CG2C), C.byref(T_CG2O), ppc, density,
                                  out.ctypes.data)
        n = int(out[1])
        return {"type": int(out[0]), "params": out[2:2 + n].copy(), "R_CG2H": out[5:14].reshape(3, 3).copy(),
                "origin_CG2H": out[14:17].copy(), "added_mass": out[17:20].copy(),
                "added_inertia": out[20:23].copy(), "Cd": out[23:26].copy(), "Cf": out[26:29].copy()}

    def compound_part_frames(self, T_O, origin, O2C):
        """(T_C of the part, basis of T_O * origin) as Compound.cpp:343-344 forms them."""
        tc = abi.Transform()
        ro = np.zeros(9)
        self.lib.ref_compound_part_frames(C.byref(T_O), C.byref(origin), C.byref(O2C), C.byref(tc),
                                          ro.ctypes.data_as(C.POINTER(C.c_double)))
        return tc, ro

    def compound_forces(self, compound, T_O, parts, meshes, ocean, settings, io, waves=None):
        """Compound::ComputeHydrodynamicForces: compound = hydro_body[1],
        parts = REF_PART_DTYPE[n] (mesh = index into meshes or NO_MESH),
        io = hydro_wrench[1] updated in place."""
        oms = (OracleMesh * max(1, len(meshes)))()
        keep = []
        for i, (xyz, faces) in enumerate(meshes):
            m = self.make_mesh(xyz, faces)
            keep.append(m)
            oms[i] = m
        w = self.make_waves(waves)
        parts = np.ascontiguousarray(parts)
        rc = self.lib.ref_compound_forces(compound.ctypes.data, C.byref(T_O), parts.ctypes.data, len(parts),
                                          C.cast(oms, C.c_void_p), len(meshes), C.byref(ocean), self._p(w),
                                          C.byref(settings), io.ctypes.data)
        if rc != 0:
            raise ValueError("wave data not expressible as the reference's two-layer texture")
        return io

    def cable_forces(self, cables, x, v, ocean, settings, out, waves=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = self.make_waves(waves)
        self.lib.ref_cable_forces(cables.ctypes.data, len(cables), x.ctypes.data, v.ctypes.data, len(x),
                                  C.byref(ocean), self._p(w), C.byref(settings), out.ctypes.data)
        return out

    def fft_spectrum(self, params):
        """GenerateWavesSpectrum: (spectrum12, spectrum34), each [N, N, 4]
        float32.  The reference's generator seed is a function-local static,
        so each call loads a fresh copy of the library."""
        import shutil
        import tempfile
        n = 1 << params.passes
        s12 = np.zeros((n, n, 4), np.float32)
        s34 = np.zeros((n, n, 4), np.float32)
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "libstonefish_ref_copy.so")
            shutil.copyfile(LIB, path)
            lib = C.CDLL(path)
            lib.ref_fft_spectrum.restype = None
            lib.ref_fft_spectrum.argtypes = [C.POINTER(abi.FftOceanParams), C.c_void_p, C.c_void_p]
            lib.ref_fft_spectrum(C.byref(params), s12.ctypes.data, s34.ctypes.data)
        return s12, s34

    def fft_butterfly(self, size: int, passes: int) -> np.ndarray:
        """ComputeButterflyLookupTable: [passes, size, 4] float32."""
        out = np.zeros((passes, size, 4), np.float32)
        self.lib.ref_fft_butterfly.restype = None
        self.lib.ref_fft_butterfly.argtypes = [C.c_uint, C.c_uint, C.c_void_p]
        self.lib.ref_fft_butterfly(size, passes, out.ctypes.data)
        return out
