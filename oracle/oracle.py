"""ctypes front end of the C oracle (oracle/hydro_oracle.c) -- test infrastructure.

The C oracle restates Stonefish's SolidEntity hydrodynamics
(Library/src/entities/SolidEntity.cpp:1239-1850); this module only marshals
numpy arrays into it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from stonefish_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
REF32, REF64, MIRROR64, MIRROR32 = 0, 1, 2, 3
T_N = 23


def oracle_lib_path() -> str:
    return os.path.join(HERE, "_build", "libhydro_oracle.so")


def build_oracle(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (gcc, no -march, no FMA contraction)."""
    path = oracle_lib_path()
    srcs = [os.path.join(HERE, f) for f in ("hydro_oracle.c", "hydro_oracle_core.inc", "hydro_oracle.h",
                                            "fft_ocean.c", "Makefile")]
    srcs.append(os.path.join(abi.INCLUDE_DIR, "stonefish_hydro.h"))
    stale = force or not os.path.exists(path) or any(
        os.path.getmtime(s) > os.path.getmtime(path) for s in srcs)
    if stale:
        subprocess.run(["make", "-s", "-B" if force else "all"], cwd=HERE, check=True)
    return path


def centred_scene(bodies: np.ndarray) -> np.ndarray:
    """The bodies shifted so that each one's CG x and y, rounded to FP32, sit
    at the origin: the scene that the library's HYDRO_FRAME_CENTRED evaluates,
    written as a world-frame scene (equivalent for a level ocean with
    position-independent currents, whose forces do not depend on x and y)."""
    b = bodies.copy()
    ox = b["T_CG"]["origin"][:, 0].astype(np.float32).astype(np.float64)
    oy = b["T_CG"]["origin"][:, 1].astype(np.float32).astype(np.float64)
    for key in ("T_CG", "T_C"):
        b[key]["origin"][:, 0] -= ox
        b[key]["origin"][:, 1] -= oy
    b["aabb_min"][:, 0] -= ox
    b["aabb_max"][:, 0] -= ox
    b["aabb_min"][:, 1] -= oy
    b["aabb_max"][:, 1] -= oy
    return b


class OracleMesh(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("stride", C.c_uint32), ("n_vertices", C.c_uint32),
                ("idx", C.c_void_p), ("n_faces", C.c_uint32)]


class OracleWaves(C.Structure):
    _fields_ = [("data", C.c_void_p), ("size", C.c_uint32), ("channels", C.c_uint32),
                ("n_layers", C.c_uint32), ("layer_channel", C.c_uint32 * 4),
                ("layer_grid_size", C.c_float * 4)]


class Oracle:
    """One loaded copy of the oracle library."""

    def __init__(self):
        self.lib = C.CDLL(build_oracle())
        L = self.lib
        vp, i32, u32, d = C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_double)
        P = C.POINTER
        L.oracle_depth.restype = C.c_float
        L.oracle_depth.argtypes = [i32, P(abi.Ocean), vp, C.c_float, C.c_float, C.c_float]
        L.oracle_depth64.restype = C.c_double
        L.oracle_depth64.argtypes = [P(abi.Ocean), vp, C.c_double, C.c_double, C.c_double]
        L.oracle_fluid_position.restype = i32
        L.oracle_fluid_position.argtypes = [P(abi.Ocean), vp, d, d]
        L.oracle_surface_forces.restype = None
        L.oracle_surface_forces.argtypes = [i32, P(abi.Settings), vp, P(abi.Ocean), vp,
                                            P(abi.Transform), P(abi.Transform), d, d,
                                            d, d, d, d, d, d, d, d]
        L.oracle_submerged_forces.restype = None
        L.oracle_submerged_forces.argtypes = [i32, vp, P(abi.Ocean), P(abi.Transform),
                                              P(abi.Transform), d, d, d, d, d, d]
        L.oracle_correct_forces.restype = None
        L.oracle_correct_forces.argtypes = [P(abi.Ocean), d, d, d, d, d, d, d]
        L.oracle_body_forces.restype = None
        L.oracle_body_forces.argtypes = [i32, vp, vp, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.oracle_surface_face_terms.restype = None
        L.oracle_surface_face_terms.argtypes = [i32, P(abi.Settings), vp, P(abi.Ocean), vp,
                                                P(abi.Transform), P(abi.Transform), d, d, vp]
        L.oracle_batch.restype = C.c_double
        L.oracle_batch.argtypes = [i32, i32, vp, u32, vp, u32, P(abi.Ocean), vp,
                                   P(abi.Settings), vp]
        L.oracle_hardware_threads.restype = i32
        L.oracle_hardware_threads.argtypes = []
        L.oracle_mesh_properties.restype = None
        L.oracle_mesh_properties.argtypes = [vp, C.c_double, C.c_double, vp]
        L.oracle_fft_ocean.restype = None
        L.oracle_fft_ocean.argtypes = [P(abi.FftOceanParams), C.c_float, vp]
        L.oracle_fft_ocean_init_only.restype = None
        L.oracle_fft_ocean_init_only.argtypes = [P(abi.FftOceanParams), C.c_float, vp]
        L.oracle_cable_forces.restype = None
        L.oracle_cable_forces.argtypes = [vp, u32, vp, vp, u32, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.oracle_compound_forces.restype = None
        L.oracle_compound_forces.argtypes = [i32, vp, vp, u32, vp, P(abi.Ocean), vp, P(abi.Settings), vp]
        L.oracle_aero_forces.restype = None
        L.oracle_aero_forces.argtypes = [i32, vp, P(abi.Atmosphere), P(abi.Transform), P(abi.Transform),
                                         d, d, d, d]
        L.oracle_aero_correct.restype = None
        L.oracle_aero_correct.argtypes = [P(abi.AeroParams), d, d]
        self._keep = []

    # ------------------------------------------------------------ helpers
    @staticmethod
    def make_mesh(xyz: np.ndarray, faces: np.ndarray):
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        faces = np.ascontiguousarray(faces, dtype=np.uint32)
        m = OracleMesh(xyz.ctypes.data, 3, xyz.shape[0], faces.ctypes.data, faces.shape[0])
        m._arrays = (xyz, faces)  # keep alive
        return m

    @staticmethod
    def make_waves(waves):
        """waves: None or dict(data=float32[N,N,C] or [N,N], layers=[(channel, grid_size)...])."""
        if waves is None:
            return None
        data = np.ascontiguousarray(waves["data"], dtype=np.float32)
        n = data.shape[0]
        ch = 1 if data.ndim == 2 else data.shape[2]
        w = OracleWaves()
        w.data = data.ctypes.data
        w.size = n
        w.channels = ch
        w.n_layers = len(waves["layers"])
        for i, (c, gs) in enumerate(waves["layers"]):
            w.layer_channel[i] = c
            w.layer_grid_size[i] = gs
        w._arrays = (data,)
        return w

    @staticmethod
    def _p(obj):
        return None if obj is None else C.cast(C.pointer(obj), C.c_void_p)

    @staticmethod
    def _vec(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        return a, a.ctypes.data_as(C.POINTER(C.c_double))

    # ------------------------------------------------------------- calls
    def hardware_threads(self) -> int:
        return int(self.lib.oracle_hardware_threads())

    def depth(self, ocean, waves, x, y, z) -> float:
        w = self.make_waves(waves)
        return float(self.lib.oracle_depth(REF32, C.byref(ocean), self._p(w), x, y, z))

    def depth64(self, ocean, waves, x, y, z) -> float:
        w = self.make_waves(waves)
        return float(self.lib.oracle_depth64(C.byref(ocean), self._p(w), x, y, z))

    def fluid_position(self, ocean, aabb_min, aabb_max, waves=None) -> int:
        w = self.make_waves(waves)
        a, pa = self._vec(aabb_min)
        b, pb = self._vec(aabb_max)
        return int(self.lib.oracle_fluid_position(C.byref(ocean), self._p(w), pa, pb))

    def body_forces(self, variant, body, mesh, ocean, settings, io, waves=None):
        """body: BODY_DTYPE record array (1,), io: WRENCH_DTYPE array (1,) updated in place."""
        m = None if mesh is None else self.make_mesh(*mesh)
        w = self.make_waves(waves)
        self.lib.oracle_body_forces(variant, body.ctypes.data, self._p(m), C.byref(ocean),
                                    self._p(w), C.byref(settings), io.ctypes.data)
        return io

    def batch(self, variant, threads, bodies, meshes, ocean, settings, io, waves=None) -> float:
        oms = (OracleMesh * max(1, len(meshes)))()
        keep = []
        for i, (xyz, faces) in enumerate(meshes):
            m = self.make_mesh(xyz, faces)
            keep.append(m)
            oms[i] = m
        w = self.make_waves(waves)
        return float(self.lib.oracle_batch(variant, threads, bodies.ctypes.data, len(bodies),
                                           C.cast(oms, C.c_void_p), len(meshes), C.byref(ocean),
                                           self._p(w), C.byref(settings), io.ctypes.data))

    def surface_forces(self, variant, settings, mesh, ocean, T_CG, T_C, v, omega, io,
                       waves=None):
        """io: dict of float64 arrays Fb,Tb,Fdq,Tdq,Fdf,Tdf (3,) and Swet,Vsub (1,), in place."""
        m = None if mesh is None else self.make_mesh(*mesh)
        w = self.make_waves(waves)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in
                ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf", "Swet", "Vsub")]
        self.lib.oracle_surface_forces(variant, C.byref(settings), self._p(m), C.byref(ocean),
                                       self._p(w), C.byref(T_CG), C.byref(T_C), pv, pw, *ptrs)
        return io

    def submerged_forces(self, variant, mesh, ocean, T_CG, T_C, v, omega, io):
        m = None if mesh is None else self.make_mesh(*mesh)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self.lib.oracle_submerged_forces(variant, self._p(m), C.byref(ocean), C.byref(T_CG),
                                         C.byref(T_C), pv, pw, *ptrs)
        return io

    def correct_forces(self, ocean, io, Cd, Cf, R_O):
        cd, pcd = self._vec(Cd)
        cf, pcf = self._vec(Cf)
        ro, pro = self._vec(R_O)
        ptrs = [io[k].ctypes.data_as(C.POINTER(C.c_double)) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self.lib.oracle_correct_forces(C.byref(ocean), *ptrs, pcd, pcf, pro)
        return io

    def mesh_properties(self, mesh, thickness: float, density: float) -> dict:
        """ComputePhysicalProperties: mass, volume, surface, CG and the trace
        of the inertia tensor about the CG."""
        m = self.make_mesh(*mesh)
        out = np.zeros(7)
        self.lib.oracle_mesh_properties(self._p(m), thickness, density, out.ctypes.data)
        return {"mass": out[0], "volume": out[1], "surface": out[2], "CG": out[3:6].copy(), "trace": out[6]}

    def fft_ocean(self, params, t: float, init_only: bool = False) -> np.ndarray:
        """The reference's FFT ocean at time t: [N, N, 4] float32 (heights of
        the four grids), or the h(k,t) field before the FFTs."""
        N = 1 << params.passes
        out = np.zeros((N, N, 4), dtype=np.float32)
        fn = self.lib.oracle_fft_ocean_init_only if init_only else self.lib.oracle_fft_ocean
        fn(C.byref(params), t, out.ctypes.data)
        return out

    def cable_forces(self, cables, x, v, ocean, settings, out, waves=None):
        """CableEntity::ComputeHydrodynamicForces for every cable; out
        (CABLE_FORCES_DTYPE per node) updated in place."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        w = self.make_waves(waves)
        self.lib.oracle_cable_forces(cables.ctypes.data if len(cables) else None, len(cables), x.ctypes.data,
                                     v.ctypes.data, len(x), C.byref(ocean), self._p(w), C.byref(settings),
                                     out.ctypes.data)
        return out

    def compound_forces(self, variant, compound, parts, part_meshes, ocean, settings, io, waves=None):
        """Compound::ComputeHydrodynamicForces: compound = hydro_body[1],
        parts = hydro_compound_part[n], part_meshes = [(xyz, faces) or None];
        io = hydro_wrench[1], in place."""
        ms = [None if m is None else self.make_mesh(*m) for m in part_meshes]
        ptrs = (C.c_void_p * max(1, len(ms)))(*[self._p(m) for m in ms])
        w = self.make_waves(waves)
        parts = np.ascontiguousarray(parts)
        self.lib.oracle_compound_forces(variant, compound.ctypes.data, parts.ctypes.data if len(parts) else None,
                                        len(parts), C.cast(ptrs, C.c_void_p), C.byref(ocean), self._p(w),
                                        C.byref(settings), io.ctypes.data)
        return io

    def aero_forces(self, variant, mesh, atm, T_CG, T_C, v, omega):
        """SolidEntity::ComputeAerodynamicForces (static form): (Fda, Tda)."""
        m = None if mesh is None else self.make_mesh(*mesh)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        F = np.zeros(3)
        T = np.zeros(3)
        self.lib.oracle_aero_forces(variant, self._p(m), C.byref(atm), C.byref(T_CG), C.byref(T_C), pv, pw,
                                    F.ctypes.data_as(C.POINTER(C.c_double)), T.ctypes.data_as(C.POINTER(C.c_double)))
        return F, T

    def aero_correct(self, params, Fda, Tda):
        F = np.array(Fda, dtype=np.float64)
        T = np.array(Tda, dtype=np.float64)
        self.lib.oracle_aero_correct(C.byref(params), F.ctypes.data_as(C.POINTER(C.c_double)),
                                     T.ctypes.data_as(C.POINTER(C.c_double)))
        return F, T

    def face_terms(self, variant, settings, mesh, ocean, T_CG, T_C, v, omega, waves=None):
        m = self.make_mesh(*mesh)
        w = self.make_waves(waves)
        out = np.zeros((m.n_faces, T_N), dtype=np.float32)
        vv, pv = self._vec(v)
        ww, pw = self._vec(omega)
        self.lib.oracle_surface_face_terms(variant, C.byref(settings), self._p(m), C.byref(ocean),
                                           self._p(w), C.byref(T_CG), C.byref(T_C), pv, pw,
                                           out.ctypes.data)
        return out
