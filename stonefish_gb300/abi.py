"""ctypes/numpy mirror of include/stonefish_hydro.h.

The numpy structured dtypes have exactly the C layout, so arrays of bodies
and wrenches can be handed to the C ABI (host pointers) or copied into
device buffers as raw bytes.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libstonefish_hydro.so")
TILE_FACES = 448   # HYDRO_TILE_FACES: faces per mesh tile, the unit of work chunks
INCLUDE_DIR = os.path.join(REPO, "include")

# status codes
HYDRO_OK = 0
HYDRO_ERR_INVALID_ARG = 1
HYDRO_ERR_OOM = 2
HYDRO_ERR_TIMEOUT = 3
HYDRO_ERR_DEVICE = 4
HYDRO_ERR_NOT_FOUND = 5
HYDRO_ERR_INDEX_RANGE = 6
HYDRO_ERR_UNSUPPORTED = 7
HYDRO_ERR_MISMATCH = 8

# PhysicsMode
MODE_DISABLED, MODE_SURFACE, MODE_FLOATING, MODE_SUBMERGED, MODE_AERODYNAMIC = range(5)
# BodyFluidPosition
INSIDE, OUTSIDE, CROSSING_SURFACE, SKIPPED = 0, 1, 2, -1
# VelocityFieldType
CURRENT_UNIFORM, CURRENT_JET, CURRENT_PIPE = 0, 1, 2
CUT_FP64, CUT_FP32 = 0, 1
FRAME_WORLD, FRAME_CENTRED = 0, 1
ABI_VERSION = 1     # HYDRO_ABI_VERSION
MAX_CURRENTS = 8
MAX_WAVE_LAYERS = 4
NO_MESH = 0xFFFFFFFF
STATIC_MAX_BODIES = 4096
STATIC_SCRATCH_BYTES = 4 << 20

_d3 = C.c_double * 3


class Transform(C.Structure):
    _fields_ = [("basis", C.c_double * 9), ("origin", _d3)]


class Settings(C.Structure):
    _fields_ = [("damping_forces", C.c_int32), ("realistic_buoyancy", C.c_int32)]


class Current(C.Structure):
    _fields_ = [("type", C.c_int32), ("enabled", C.c_int32), ("vel", _d3),
                ("point", _d3), ("dir", _d3), ("radius", C.c_double),
                ("radius2", C.c_double), ("length", C.c_double),
                ("speed", C.c_double), ("gamma", C.c_double)]


class Ocean(C.Structure):
    _fields_ = [("density", C.c_double), ("gravity", C.c_double),
                ("waves", C.c_int32), ("currents_enabled", C.c_int32),
                ("n_currents", C.c_uint32), ("reserved", C.c_uint32),
                ("currents", Current * MAX_CURRENTS)]


class CompoundPart(C.Structure):
    _fields_ = [("T_C", Transform), ("R_O", C.c_double * 9), ("Cd", _d3), ("Cf", _d3),
                ("mesh", C.c_uint32), ("mode", C.c_int32), ("buoyant", C.c_int32), ("external", C.c_int32)]


class MeshProperties(C.Structure):
    _fields_ = [("mass", C.c_double), ("volume", C.c_double), ("surface", C.c_double), ("CG", _d3),
                ("Ipri", _d3), ("Irot", C.c_double * 9)]


class FluidApprox(C.Structure):
    _fields_ = [("approx_type", C.c_int32), ("n_params", C.c_int32), ("params", _d3), ("T_CG2H", Transform),
                ("added_mass", _d3), ("added_inertia", _d3), ("Cd", _d3), ("Cf", _d3)]


class FftOceanParams(C.Structure):
    _fields_ = [("wind", C.c_float), ("omega", C.c_float), ("amplitude", C.c_float), ("km", C.c_float),
                ("cm", C.c_float), ("grid_sizes", C.c_float * 4), ("passes", C.c_uint32), ("propagate", C.c_int32)]


class Cable(C.Structure):
    _fields_ = [("first_node", C.c_uint32), ("n_nodes", C.c_uint32), ("radius", C.c_double),
                ("mode", C.c_int32), ("buoyancy", C.c_int32)]


class CableNodeForces(C.Structure):
    _fields_ = [("Fb", _d3), ("Fdq", _d3), ("Fdf", _d3)]


class Atmosphere(C.Structure):
    _fields_ = [("density", C.c_double), ("n_winds", C.c_uint32), ("reserved", C.c_uint32),
                ("winds", Current * MAX_CURRENTS)]


class AeroParams(C.Structure):
    _fields_ = [("approx_type", C.c_int32), ("reserved", C.c_int32), ("R_CG2H", C.c_double * 9),
                ("approx_params", _d3)]


class AeroWrench(C.Structure):
    _fields_ = [("Fda", _d3), ("Tda", _d3), ("status", C.c_int32), ("reserved", C.c_int32)]


class Body(C.Structure):
    _fields_ = [("T_CG", Transform), ("T_C", Transform), ("R_O", C.c_double * 9),
                ("v", _d3), ("omega", _d3), ("Cd", _d3), ("Cf", _d3), ("P_CB", _d3),
                ("volume", C.c_double), ("surface", C.c_double),
                ("aabb_min", _d3), ("aabb_max", _d3), ("mesh", C.c_uint32),
                ("mode", C.c_int32), ("buoyancy", C.c_int32), ("reserved", C.c_int32)]


class Wrench(C.Structure):
    _fields_ = [("Fb", _d3), ("Tb", _d3), ("Fdq", _d3), ("Tdq", _d3), ("Fdf", _d3),
                ("Tdf", _d3), ("Swet", C.c_double), ("Vsub", C.c_double),
                ("position", C.c_int32), ("status", C.c_int32)]


class RigidState(C.Structure):
    _fields_ = [("p", _d3), ("q", C.c_double * 4), ("v", _d3), ("w", _d3),
                ("thrust_force", _d3), ("thrust_torque", _d3), ("mass", C.c_double),
                ("inertial_mass", C.c_double), ("inertia", _d3), ("half_extents", _d3)]


class NnLayer(C.Structure):
    _fields_ = [("w", C.c_void_p), ("b", C.c_void_p), ("mw", C.c_void_p), ("vw", C.c_void_p),
                ("mb", C.c_void_p), ("vb", C.c_void_p), ("gw", C.c_void_p), ("gb", C.c_void_p),
                ("w16", C.c_void_p), ("wt16", C.c_void_p), ("k", C.c_int32), ("n", C.c_int32)]


class NnNet(C.Structure):
    _fields_ = [("layer", NnLayer * 4), ("z", C.c_void_p * 4), ("x", C.c_void_p * 3), ("dz", C.c_void_p * 4),
                ("xt", C.c_void_p * 4), ("tmean", C.c_void_p), ("tistd", C.c_void_p), ("loss", C.c_void_p),
                ("batch", C.c_int32), ("n_out", C.c_int32)]


class TuneResult(C.Structure):
    _fields_ = [("chunk_faces", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("ms_per_step", C.c_float),
                ("from_cache", C.c_int32), ("n_candidates", C.c_uint32), ("candidate_ms", C.c_float * 16)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("cut_precision", C.c_int32),
                ("tile_faces", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("tune_cache_path", C.c_char_p)]


def _dtype_of(struct) -> np.dtype:
    names, formats, offsets = [], [], []
    for name, ctype in struct._fields_:
        field = getattr(struct, name)
        names.append(name)
        offsets.append(field.offset)
        if issubclass(ctype, C.Structure):
            formats.append(_dtype_of(ctype))
        elif issubclass(ctype, C.Array):
            base = ctype._type_
            if issubclass(base, C.Structure):
                formats.append((_dtype_of(base), (ctype._length_,)))
            else:
                formats.append((np.dtype(base), (ctype._length_,)))
        else:
            formats.append(np.dtype(ctype))
    return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                     "itemsize": C.sizeof(struct)})


TRANSFORM_DTYPE = _dtype_of(Transform)
BODY_DTYPE = _dtype_of(Body)
WRENCH_DTYPE = _dtype_of(Wrench)
OCEAN_DTYPE = _dtype_of(Ocean)
CURRENT_DTYPE = _dtype_of(Current)
RIGID_DTYPE = _dtype_of(RigidState)
AERO_PARAMS_DTYPE = _dtype_of(AeroParams)
COMPOUND_PART_DTYPE = _dtype_of(CompoundPart)
CABLE_DTYPE = _dtype_of(Cable)
CABLE_FORCES_DTYPE = _dtype_of(CableNodeForces)
AERO_WRENCH_DTYPE = _dtype_of(AeroWrench)
APPROX_AUTO, APPROX_SPHERE, APPROX_CYLINDER, APPROX_ELLIPSOID = range(4)

WRENCH_VECTORS = ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf")


def ptr(a: np.ndarray, ctype=C.c_void_p):
    return C.cast(a.ctypes.data, ctype)


class HydroError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"hydro status {status}: {msg}")
        self.status = status


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with stonefish_gb300.build.build()")
    lib = C.CDLL(p)
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int32
    d = C.POINTER(C.c_double)
    sig = {
        "hydro_config_default": (None, [C.POINTER(Config)]),
        "hydro_create": (i32, [C.POINTER(vp), C.POINTER(Config)]),
        "hydro_destroy": (None, [vp]),
        "hydro_last_error": (C.c_char_p, [vp]),
        "hydro_status_string": (C.c_char_p, [i32]),
        "hydro_abi_version": (i32, []),
        "hydro_set_frame": (i32, [vp, i32]),
        "hydro_mesh_upload": (i32, [vp, vp, C.c_size_t, u32, vp, u32, C.POINTER(u32)]),
        "hydro_mesh_info": (i32, [vp, u32, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]),
        "hydro_wave_grid_set": (i32, [vp, vp, u32, u32, u32, vp, vp]),
        "hydro_depth": (i32, [vp, C.POINTER(Ocean), vp, u32, vp]),
        "hydro_batch_create": (i32, [vp, vp, u32, C.POINTER(vp)]),
        "hydro_batch_destroy": (None, [vp]),
        "hydro_batch_compute_device": (i32, [vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp, vp]),
        "hydro_batch_create_ex": (i32, [vp, vp, u32, u32, C.POINTER(vp)]),
        "hydro_batch_autotune": (i32, [vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp, vp, u32,
                                       C.POINTER(TuneResult)]),
        "hydro_batch_compute_device_prefix": (i32, [vp, vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp,
                                                    vp]),
        "hydro_batch_compute": (i32, [vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp]),
        "hydro_batch_last_launches": (u32, [vp]),
        "hydro_batch_profile": (i32, [vp, C.c_int]),
        "hydro_batch_kernel_ms": (i32, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "hydro_body_forces": (i32, [vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp]),
        "hydro_surface_forces": (i32, [vp, C.POINTER(Settings), u32, C.POINTER(Ocean),
                                       C.POINTER(Transform), C.POINTER(Transform), d, d,
                                       d, d, d, d, d, d, d, d]),
        "hydro_submerged_forces": (i32, [vp, u32, C.POINTER(Ocean), C.POINTER(Transform),
                                         C.POINTER(Transform), d, d, d, d, d, d]),
        "hydro_correct_forces": (i32, [vp, C.POINTER(Ocean), d, d, d, d, d, d, d]),
        "hydro_fluid_position": (i32, [vp, C.POINTER(Ocean), d, d, C.POINTER(i32)]),
        "hydro_debug_division_check": (i32, [vp, C.c_uint64, C.c_uint64, vp]),
        "hydro_debug_surface_outline": (i32, [vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp, u32,
                                              C.POINTER(u32)]),
        "hydro_debug_tile_order": (i32, [vp, u32, u32, vp, vp, u32, C.POINTER(u32)]),
        "hydro_mapped_host_ptr": (i32, [vp, C.POINTER(vp)]),
        "hydro_compute_wrenches": (i32, [vp, vp, u32, vp, vp, vp, vp, vp]),
        "hydro_debug_arith_check": (i32, [vp, C.c_uint64, C.c_uint64, vp, vp, vp]),
        "hydro_debug_wait_timeout": (i32, [vp, u32, C.POINTER(i32)]),
        "hydro_compute_wrenches_static": (i32, [vp, vp, u32, vp, C.POINTER(Ocean), C.POINTER(Settings),
                                                vp, vp]),
        "hydro_nn_gemm": (i32, [vp, i32, vp, i32, vp, i32, i32, i32, i32, vp, vp, vp, vp, i32, vp]),
        "hydro_nn_transpose": (i32, [vp, vp, vp, i32, i32, vp]),
        "hydro_nn_mse_grad": (i32, [vp, vp, vp, i32, i32, i32, vp, vp, vp, vp, vp]),
        "hydro_nn_colsum": (i32, [vp, vp, i32, i32, vp, vp]),
        "hydro_nn_adamw": (i32, [vp, vp, vp, vp, vp, i32, i32, i32, C.c_float, C.c_float, C.c_float,
                                 C.c_float, C.c_float, i32, vp, vp, vp]),
        "hydro_nn_train": (i32, [vp, C.POINTER(NnNet), vp, vp, C.c_int64, vp, vp, i32, i32, C.c_float, C.c_float,
                                 C.c_float, C.c_float, vp]),
        "hydro_nn_to_bf16": (i32, [vp, vp, i32, i32, i32, vp, vp, vp, vp]),
        "hydro_nn_features": (i32, [vp, vp, u32, C.POINTER(Ocean), vp, vp]),
        "hydro_nn_gate": (i32, [vp, vp, u32, vp, vp, vp, vp, C.c_float, vp, vp]),
        "hydro_nn_route": (i32, [vp, vp, vp, u32, vp, vp, vp, vp, vp, vp]),
        "hydro_nn_merge": (i32, [vp, vp, vp, i32, vp, vp, u32, vp, vp]),
        "hydro_nn_wrench_body": (i32, [vp, vp, vp, u32, vp, vp]),
        "hydro_nn_pack_sw128": (i32, [vp, vp, i32, i32, i32, i32, vp, vp]),
        "hydro_nn_mlp_tc": (i32, [vp, vp, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "hydro_compound_batch_create": (i32, [vp, vp, vp, u32, C.POINTER(vp)]),
        "hydro_compound_batch_destroy": (None, [vp]),
        "hydro_compound_compute_device": (i32, [vp, vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp, vp]),
        "hydro_compound_compute": (i32, [vp, vp, vp, C.POINTER(Ocean), C.POINTER(Settings), vp]),
        "hydro_mesh_compute_properties": (i32, [vp, u32, C.c_double, C.c_double, C.POINTER(MeshProperties)]),
        "hydro_nn_gate_inside": (i32, [vp, vp, u32, C.POINTER(Ocean), vp, vp]),
        "hydro_nn_ensemble": (i32, [vp, vp, vp, i32, u32, C.c_double, C.c_double, C.c_float, vp, vp]),
        "hydro_nn_audit_pick": (i32, [vp, vp, u32, u32, u32, u32, vp, vp]),
        "hydro_nn_audit_error": (i32, [vp, vp, vp, i32, vp, vp, vp, u32, C.c_double, C.c_double, vp, vp]),
        "hydro_debug_fft_ocean_tables": (i32, [C.POINTER(FftOceanParams), vp, vp, vp, vp]),
        "hydro_fluid_approx": (i32, [vp, C.c_size_t, u32, i32, C.POINTER(Transform), C.POINTER(Transform), d,
                                     C.c_double, C.POINTER(FluidApprox)]),
        "hydro_obj_parse": (i32, [C.c_char_p, C.c_size_t, C.c_float, C.c_float, vp, u32, vp, u32, C.POINTER(u32),
                                  C.POINTER(u32)]),
        "hydro_mesh_upload_obj": (i32, [vp, C.c_char_p, C.c_size_t, C.c_float, C.c_float, C.POINTER(u32)]),
        "hydro_fft_ocean_params_for_state": (None, [C.c_float, C.POINTER(FftOceanParams)]),
        "hydro_fft_ocean_create": (i32, [vp, C.POINTER(FftOceanParams), C.POINTER(vp)]),
        "hydro_fft_ocean_destroy": (None, [vp]),
        "hydro_fft_ocean_update": (i32, [vp, C.c_float, vp]),
        "hydro_fft_ocean_read": (i32, [vp, vp]),
        "hydro_cable_forces_device": (i32, [vp, vp, u32, vp, vp, u32, C.POINTER(Ocean), C.POINTER(Settings), vp,
                                            vp]),
        "hydro_cable_forces": (i32, [vp, vp, u32, vp, vp, u32, C.POINTER(Ocean), C.POINTER(Settings), vp]),
        "hydro_aero_forces": (i32, [vp, u32, C.POINTER(Atmosphere), C.POINTER(Transform), C.POINTER(Transform),
                                    d, d, d, d]),
        "hydro_aero_correct": (i32, [vp, C.POINTER(AeroParams), d, d]),
        "hydro_batch_compute_aero_device": (i32, [vp, vp, vp, C.POINTER(Atmosphere), vp, vp]),
        "hydro_batch_compute_aero": (i32, [vp, vp, vp, C.POINTER(Atmosphere), vp]),
        "hydro_rigid_step": (i32, [vp, vp, vp, vp, vp, u32, C.c_double, C.c_double, vp]),
        "hydro_rigid_write_bodies": (i32, [vp, vp, vp, u32, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def exported_symbols_from_header(header: str | None = None) -> list[str]:
    """Function names declared in include/stonefish_hydro.h."""
    import re
    path = header or os.path.join(INCLUDE_DIR, "stonefish_hydro.h")
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hydro_[a-z0-9_]+)\s*\(", text)))


def mapped_host_ptr(host_ptr: int, lib_path: str | None = None) -> int:
    """hydro_mapped_host_ptr: the device address of page-locked mapped host memory."""
    lib = load_library(lib_path)
    d = C.c_void_p()
    st = lib.hydro_mapped_host_ptr(C.c_void_p(host_ptr), C.byref(d))
    if st != HYDRO_OK:
        raise HydroError(st, "host memory is not page-locked and mapped")
    return int(d.value)


def tile_order(faces: np.ndarray, n_vertices: int, lib_path: str | None = None):
    """hydro_debug_tile_order: the faces in the upload's tile order and each
    tile's first position in it (plus the end); host code only, no GPU."""
    lib = load_library(lib_path)
    fc = np.ascontiguousarray(faces, dtype=np.uint32)
    nf = len(fc)
    order = np.zeros(nf, dtype=np.uint32)
    nt = C.c_uint32(0)
    cap = nf + 1
    starts = np.zeros(cap, dtype=np.uint32)
    st = lib.hydro_debug_tile_order(fc.ctypes.data, int(n_vertices), nf, order.ctypes.data, starts.ctypes.data,
                                    cap, C.byref(nt))
    if st != HYDRO_OK:
        raise HydroError(st, "tile order")
    return order, starts[: nt.value + 1].copy()


def obj_parse(text: str, scale: float = 1.0, refine_threshold: float = 0.0, lib_path: str | None = None):
    """hydro_obj_parse (host only): OBJ text -> (xyz float32 [V,3], faces uint32 [F,3])."""
    lib = load_library(lib_path)
    b = text.encode()
    nv, nf = C.c_uint32(), C.c_uint32()
    st = lib.hydro_obj_parse(b, len(b), scale, refine_threshold, None, 0, None, 0, C.byref(nv), C.byref(nf))
    if st != HYDRO_OK:
        raise HydroError(st, "hydro_obj_parse")
    xyz = np.zeros((nv.value, 3), dtype=np.float32)
    faces = np.zeros((nf.value, 3), dtype=np.uint32)
    st = lib.hydro_obj_parse(b, len(b), scale, refine_threshold, xyz.ctypes.data, nv.value, faces.ctypes.data,
                             nf.value, C.byref(nv), C.byref(nf))
    if st != HYDRO_OK:
        raise HydroError(st, "hydro_obj_parse")
    return xyz, faces


def fluid_approx(vertices: np.ndarray, approx: int, T_CG2C, T_CG2O, P_CB, density: float = 1000.0,
                 vertex_stride: int | None = None, lib_path: str | None = None) -> dict:
    """hydro_fluid_approx (host only): the proxy shape, Cd/Cf and added mass of
    a body from its physics-mesh vertices.  ``vertices`` is float32 [V, 3] or
    the reference's interleaved vertex array (give ``vertex_stride`` in bytes)."""
    lib = load_library(lib_path)
    v = np.ascontiguousarray(vertices)
    stride = vertex_stride if vertex_stride is not None else 12
    n = v.nbytes // stride
    pcb = np.ascontiguousarray(P_CB, dtype=np.float64)
    out = FluidApprox()
    st = lib.hydro_fluid_approx(v.ctypes.data, stride, n, approx, C.byref(T_CG2C), C.byref(T_CG2O),
                                pcb.ctypes.data_as(C.POINTER(C.c_double)), density, C.byref(out))
    if st != HYDRO_OK:
        raise HydroError(st, "hydro_fluid_approx")
    k = out.n_params
    return {"type": out.approx_type, "params": np.array(out.params[:k]),
            "R_CG2H": np.array(out.T_CG2H.basis[:]).reshape(3, 3), "origin_CG2H": np.array(out.T_CG2H.origin[:]),
            "added_mass": np.array(out.added_mass[:]), "added_inertia": np.array(out.added_inertia[:]),
            "Cd": np.array(out.Cd[:]), "Cf": np.array(out.Cf[:])}


def fft_ocean_tables(params, lib_path: str | None = None):
    """hydro_debug_fft_ocean_tables (host only): (s12 [N,N,4], s34 [N,N,4],
    butterfly indices [passes, N, 2], butterfly weights [passes, N, 2])."""
    lib = load_library(lib_path)
    n = 1 << params.passes
    s12 = np.zeros((n, n, 4), np.float32)
    s34 = np.zeros((n, n, 4), np.float32)
    idx = np.zeros((params.passes, n, 2), np.int32)
    w = np.zeros((params.passes, n, 2), np.float32)
    st = lib.hydro_debug_fft_ocean_tables(C.byref(params), s12.ctypes.data, s34.ctypes.data, idx.ctypes.data,
                                          w.ctypes.data)
    if st != HYDRO_OK:
        raise HydroError(st, "hydro_debug_fft_ocean_tables")
    return s12, s34, idx, w
