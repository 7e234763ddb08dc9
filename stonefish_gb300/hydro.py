"""Python front end of the GB300 hydrodynamics library (C ABI via ctypes).

The method names mirror the reference's call surface:

* ``surface_forces``   -- SolidEntity::ComputeHydrodynamicForcesSurface
  (Library/src/entities/SolidEntity.cpp:1289-1721)
* ``submerged_forces`` -- SolidEntity::ComputeHydrodynamicForcesSubmerged (:1723-1797)
* ``correct_forces``   -- SolidEntity::CorrectHydrodynamicForces (:1263-1287)
* ``fluid_position``   -- SolidEntity::CheckBodyFluidPosition (:1239-1261)
* ``body_forces``      -- SolidEntity::ComputeHydrodynamicForces (:1799-1850)
* ``Batch.compute``    -- the per-body loop of the hydrodynamics block of
  SimulationManager::SimulationTickCallback (SimulationManager.cpp:1620-1655)

Every call runs on the GPU; there is no CPU path.  A missing library raises
ImportError, a failing call raises ``abi.HydroError``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def _check(lib, ctx, status: int) -> None:
    if status != abi.HYDRO_OK:
        msg = lib.hydro_last_error(ctx).decode(errors="replace") if ctx else ""
        raise abi.HydroError(status, msg or lib.hydro_status_string(status).decode())


def transform(R, origin) -> abi.Transform:
    t = abi.Transform()
    R = np.asarray(R, dtype=np.float64).reshape(9)
    for i in range(9):
        t.basis[i] = R[i]
    for i in range(3):
        t.origin[i] = float(origin[i])
    return t


def _d3(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(3))
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class HydroContext:
    """Owns a hydro_ctx: device meshes, the wave grid and small buffers."""

    def __init__(self, device: int = 0, cut_precision: int = abi.CUT_FP32,
                 tile_faces: int = 0, ctas_per_sm: int = 0, lib_path: str | None = None,
                 tune_cache_path: str | None = None, frame: int = abi.FRAME_WORLD):
        self.lib = abi.load_library(lib_path)
        lib = self.lib
        if not hasattr(lib, "_debug_declared"):
            lib.hydro_debug_face_terms.restype = C.c_int32
            lib.hydro_debug_face_terms.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(abi.Ocean),
                                                   C.POINTER(abi.Settings), C.c_int32, C.c_void_p]
            lib._debug_declared = True
        cfg = abi.Config()
        lib.hydro_config_default(C.byref(cfg))
        cfg.device = device
        cfg.cut_precision = cut_precision
        cfg.tile_faces = tile_faces
        cfg.ctas_per_sm = ctas_per_sm
        self._tune_path = tune_cache_path.encode() if tune_cache_path else None
        cfg.tune_cache_path = self._tune_path
        h = C.c_void_p()
        st = lib.hydro_create(C.byref(h), C.byref(cfg))
        if st != abi.HYDRO_OK:
            raise abi.HydroError(st, "hydro_create: " + lib.hydro_status_string(st).decode())
        self.ctx = h
        self.device = device
        self.cut_precision = cut_precision
        self.frame = frame
        if frame != abi.FRAME_WORLD:
            self._ck(lib.hydro_set_frame(self.ctx, frame))
        self.mesh_faces: dict[int, int] = {}

    def close(self) -> None:
        if self.ctx:
            self.lib.hydro_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st: int) -> None:
        _check(self.lib, self.ctx, st)

    # --------------------------------------------------------------- meshes
    def upload_mesh(self, xyz: np.ndarray, faces: np.ndarray, stride: int | None = None) -> int:
        """Uploads a physics mesh.  ``xyz`` may be packed (V,3) float32 or the
        reference's interleaved vertex array with ``stride`` bytes per vertex."""
        xyz = np.ascontiguousarray(xyz)
        faces = np.ascontiguousarray(faces, dtype=np.uint32)
        if stride is None:
            xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
            stride = 12
            nv = xyz.shape[0]
        else:
            nv = xyz.nbytes // stride
        mid = C.c_uint32()
        self._ck(self.lib.hydro_mesh_upload(self.ctx, xyz.ctypes.data, stride, nv,
                                            faces.ctypes.data, faces.size // 3, C.byref(mid)))
        self.mesh_faces[int(mid.value)] = faces.size // 3
        return int(mid.value)

    def upload_obj(self, text: str, scale: float = 1.0, refine_threshold: float = 3.0) -> int:
        """hydro_mesh_upload_obj: OBJ text -> refined physics mesh on the device."""
        b = text.encode()
        mid = C.c_uint32()
        self._ck(self.lib.hydro_mesh_upload_obj(self.ctx, b, len(b), scale, refine_threshold, C.byref(mid)))
        return int(mid.value)

    def mesh_properties(self, mesh: int, thickness: float = 0.0, density: float = 1000.0) -> dict:
        """hydro_mesh_compute_properties (ComputePhysicalProperties)."""
        p = abi.MeshProperties()
        self._ck(self.lib.hydro_mesh_compute_properties(self.ctx, mesh, thickness, density, C.byref(p)))
        return {"mass": p.mass, "volume": p.volume, "surface": p.surface, "CG": np.array(p.CG[:]),
                "Ipri": np.array(p.Ipri[:]), "Irot": np.array(p.Irot[:]).reshape(3, 3)}

    def mesh_info(self, mesh: int) -> tuple[int, int, int]:
        nv, nf, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._ck(self.lib.hydro_mesh_info(self.ctx, mesh, C.byref(nv), C.byref(nf), C.byref(nt)))
        return nv.value, nf.value, nt.value

    def set_wave_grid(self, waves: dict) -> None:
        data = np.ascontiguousarray(waves["data"], dtype=np.float32)
        n = data.shape[0]
        ch = 1 if data.ndim == 2 else data.shape[2]
        layers = waves["layers"]
        lc = np.array([c for c, _ in layers], dtype=np.uint32)
        gs = np.array([g for _, g in layers], dtype=np.float32)
        self._ck(self.lib.hydro_wave_grid_set(self.ctx, data.ctypes.data, n, ch, len(layers),
                                              lc.ctypes.data, gs.ctypes.data))

    # ---------------------------------------------------------- entry points
    def depth(self, ocean: abi.Ocean, xyz: np.ndarray) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        out = np.empty(xyz.shape[0], dtype=np.float32)
        self._ck(self.lib.hydro_depth(self.ctx, C.byref(ocean), xyz.ctypes.data, xyz.shape[0],
                                      out.ctypes.data))
        return out

    def fluid_position(self, ocean: abi.Ocean, aabb_min, aabb_max) -> int:
        a, pa = _d3(aabb_min)
        b, pb = _d3(aabb_max)
        r = C.c_int32()
        self._ck(self.lib.hydro_fluid_position(self.ctx, C.byref(ocean), pa, pb, C.byref(r)))
        return int(r.value)

    def body_forces(self, body: np.ndarray, ocean: abi.Ocean, settings: abi.Settings,
                    io: np.ndarray) -> np.ndarray:
        """SolidEntity::ComputeHydrodynamicForces for one body record; io is updated in place."""
        assert body.dtype == abi.BODY_DTYPE and io.dtype == abi.WRENCH_DTYPE
        self._ck(self.lib.hydro_body_forces(self.ctx, body.ctypes.data, C.byref(ocean),
                                            C.byref(settings), io.ctypes.data))
        return io

    def surface_forces(self, settings, mesh, ocean, T_CG, T_C, v, omega, io: dict) -> dict:
        """io: dict of float64 arrays Fb, Tb, Fdq, Tdq, Fdf, Tdf (3,), Swet, Vsub (1,)."""
        vv, pv = _d3(v)
        ww, pw = _d3(omega)
        P = C.POINTER(C.c_double)
        ptrs = [io[k].ctypes.data_as(P) for k in ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf", "Swet", "Vsub")]
        self._ck(self.lib.hydro_surface_forces(self.ctx, C.byref(settings), mesh, C.byref(ocean),
                                               C.byref(T_CG), C.byref(T_C), pv, pw, *ptrs))
        return io

    def submerged_forces(self, mesh, ocean, T_CG, T_C, v, omega, io: dict) -> dict:
        vv, pv = _d3(v)
        ww, pw = _d3(omega)
        P = C.POINTER(C.c_double)
        ptrs = [io[k].ctypes.data_as(P) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self._ck(self.lib.hydro_submerged_forces(self.ctx, mesh, C.byref(ocean), C.byref(T_CG),
                                                 C.byref(T_C), pv, pw, *ptrs))
        return io

    def correct_forces(self, ocean, io: dict, Cd, Cf, R_O) -> dict:
        cd, pcd = _d3(Cd)
        cf, pcf = _d3(Cf)
        ro = np.ascontiguousarray(np.asarray(R_O, dtype=np.float64).reshape(9))
        P = C.POINTER(C.c_double)
        ptrs = [io[k].ctypes.data_as(P) for k in ("Fdq", "Tdq", "Fdf", "Tdf")]
        self._ck(self.lib.hydro_correct_forces(self.ctx, C.byref(ocean), *ptrs, pcd, pcf,
                                               ro.ctypes.data_as(P)))
        return io

    def cable_forces(self, cables: np.ndarray, x, v, ocean, settings, out: np.ndarray) -> np.ndarray:
        """CableEntity::ComputeHydrodynamicForces (CableEntity.cpp:240-376) for
        every cable (host buffers): out = nodal forces, in place."""
        assert cables.dtype == abi.CABLE_DTYPE and out.dtype == abi.CABLE_FORCES_DTYPE
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        assert x.shape == v.shape and x.shape[0] == out.size
        self._ck(self.lib.hydro_cable_forces(self.ctx, cables.ctypes.data if cables.size else None, cables.size,
                                             x.ctypes.data, v.ctypes.data, x.shape[0], C.byref(ocean),
                                             C.byref(settings), out.ctypes.data))
        return out

    def aero_forces(self, mesh, atm, T_CG, T_C, v, omega):
        """SolidEntity::ComputeAerodynamicForces (static form,
        SolidEntity.cpp:1865-1923): returns (Fda, Tda)."""
        F = np.zeros(3)
        T = np.zeros(3)
        vv, pv = _d3(v)
        wv, pw = _d3(omega)
        self._ck(self.lib.hydro_aero_forces(self.ctx, mesh, C.byref(atm), C.byref(T_CG), C.byref(T_C), pv, pw,
                                            F.ctypes.data_as(C.POINTER(C.c_double)),
                                            T.ctypes.data_as(C.POINTER(C.c_double))))
        return F, T

    def aero_correct(self, params, Fda, Tda):
        """SolidEntity::CorrectAerodynamicForces (SolidEntity.cpp:1925-1956)."""
        F = np.array(Fda, dtype=np.float64)
        T = np.array(Tda, dtype=np.float64)
        self._ck(self.lib.hydro_aero_correct(self.ctx, C.byref(params), F.ctypes.data_as(C.POINTER(C.c_double)),
                                             T.ctypes.data_as(C.POINTER(C.c_double))))
        return F, T

    def face_terms(self, body: np.ndarray, ocean, settings, packed: bool = True) -> np.ndarray:
        """Per-face surface-loop terms (n_faces, 23) float32 of one body; packed
        evaluates pairs of submerged faces on the packed FP32 path."""
        nf = self.mesh_faces[int(body["mesh"][0])]
        out = np.zeros((nf, 23), dtype=np.float32)
        self._ck(self.lib.hydro_debug_face_terms(self.ctx, body.ctypes.data, C.byref(ocean),
                                                 C.byref(settings), int(packed), out.ctypes.data))
        return out

    def surface_outline(self, body: np.ndarray, ocean, settings) -> np.ndarray:
        """hydro_debug_surface_outline: the reference's DEBUG_HYDRO points of
        one body's surface loop, float32 (n, 3), two per outline segment."""
        n = C.c_uint32(0)
        self._ck(self.lib.hydro_debug_surface_outline(self.ctx, body.ctypes.data, C.byref(ocean), C.byref(settings),
                                                      None, 0, C.byref(n)))
        pts = np.zeros((n.value, 3), dtype=np.float32)
        if n.value:
            self._ck(self.lib.hydro_debug_surface_outline(self.ctx, body.ctypes.data, C.byref(ocean),
                                                          C.byref(settings), pts.ctypes.data, n.value, C.byref(n)))
        return pts

    def division_check(self, n_pairs: int = 1 << 26, seed: int = 1) -> list[int]:
        """Mismatch counts of the kernels' FMA-corrected division against IEEE
        division (x/3 over all floats, two sets of random pairs)."""
        out = (C.c_uint64 * 3)()
        self._ck(self.lib.hydro_debug_division_check(self.ctx, n_pairs, seed, out))
        return list(out)

    def wait_timeout(self, limit_us: int = 20000) -> int:
        """Status of a bounded device wait that nothing completes (expects
        HYDRO_ERR_TIMEOUT)."""
        st = C.c_int32(-1)
        self._ck(self.lib.hydro_debug_wait_timeout(self.ctx, limit_us, C.byref(st)))
        return int(st.value)

    def arith_check(self, n_pairs: int = 1 << 24, seed: int = 1):
        """(division mismatches[3], packed-op mismatches[4], failing examples[16])."""
        d = (C.c_uint64 * 3)()
        p = (C.c_uint64 * 4)()
        ex = (C.c_float * 16)()
        self._ck(self.lib.hydro_debug_arith_check(self.ctx, n_pairs, seed, d, p, ex))
        return list(d), list(p), list(ex)

    def compute_static(self, mesh_of_body, d_bodies: int, ocean, settings, d_io: int,
                       stream: int = 0) -> None:
        """Allocation-free step (hydro_compute_wrenches_static): device pointers
        in/out, all scratch in the library's static device array."""
        ids = np.ascontiguousarray(mesh_of_body, dtype=np.uint32)
        self._ck(self.lib.hydro_compute_wrenches_static(self.ctx, ids.ctypes.data, ids.size, d_bodies,
                                                        C.byref(ocean), C.byref(settings), d_io,
                                                        stream or None))

    def compute_wrenches(self, mesh_of_body, d_bodies: int, ocean, settings, d_io: int, stream: int = 0) -> None:
        """hydro_compute_wrenches: one call per tick, device pointers in/out; the
        context keeps the batch for this list of meshes between calls."""
        ids = np.ascontiguousarray(mesh_of_body, dtype=np.uint32)
        self._ck(self.lib.hydro_compute_wrenches(self.ctx, ids.ctypes.data, ids.size, d_bodies, C.byref(ocean),
                                                 C.byref(settings), d_io, stream or None))

    def batch(self, mesh_of_body, chunk_faces: int = 0) -> "Batch":
        return Batch(self, mesh_of_body, chunk_faces)


class Batch:
    """A fixed set of bodies (mesh per body) stepped together."""

    def __init__(self, hctx: HydroContext, mesh_of_body, chunk_faces: int = 0):
        self.h = hctx
        self.lib = hctx.lib
        ids = np.ascontiguousarray(mesh_of_body, dtype=np.uint32)
        self.n = ids.size
        b = C.c_void_p()
        _check(self.lib, hctx.ctx, self.lib.hydro_batch_create_ex(hctx.ctx, ids.ctypes.data, ids.size,
                                                                  chunk_faces, C.byref(b)))
        self.b = b

    def close(self) -> None:
        if self.b:
            self.lib.hydro_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def compute(self, bodies: np.ndarray, ocean, settings, io: np.ndarray) -> np.ndarray:
        """Host buffers in/out (copies inside the call)."""
        assert bodies.dtype == abi.BODY_DTYPE and io.dtype == abi.WRENCH_DTYPE
        assert bodies.size == self.n and io.size == self.n
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute(self.b, bodies.ctypes.data,
                                                                  C.byref(ocean), C.byref(settings),
                                                                  io.ctypes.data))
        return io

    def compute_ptr(self, bodies_ptr: int, ocean, settings, io_ptr: int) -> None:
        """Host pointers (e.g. pinned torch tensors) in/out."""
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute(self.b, bodies_ptr, C.byref(ocean),
                                                                  C.byref(settings), io_ptr))

    def compute_device(self, d_bodies: int, ocean, settings, d_io: int, stream: int = 0) -> None:
        """Device pointers in/out; enqueued on ``stream`` (cudaStream_t as int)."""
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute_device(
            self.b, d_bodies, C.byref(ocean), C.byref(settings), d_io, stream or None))

    def compute_aero(self, bodies: np.ndarray, params: np.ndarray, atm, out: np.ndarray) -> np.ndarray:
        """SolidEntity::ComputeAerodynamicForces(Atmosphere*) for every body
        (host buffers; bodies not in AERODYNAMIC mode are left untouched)."""
        assert bodies.dtype == abi.BODY_DTYPE and params.dtype == abi.AERO_PARAMS_DTYPE
        assert out.dtype == abi.AERO_WRENCH_DTYPE and bodies.size == params.size == out.size == self.n
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute_aero(self.b, bodies.ctypes.data, params.ctypes.data,
                                                                       C.byref(atm), out.ctypes.data))
        return out

    def compute_aero_device(self, d_bodies: int, d_params: int, atm, d_out: int, stream: int = 0) -> None:
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute_aero_device(self.b, d_bodies, d_params,
                                                                              C.byref(atm), d_out, stream or None))

    def compute_device_prefix(self, d_bodies: int, d_count: int, ocean, settings, d_io: int,
                              stream: int = 0) -> None:
        """As compute_device for the first *d_count bodies (device uint32)."""
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_compute_device_prefix(
            self.b, d_bodies, d_count, C.byref(ocean), C.byref(settings), d_io, stream or None))

    def autotune(self, d_bodies: int, ocean, settings, d_scratch: int, stream: int = 0, reps: int = 5) -> dict:
        """hydro_batch_autotune: picks chunk size and CTAs per SM for this batch."""
        r = abi.TuneResult()
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_autotune(self.b, d_bodies, C.byref(ocean),
                                                                   C.byref(settings), d_scratch,
                                                                   stream or None, reps, C.byref(r)))
        return {"chunk_faces": r.chunk_faces, "ctas_per_sm": r.ctas_per_sm, "ms_per_step": r.ms_per_step,
                "from_cache": bool(r.from_cache),
                "candidate_ms": [float(x) for x in r.candidate_ms[: r.n_candidates]]}

    def last_launches(self) -> int:
        return int(self.lib.hydro_batch_last_launches(self.b))

    def profile(self, enable: bool = True) -> None:
        """hydro_batch_profile: record per-kernel events on later steps."""
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_profile(self.b, int(enable)))

    def kernel_ms(self) -> dict:
        """hydro_batch_kernel_ms: prep, chunk and finalize times of the last step."""
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        _check(self.lib, self.h.ctx, self.lib.hydro_batch_kernel_ms(self.b, C.byref(a), C.byref(b), C.byref(c)))
        return {"prep": a.value, "chunk": b.value, "finalize": c.value}


class CompoundBatch:
    """Compounds with fixed part lists (hydro_compound_batch): compound c owns
    parts_per_compound[c] consecutive parts, in the reference's part order."""

    def __init__(self, hctx: HydroContext, part_mesh, parts_per_compound):
        self.h = hctx
        self.lib = hctx.lib
        pm = np.ascontiguousarray(part_mesh, dtype=np.uint32)
        ppc = np.ascontiguousarray(parts_per_compound, dtype=np.uint32)
        self.n = ppc.size
        self.n_parts = int(ppc.sum())
        b = C.c_void_p()
        _check(self.lib, hctx.ctx, self.lib.hydro_compound_batch_create(hctx.ctx, pm.ctypes.data if pm.size else None,
                                                                        ppc.ctypes.data, ppc.size, C.byref(b)))
        self.b = b

    def close(self) -> None:
        if self.b:
            self.lib.hydro_compound_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def compute(self, compounds: np.ndarray, parts: np.ndarray, ocean, settings, io: np.ndarray) -> np.ndarray:
        """Compound::ComputeHydrodynamicForces for every compound (host buffers)."""
        assert compounds.dtype == abi.BODY_DTYPE and io.dtype == abi.WRENCH_DTYPE
        assert parts.dtype == abi.COMPOUND_PART_DTYPE and parts.size == self.n_parts
        assert compounds.size == io.size == self.n
        _check(self.lib, self.h.ctx, self.lib.hydro_compound_compute(self.b, compounds.ctypes.data,
                                                                     parts.ctypes.data if parts.size else None,
                                                                     C.byref(ocean), C.byref(settings),
                                                                     io.ctypes.data))
        return io

    def compute_device(self, d_compounds: int, d_parts: int, ocean, settings, d_io: int, stream: int = 0) -> None:
        _check(self.lib, self.h.ctx, self.lib.hydro_compound_compute_device(self.b, d_compounds, d_parts,
                                                                            C.byref(ocean), C.byref(settings),
                                                                            d_io, stream or None))


def fft_ocean_params(state: float = 1.0, passes: int = 8) -> abi.FftOceanParams:
    """OpenGLRealOcean's parameters for a sea state (hydro_fft_ocean_params_for_state)."""
    lib = abi.load_library()
    p = abi.FftOceanParams()
    lib.hydro_fft_ocean_params_for_state(state, C.byref(p))
    p.passes = passes
    return p


class FftOcean:
    """The reference's FFT ocean on the GPU (hydro_fft_ocean_*): writes the
    context's wave grid; depth queries and wrench steps with ocean.waves = 1
    then use it."""

    def __init__(self, hctx: HydroContext, params: abi.FftOceanParams):
        self.h = hctx
        self.lib = hctx.lib
        self.N = 1 << params.passes
        o = C.c_void_p()
        _check(self.lib, hctx.ctx, self.lib.hydro_fft_ocean_create(hctx.ctx, C.byref(params), C.byref(o)))
        self.o = o

    def update(self, t: float, stream: int = 0) -> None:
        _check(self.lib, self.h.ctx, self.lib.hydro_fft_ocean_update(self.o, t, stream or None))

    def read(self) -> np.ndarray:
        out = np.zeros((self.N, self.N, 4), dtype=np.float32)
        _check(self.lib, self.h.ctx, self.lib.hydro_fft_ocean_read(self.o, out.ctypes.data))
        return out

    def close(self) -> None:
        if self.o:
            self.lib.hydro_fft_ocean_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
