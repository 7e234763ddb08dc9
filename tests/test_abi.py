"""C ABI: struct layouts match the header, the library exports every declared
symbol, and argument checks that need no device return errors (no GPU)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from stonefish_gb300 import abi

LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "stonefish_hydro.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
#define S(T) printf(#T " %zu\n", sizeof(T))
int main(void) {
  S(hydro_transform); S(hydro_settings); S(hydro_current); S(hydro_ocean);
  S(hydro_body); S(hydro_wrench); S(hydro_config); S(hydro_rigid_state);
  P(hydro_rigid_state, q); P(hydro_rigid_state, thrust_torque); P(hydro_rigid_state, mass); P(hydro_rigid_state, inertial_mass);
  P(hydro_rigid_state, half_extents);
  P(hydro_body, T_C); P(hydro_body, R_O); P(hydro_body, v); P(hydro_body, omega);
  P(hydro_body, Cd); P(hydro_body, Cf); P(hydro_body, P_CB); P(hydro_body, volume);
  P(hydro_body, surface); P(hydro_body, aabb_min); P(hydro_body, aabb_max);
  P(hydro_body, mesh); P(hydro_body, mode); P(hydro_body, buoyancy);
  P(hydro_wrench, Swet); P(hydro_wrench, Vsub); P(hydro_wrench, position); P(hydro_wrench, status);
  P(hydro_ocean, waves); P(hydro_ocean, n_currents); P(hydro_ocean, currents);
  P(hydro_current, vel); P(hydro_current, gamma);
  return 0;
}
"""


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", abi.INCLUDE_DIR, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    got = {k: int(v) for k, v in got.items()}
    sizes = {"hydro_transform": abi.Transform, "hydro_settings": abi.Settings,
             "hydro_current": abi.Current, "hydro_ocean": abi.Ocean, "hydro_body": abi.Body,
             "hydro_wrench": abi.Wrench, "hydro_config": abi.Config,
             "hydro_rigid_state": abi.RigidState}
    for name, st in sizes.items():
        assert got[name] == C.sizeof(st), name
    for key, off in got.items():
        if "." not in key:
            continue
        t, f = key.split(".")
        st = {"hydro_body": abi.Body, "hydro_wrench": abi.Wrench, "hydro_ocean": abi.Ocean,
              "hydro_current": abi.Current, "hydro_rigid_state": abi.RigidState}[t]
        assert getattr(st, f).offset == off, key
    assert abi.BODY_DTYPE.itemsize == got["hydro_body"]
    assert abi.WRENCH_DTYPE.itemsize == got["hydro_wrench"]


def test_library_exports_every_declared_symbol(built_library):
    lib = C.CDLL(built_library)
    names = abi.exported_symbols_from_header()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_header_symbols_are_documented_with_reference_or_role():
    text = open(os.path.join(abi.INCLUDE_DIR, "stonefish_hydro.h")).read()
    for n in ("hydro_surface_forces", "hydro_submerged_forces", "hydro_correct_forces",
              "hydro_fluid_position", "hydro_body_forces", "hydro_batch_compute"):
        assert n in text


def test_null_context_is_rejected_without_device(built_library):
    lib = abi.load_library(built_library)
    assert lib.hydro_abi_version() == 1
    cfg = abi.Config()
    lib.hydro_config_default(C.byref(cfg))
    assert cfg.cut_precision == abi.CUT_FP32 and cfg.tile_faces == 0
    oc = abi.Ocean()
    st = abi.Settings(1, 1)
    xyz = np.zeros((3, 3), np.float32)
    idx = np.array([0, 1, 2], np.uint32)
    mid = C.c_uint32()
    assert lib.hydro_mesh_upload(None, xyz.ctypes.data, 12, 3, idx.ctypes.data, 1, C.byref(mid)) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_batch_compute(None, None, C.byref(oc), C.byref(st), None) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_batch_compute_device(None, None, C.byref(oc), C.byref(st), None, None) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_body_forces(None, None, C.byref(oc), C.byref(st), None) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_compute_wrenches(None, None, 0, None, C.byref(oc), C.byref(st), None, None) == abi.HYDRO_ERR_INVALID_ARG
    d = C.c_void_p()
    assert lib.hydro_mapped_host_ptr(None, C.byref(d)) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_create(None, None) == abi.HYDRO_ERR_INVALID_ARG
    assert lib.hydro_status_string(abi.HYDRO_ERR_INDEX_RANGE) == b"face index out of range"
    assert lib.hydro_last_error(None) == b"null context"
    lib.hydro_destroy(None)
    lib.hydro_batch_destroy(None)


def test_every_entry_point_rejects_null_arguments(built_library):
    """Each status-returning entry point declared in the header, called with
    null handles and pointers and zero counts, returns HYDRO_ERR_INVALID_ARG
    without touching the device and without aborting the process."""
    lib = abi.load_library(built_library)
    checked = 0
    for name in abi.exported_symbols_from_header():
        fn = getattr(lib, name)
        if fn.restype is not C.c_int32 or not fn.argtypes:
            continue
        args = []
        for t in fn.argtypes:
            if t in (C.c_float, C.c_double):
                args.append(0.0)
            elif t in (C.c_int32, C.c_uint32, C.c_int64, C.c_uint64, C.c_size_t, C.c_int):
                args.append(0)
            else:
                args.append(None)
        assert fn(*args) == abi.HYDRO_ERR_INVALID_ARG, name
        checked += 1
    assert checked >= 60


def test_create_reports_device_error_without_gpu(built_library):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = abi.load_library(built_library)
    h = C.c_void_p()
    st = lib.hydro_create(C.byref(h), None)
    assert st == abi.HYDRO_ERR_DEVICE
    assert not h.value


def test_product_does_not_reference_oracle():
    """The GPU library and the package never load the CPU oracle."""
    root = os.path.dirname(abi.HERE)
    for dirpath, _, files in os.walk(abi.HERE):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f), errors="replace").read()
                assert "import oracle" not in text and "from oracle" not in text, f
                assert "hydro_oracle" not in text, f
    assert os.path.isdir(os.path.join(root, "oracle"))


def test_tile_size_constant_matches_header():
    import re
    with open(os.path.join(abi.INCLUDE_DIR, "stonefish_hydro.h")) as fh:
        m = re.search(r"#define HYDRO_TILE_FACES (\d+)", fh.read())
    assert m and int(m.group(1)) == abi.TILE_FACES
