"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bars:
* per-face contributions: bit-identical to the oracle variant with the same
  arithmetic (MIRROR32 for the default FP32 cut points, which is also the
  reference's own face arithmetic; MIRROR64 for FP64 cut points);
* per-body wrenches: within 2e-6 of the body's force scale (torques: force
  scale x body size) of MIRROR (same face arithmetic, exact sums); the GPU's
  only difference is the summation order of FP32 face terms;
* against the all-FP64 oracle REF64 the GPU must do as well as the
  reference's own FP32 arithmetic (REF32): median pair-scaled error < 1e-6,
  99th percentile < 1e-4, and no worse than REF32's error plus 1e-6.
"""
import math

import numpy as np
import pytest

from oracle import MIRROR32, MIRROR64, REF32, REF64
from stonefish_gb300 import abi, meshes, scenarios
from tests.helpers import body_transform, io_dict, scaled_errors

pytestmark = pytest.mark.gpu

TOL_MIRROR = 2e-6


def run_batch(h, sc, settings=None, io=None):
    ids = [h_id for h_id in sc["_ids"]]
    b = h.batch(np.asarray(ids, dtype=np.uint32)[sc["bodies"]["mesh"]])
    bodies = sc["bodies"].copy()
    bodies["mesh"] = np.asarray(ids, dtype=np.uint32)[sc["bodies"]["mesh"]]
    out = scenarios.new_wrenches(len(bodies)) if io is None else io
    b.compute(bodies, sc["ocean"], settings or scenarios.settings(), out)
    b.close()
    return out


def upload(h, sc):
    if sc.get("waves") is not None:
        h.set_wave_grid(sc["waves"])
    sc["_ids"] = [h.upload_mesh(x, f) for x, f in sc["meshes"]]
    return sc


def run_oracle(oracle, variant, sc, settings=None, io=None):
    out = scenarios.new_wrenches(len(sc["bodies"])) if io is None else io
    oracle.batch(variant, oracle.hardware_threads(), sc["bodies"], sc["meshes"], sc["ocean"],
                 settings or scenarios.settings(), out, waves=sc.get("waves"))
    return out


@pytest.fixture(scope="module")
def sphere_run(hctx):
    sc = upload(hctx, scenarios.single_sphere(steps=1000))
    return sc


def body_lengths(sc):
    h = np.maximum(sc["bodies"]["aabb_max"] - sc["bodies"]["aabb_min"], 0)
    return 0.5 * np.linalg.norm(h, axis=1)


# ------------------------------------------------------------- face terms
@pytest.mark.parametrize("cut", ["fp64", "fp32"])
def test_face_terms_bit_identical(oracle, hctx, hctx64, sphere_run, cut):
    h = hctx64 if cut == "fp64" else hctx
    variant = MIRROR64 if cut == "fp64" else MIRROR32
    sc = sphere_run
    mid = h.upload_mesh(*sc["meshes"][0]) if h is hctx64 else sc["_ids"][0]
    checked = 0
    for i in range(0, 1000, 7):
        b = sc["bodies"][i:i + 1].copy()
        b["mesh"] = mid
        cpu = oracle.face_terms(variant, scenarios.settings(), sc["meshes"][0], sc["ocean"],
                                body_transform(b, "T_CG"), body_transform(b, "T_C"),
                                b["v"][0], b["omega"][0])
        for packed in (False, True):
            gpu = h.face_terms(b, sc["ocean"], scenarios.settings(), packed=packed)
            bad = np.argwhere(gpu != cpu)
            assert bad.size == 0, f"step {i} packed={packed}: {len(bad)} differing terms, first {bad[:3]}"
        checked += int(np.any(cpu != 0))
    assert checked > 50


@pytest.mark.parametrize("cut", ["fp64", "fp32"])
def test_face_terms_every_sign_pattern(oracle, hctx, hctx64, cut):
    """One triangle placed so that each corner is above, on, or below the
    surface: all 27 depth-sign patterns, bit-identical terms."""
    h = hctx64 if cut == "fp64" else hctx
    variant = MIRROR64 if cut == "fp64" else MIRROR32
    xyz = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 1.0, 0.0]], dtype=np.float32)
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    levels = (-0.3, 0.0, 0.25)
    oc = scenarios.flat_ocean((0.2, 0.1, -0.3))
    for a in levels:
        for b_ in levels:
            for c in levels:
                p = xyz.copy()
                p[:, 2] = (a, b_, c)
                mid = h.upload_mesh(p, faces)
                body = scenarios.fill_bodies(1, np.eye(3)[None], np.zeros((1, 3)),
                                             np.array([[0.3, -0.2, 0.1]]), np.array([[0.1, 0.2, -0.3]]),
                                             np.ones((1, 3)), 1.0, 1.0, (1, 1, 1), (.1, .1, .1), mid)
                gpu = h.face_terms(body, oc, scenarios.settings(), packed=False)
                T = body_transform(body)
                cpu = oracle.face_terms(variant, scenarios.settings(), (p, faces), oc, T, T,
                                        body["v"][0], body["omega"][0])
                assert np.array_equal(gpu, cpu), (a, b_, c)


# ---------------------------------------------------------- single sphere
def test_single_sphere_matches_mirror_and_fp64(oracle, hctx, sphere_run):
    sc = sphere_run
    gpu = run_batch(hctx, sc)
    mir = run_oracle(oracle, MIRROR32, sc)
    r32 = run_oracle(oracle, REF32, sc)
    r64 = run_oracle(oracle, REF64, sc)
    assert np.array_equal(gpu["position"], mir["position"])
    assert set(np.unique(gpu["position"])) == {abi.OUTSIDE, abi.CROSSING_SURFACE}
    L = body_lengths(sc)
    cross = gpu["position"] == abi.CROSSING_SURFACE
    e = scaled_errors(gpu, mir, L)
    for k, v in e.items():
        assert np.max(v[cross]) < TOL_MIRROR, (k, float(np.max(v[cross])))
    out = gpu["position"] == abi.OUTSIDE
    for k in abi.WRENCH_VECTORS:
        assert np.all(gpu[k][out] == 0.0)
    e64 = scaled_errors(gpu, r64, L)
    e32 = scaled_errors(r32, r64, L)
    for k in e64:
        assert np.median(e64[k][cross]) < 1e-6, k
        assert np.percentile(e64[k][cross], 99) < 1e-4, k
        assert np.percentile(e64[k][cross], 99) <= np.percentile(e32[k][cross], 99) + 1e-6, k


def test_single_sphere_fully_submerged(oracle, hctx):
    sc = upload(hctx, scenarios.single_sphere(steps=200, depth=(0.5, 1.5), seed=5))
    io0 = scenarios.new_wrenches(200)
    io0["Vsub"] = 0.25
    gpu = run_batch(hctx, sc, io=io0.copy())
    mir = run_oracle(oracle, MIRROR32, sc, io=io0.copy())
    assert np.array_equal(gpu["position"], mir["position"])
    inside = gpu["position"] == abi.INSIDE
    assert inside.sum() > 20
    assert np.all(gpu["Vsub"][inside] == 0.25)                   # INSIDE keeps Vsub
    assert np.all(gpu["Fb"][inside] == mir["Fb"][inside])        # FP64 analytic, bit-exact
    assert np.all(gpu["Swet"][inside] == 4 * math.pi * 0.25)
    e = scaled_errors(gpu, mir, body_lengths(sc))
    for k, v in e.items():
        assert np.max(v) < TOL_MIRROR, k


def test_deterministic_and_stale_outputs(hctx, sphere_run):
    sc = sphere_run
    a = run_batch(hctx, sc)
    b = run_batch(hctx, sc)
    assert a.tobytes() == b.tobytes()
    # tiny Vsub keeps Fb/Tb/Vsub from the previous call
    xyz = sc["meshes"][0][0]
    zmax = float(xyz[:, 2].max())
    body = scenarios.fill_bodies(1, np.eye(3)[None], np.array([[0.0, 0.0, -(zmax - 1e-5)]]),
                                 np.zeros((1, 3)), np.zeros((1, 3)), np.full((1, 3), zmax),
                                 1.0, 1.0, (1, 1, 1), (.1, .1, .1), sc["_ids"][0])
    io = scenarios.new_wrenches(1)
    io["Fb"] = (1.0, 2.0, 3.0)
    io["Vsub"] = 9.0
    hctx.body_forces(body, sc["ocean"], scenarios.settings(), io)
    assert io["position"][0] == abi.CROSSING_SURFACE
    assert tuple(io["Fb"][0]) == (1.0, 2.0, 3.0) and io["Vsub"][0] == 9.0


# ------------------------------------------------------- static entry points
def test_static_entry_points(oracle, hctx, sphere_run):
    sc = sphere_run
    mesh = sc["meshes"][0]
    for i in (3, 10, 42, 77):
        b = sc["bodies"][i:i + 1]
        T_CG, T_C = body_transform(b, "T_CG"), body_transform(b, "T_C")
        for settings in (scenarios.settings(), scenarios.settings(damping=False),
                         scenarios.settings(buoyancy=False)):
            g, c = io_dict(), io_dict()
            for d in (g, c):
                d["Fb"][:] = 1.5
                d["Vsub"][:] = 0.5
            hctx.surface_forces(settings, sc["_ids"][0], sc["ocean"], T_CG, T_C, b["v"][0], b["omega"][0], g)
            oracle.surface_forces(MIRROR32, settings, mesh, sc["ocean"], T_CG, T_C, b["v"][0], b["omega"][0], c)
            S = max(np.linalg.norm(c["Fb"]), np.linalg.norm(c["Fdq"]), np.linalg.norm(c["Fdf"]), 1e-30)
            for k in ("Fb", "Fdq", "Fdf"):
                assert np.linalg.norm(g[k] - c[k]) <= TOL_MIRROR * S, k
            for k in ("Tb", "Tdq", "Tdf"):
                assert np.linalg.norm(g[k] - c[k]) <= TOL_MIRROR * S * 0.5, k
            assert g["Swet"][0] == pytest.approx(c["Swet"][0], rel=TOL_MIRROR, abs=1e-12)
            assert g["Vsub"][0] == pytest.approx(c["Vsub"][0], rel=TOL_MIRROR, abs=1e-12)
        g, c = io_dict(), io_dict()
        hctx.submerged_forces(sc["_ids"][0], sc["ocean"], T_CG, T_C, b["v"][0], b["omega"][0], g)
        oracle.submerged_forces(MIRROR32, mesh, sc["ocean"], T_CG, T_C, b["v"][0], b["omega"][0], c)
        S = max(np.linalg.norm(c["Fdq"]), np.linalg.norm(c["Fdf"]))
        for k in ("Fdq", "Fdf", "Tdq", "Tdf"):
            assert np.linalg.norm(g[k] - c[k]) <= TOL_MIRROR * S, k
        # the correction is FP64 arithmetic in the same order: bit-identical
        g2 = {k: c[k].copy() for k in c}
        c2 = {k: c[k].copy() for k in c}
        hctx.correct_forces(sc["ocean"], g2, b["Cd"][0], b["Cf"][0], b["R_O"][0])
        oracle.correct_forces(sc["ocean"], c2, b["Cd"][0], b["Cf"][0], b["R_O"][0])
        for k in ("Fdq", "Tdq", "Fdf", "Tdf"):
            assert np.array_equal(g2[k], c2[k]), k
        pos_g = hctx.fluid_position(sc["ocean"], b["aabb_min"][0], b["aabb_max"][0])
        assert pos_g == oracle.fluid_position(sc["ocean"], b["aabb_min"][0], b["aabb_max"][0])


def test_null_mesh_and_mode_gate(hctx, sphere_run):
    sc = sphere_run
    bodies = sc["bodies"][:4].copy()
    bodies["mesh"] = sc["_ids"][0]
    bodies["mode"][1] = abi.MODE_DISABLED
    bodies["mesh"][2] = abi.NO_MESH
    bodies["T_CG"]["origin"][:, 2] = 0.0
    bodies["T_C"]["origin"][:, 2] = 0.0
    bodies["aabb_min"][:, 2] = -0.5
    bodies["aabb_max"][:, 2] = 0.5
    ids = bodies["mesh"].copy()
    bt = hctx.batch(ids)
    io = scenarios.new_wrenches(4)
    for k in abi.WRENCH_VECTORS:
        io[k] = 4.0
    io["Swet"] = io["Vsub"] = 4.0
    bt.compute(bodies, sc["ocean"], scenarios.settings(), io)
    assert io["position"][1] == abi.SKIPPED and np.all(io["Fb"][1] == 4.0)
    assert io["position"][2] == abi.CROSSING_SURFACE
    assert np.all(io["Fb"][2] == 0.0) and io["Swet"][2] == 0.0 and io["Vsub"][2] == 0.0
    # a body whose mesh differs from the batch's is flagged and left untouched
    bodies["mesh"][3] = abi.NO_MESH
    io2 = io.copy()
    bt.compute(bodies, sc["ocean"], scenarios.settings(), io2)
    assert io2["status"][3] == abi.HYDRO_ERR_MISMATCH
    assert np.array_equal(io2["Fb"][3], io["Fb"][3])
    bt.close()


def test_jet_and_pipe_currents(oracle, hctx, sphere_run):
    sc = sphere_run
    oc = scenarios.flat_ocean((0.1, 0.0, 0.0))
    oc.n_currents = 3
    c = oc.currents[1]
    c.type, c.enabled = abi.CURRENT_JET, 1
    c.point[:] = (-2.0, 0.0, 0.2)
    c.dir[:] = (1.0, 0.0, 0.0)
    c.radius, c.speed = 0.3, 2.0
    p = oc.currents[2]
    p.type, p.enabled = abi.CURRENT_PIPE, 1
    p.point[:] = (0.0, -2.0, 0.1)
    p.dir[:] = (0.0, 1.0, 0.0)
    p.radius, p.radius2, p.length, p.speed, p.gamma = 0.5, 1.0, 5.0, 1.5, 0.7
    sub = {"meshes": sc["meshes"], "bodies": sc["bodies"][:200].copy(), "ocean": oc, "_ids": sc["_ids"]}
    gpu = run_batch(hctx, sub)
    mir = run_oracle(oracle, MIRROR32, sub)
    cross = gpu["position"] == abi.CROSSING_SURFACE
    e = scaled_errors(gpu, mir, body_lengths(sub))
    # exp/pow of CUDA and the host libm may differ by an ulp in FP64
    for k, v in e.items():
        assert np.max(v[cross]) < 1e-5, k


# ------------------------------------------------------------- batches
@pytest.mark.parametrize("cut", ["fp64", "fp32"])
def test_mixed_batch_matches_mirror(oracle, hctx, hctx64, cut):
    h = hctx64 if cut == "fp64" else hctx
    sc = upload(h, scenarios.mixed_batch(n_bodies=96, seed=11, scale_faces=0.1))
    gpu = run_batch(h, sc)
    mir = run_oracle(oracle, MIRROR64 if cut == "fp64" else MIRROR32, sc)
    assert np.array_equal(gpu["position"], mir["position"])
    act = gpu["position"] != abi.OUTSIDE
    e = scaled_errors(gpu, mir, body_lengths(sc))
    for k, v in e.items():
        assert np.max(v[act]) < TOL_MIRROR, (k, float(np.max(v[act])))
    assert np.all(gpu["status"] == 0)


def test_host_and_device_entry_points_agree(hctx):
    torch = pytest.importorskip("torch")
    sc = upload(hctx, scenarios.mixed_batch(n_bodies=64, seed=12, scale_faces=0.05))
    ids = np.asarray(sc["_ids"], dtype=np.uint32)[sc["bodies"]["mesh"]]
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids
    bt = hctx.batch(ids)
    host = scenarios.new_wrenches(len(bodies))
    bt.compute(bodies, sc["ocean"], scenarios.settings(), host)
    d_b = torch.from_numpy(bodies.view(np.uint8)).cuda()
    d_w = torch.zeros(len(bodies) * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    bt.compute_device(d_b.data_ptr(), sc["ocean"], scenarios.settings(), d_w.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    dev = d_w.cpu().numpy().view(abi.WRENCH_DTYPE)
    assert dev.tobytes() == host.tobytes()
    assert bt.last_launches() == 3          # prep, chunk, finalise
    # page-locked buffers: read and written in place by the kernels
    h_b = torch.from_numpy(bodies.view(np.uint8).copy()).pin_memory()
    h_w = torch.zeros(len(bodies) * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    for _ in range(2):                      # the second call starts from the first one's outputs
        bt.compute_ptr(h_b.data_ptr(), sc["ocean"], scenarios.settings(), h_w.data_ptr())
    bt.compute_device(d_b.data_ptr(), sc["ocean"], scenarios.settings(), d_w.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    assert h_w.numpy().tobytes() == d_w.cpu().numpy().tobytes()
    bt.close()


def test_one_call_step_matches_batch(hctx):
    """hydro_compute_wrenches (the context keeps a batch per list of meshes)
    gives the batch's bits, keeps its batch while the list is unchanged and
    rebuilds it when the list changes."""
    torch = pytest.importorskip("torch")
    sc = upload(hctx, scenarios.mixed_batch(n_bodies=48, seed=14, scale_faces=0.05))
    ids = np.asarray(sc["_ids"], dtype=np.uint32)[sc["bodies"]["mesh"]]
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids
    ref = scenarios.new_wrenches(len(bodies))
    bt = hctx.batch(ids)
    bt.compute(bodies, sc["ocean"], scenarios.settings(), ref)
    bt.close()
    s = torch.cuda.current_stream().cuda_stream
    for n in (len(bodies), len(bodies), len(bodies) // 2):
        d_b = torch.from_numpy(bodies[:n].view(np.uint8).copy()).cuda()
        d_w = torch.zeros(n * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        hctx.compute_wrenches(ids[:n], d_b.data_ptr(), sc["ocean"], scenarios.settings(), d_w.data_ptr(), s)
        torch.cuda.synchronize()
        assert d_w.cpu().numpy().tobytes() == ref[:n].tobytes(), n


@pytest.mark.parametrize("chunk_faces", [abi.TILE_FACES, 4 * abi.TILE_FACES])
def test_prefix_entry_and_chunk_size(hctx, chunk_faces):
    """hydro_batch_compute_device_prefix evaluates exactly the first *count
    bodies (bit-identical to a full step of those bodies) and leaves the rest
    of the in-out array untouched; the chunk size does not change results
    beyond the FP32 summation order."""
    torch = pytest.importorskip("torch")
    sc = upload(hctx, scenarios.mixed_batch(n_bodies=80, seed=13, scale_faces=0.05))
    ids = np.asarray(sc["_ids"], dtype=np.uint32)[sc["bodies"]["mesh"]]
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids
    full = scenarios.new_wrenches(len(bodies))
    bf = hctx.batch(ids, chunk_faces=chunk_faces)
    bf.compute(bodies, sc["ocean"], scenarios.settings(), full)
    ref = scenarios.new_wrenches(len(bodies))
    b0 = hctx.batch(ids)
    b0.compute(bodies, sc["ocean"], scenarios.settings(), ref)
    e = scaled_errors(full, ref, body_lengths(sc))
    act = ref["position"] != abi.OUTSIDE
    for k, v in e.items():
        assert np.max(v[act]) < TOL_MIRROR, (k, float(np.max(v[act])))
    k = 37
    sentinel = scenarios.new_wrenches(len(bodies))
    sentinel["Swet"] = -7.0
    d_b = torch.from_numpy(bodies.view(np.uint8).copy()).cuda()
    d_w = torch.from_numpy(sentinel.view(np.uint8).copy()).cuda()
    d_k = torch.tensor([k], dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    bf.compute_device_prefix(d_b.data_ptr(), d_k.data_ptr(), sc["ocean"], scenarios.settings(), d_w.data_ptr(), s)
    torch.cuda.synchronize()
    got = d_w.cpu().numpy().view(abi.WRENCH_DTYPE)
    assert got[:k].tobytes() == full[:k].tobytes()
    assert got[k:].tobytes() == sentinel[k:].tobytes()
    bf.close()
    b0.close()


def test_wave_grid_limit(built_library):
    """A grid of 2^32 or more values is rejected before anything is read or
    allocated (the lookups use 32-bit texel offsets); the context stays
    usable."""
    import ctypes as C
    from stonefish_gb300.hydro import HydroContext
    h = HydroContext()
    try:
        tiny = np.zeros(4, dtype=np.float32)
        ch = (C.c_uint32 * 1)(0)
        gs = (C.c_float * 1)(102.4)
        for n, c in ((65536, 1), (32768, 4)):
            st = h.lib.hydro_wave_grid_set(h.ctx, tiny.ctypes.data, n, c, 1, ch, gs)
            assert st == abi.HYDRO_ERR_INVALID_ARG, (n, c)
        h.set_wave_grid(scenarios.wave_grid(n=64, n_waves=4, seed=9))
    finally:
        h.close()


@pytest.mark.parametrize("cut", ["fp64", "fp32"])
def test_waves_batch(oracle, hctx, hctx64, cut):
    h = hctx64 if cut == "fp64" else hctx
    sc = scenarios.torpedo_waves(n_bodies=64, faces=2000, grid_n=256)
    upload(h, sc)
    gpu = run_batch(h, sc)
    mir = run_oracle(oracle, MIRROR64 if cut == "fp64" else MIRROR32, sc)
    r64 = run_oracle(oracle, REF64, sc)
    assert np.array_equal(gpu["position"], mir["position"])
    act = gpu["position"] == abi.CROSSING_SURFACE
    assert act.sum() > 10
    e = scaled_errors(gpu, mir, body_lengths(sc))
    for k, v in e.items():
        assert np.max(v[act]) < TOL_MIRROR, (k, float(np.max(v[act])))
    e64 = scaled_errors(gpu, r64, body_lengths(sc))
    for k, v in e64.items():
        assert np.median(v[act]) < 1e-5, k
    # depth queries agree with the oracle's lookup bit for bit
    pts = np.random.default_rng(0).uniform(-30, 60, (1000, 3)).astype(np.float32)
    d = h.depth(sc["ocean"], pts)
    ref = np.array([oracle.depth(sc["ocean"], sc["waves"], *p) for p in pts], dtype=np.float32)
    assert np.array_equal(d, ref)


def test_cut_fp64_matches_mirror64(oracle, hctx64):
    sc = upload(hctx64, scenarios.single_sphere(steps=300, seed=9))
    gpu = run_batch(hctx64, sc)
    mir = run_oracle(oracle, MIRROR64, sc)
    cross = gpu["position"] == abi.CROSSING_SURFACE
    e = scaled_errors(gpu, mir, body_lengths(sc))
    for k, v in e.items():
        assert np.max(v[cross]) < TOL_MIRROR, k


def test_argument_errors(hctx):
    xyz = np.zeros((3, 3), np.float32)
    with pytest.raises(abi.HydroError) as ei:
        hctx.upload_mesh(xyz, np.array([[0, 1, 3]], np.uint32))
    assert ei.value.status == abi.HYDRO_ERR_INDEX_RANGE
    with pytest.raises(abi.HydroError) as ei:
        hctx.batch(np.array([10 ** 6], np.uint32))
    assert ei.value.status == abi.HYDRO_ERR_NOT_FOUND
    with pytest.raises(abi.HydroError) as ei:
        hctx.batch(np.array([], np.uint32))          # empty batch
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG
    with pytest.raises(abi.HydroError) as ei:
        hctx.upload_mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))   # empty mesh
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG


def test_hulls_barely_under_water_match_mirror(oracle, hctx):
    """A finely tiled hull at random attitudes with only its lowest 1-50 mm
    under a flat surface: most tiles lie wholly above the water and are
    skipped by the producer (bounding-sphere test); the bodies must still
    match MIRROR32, so no tile holding an underwater corner was dropped."""
    rng = np.random.default_rng(77)
    xyz, faces = meshes.capped_cylinder_for_faces(0.3, 2.0, 20000)
    n = 192
    R = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, n))
    deepest = np.max(np.einsum("nj,vj->nv", R[:, 2, :], xyz.astype(np.float64)), axis=1)
    pos = np.zeros((n, 3))
    pos[:, :2] = rng.uniform(-5.0, 5.0, (n, 2))
    pos[:, 2] = -deepest + rng.uniform(0.001, 0.05, n)
    half = np.abs(xyz).max(axis=0).astype(np.float64)     # body-frame box about the origin
    mid = hctx.upload_mesh(xyz, faces)
    bodies = scenarios.fill_bodies(n, R, pos, rng.uniform(-1, 1, (n, 3)), rng.uniform(-0.5, 0.5, (n, 3)),
                                   np.tile(half, (n, 1)), 0.5, 4.0, (0.5, 0.6, 0.7), (0.01, 0.02, 0.03), mid,
                                   mode=abi.MODE_FLOATING)
    ocean = scenarios.flat_ocean((0.2, 0.0, 0.0))
    sc = {"bodies": bodies, "meshes": [(xyz, faces)], "ocean": ocean, "_ids": [mid]}
    sc["bodies"]["mesh"] = 0
    gpu = run_batch(hctx, sc)
    mir = run_oracle(oracle, MIRROR32, sc)
    assert np.array_equal(gpu["position"], mir["position"])
    cross = gpu["position"] == abi.CROSSING_SURFACE
    assert cross.sum() > n // 2
    assert np.all(gpu["Vsub"][cross] > 0)
    # The submerged caps are small differences of large signed tetra
    # volumes, so FP32 summation runs cost more digits than on the mixed
    # batch; a dropped tile would remove O(1) of a cap.  Bar: 1e-4.
    e = scaled_errors(gpu, mir, body_lengths(sc))
    for k, v in e.items():
        assert np.max(v[cross]) < 1e-4, (k, float(np.max(v[cross])))


@pytest.mark.parametrize("floats_per_vertex", [6, 11])
def test_reference_vertex_layouts_upload_bit_identical(oracle, hctx, floats_per_vertex):
    """A mesh uploaded as the reference stores it -- interleaved Vertex (24 B:
    position, normal) or TexturableVertex (44 B: position, normal, uv,
    tangent), OpenGLDataStructs.h:120-155, what Mesh::getVertexDataPointer()
    and getVertexSize() give -- yields bit-identical face terms and wrenches
    to the packed 12-byte upload of the same positions."""
    rng = np.random.default_rng(floats_per_vertex)
    xyz, faces = meshes.build_icosphere(0.5, 3)
    aos = rng.standard_normal((len(xyz), floats_per_vertex)).astype(np.float32)
    aos[:, :3] = xyz
    m_packed = hctx.upload_mesh(xyz, faces)
    m_aos = hctx.upload_mesh(aos, faces, stride=4 * floats_per_vertex)
    sc = scenarios.single_sphere(steps=64, seed=51)
    st = scenarios.settings()
    out = []
    for mid in (m_packed, m_aos):
        b = sc["bodies"].copy()
        b["mesh"] = mid
        terms = [hctx.face_terms(b[i:i + 1], sc["ocean"], st, packed=p) for i in (0, 7) for p in (False, True)]
        bt = hctx.batch(b["mesh"])
        io = scenarios.new_wrenches(len(b))
        bt.compute(b, sc["ocean"], st, io)
        bt.close()
        out.append((terms, io))
    for ta, tb in zip(out[0][0], out[1][0]):
        assert np.array_equal(ta, tb)
    for k in list(abi.WRENCH_VECTORS) + ["Swet", "Vsub", "position"]:
        assert np.array_equal(out[0][1][k], out[1][1][k]), k
