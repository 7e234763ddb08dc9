"""The allocation-free entry point, hydro_compute_wrenches_static.

Callers that cannot allocate device memory while they run (a simulator's
real-time tick, where cudaMalloc may synchronise the device, or an
application whose device memory is reserved by another allocator) get the
batched wrench step with all scratch in a static device array.  This file is
collected last so that a failure here stops a `-x` run only after every
other test has run; it also passes on its own in a fresh process."""
import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios
from tests.helpers import scaled_errors

pytestmark = pytest.mark.gpu


def _device_arrays(torch, bodies, n):
    d_b = torch.from_numpy(bodies.view(np.uint8).copy()).cuda()
    d_w = torch.zeros(n * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    return d_b, d_w


def test_static_step_matches_batch_on_two_calls(hctx):
    torch = pytest.importorskip("torch")
    sc = scenarios.mixed_batch(n_bodies=128, seed=21, scale_faces=0.1)
    ids = np.array([hctx.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids[sc["bodies"]["mesh"]]
    n = len(bodies)
    st = scenarios.settings()
    # the existing entry point
    bt = hctx.batch(bodies["mesh"])
    d_b, d_ref = _device_arrays(torch, bodies, n)
    stream = torch.cuda.current_stream().cuda_stream
    bt.compute_device(d_b.data_ptr(), sc["ocean"], st, d_ref.data_ptr(), stream)
    torch.cuda.synchronize()
    ref = d_ref.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
    bt.close()
    # the allocation-free one, twice in a row on the same in-out buffer
    _, d_w = _device_arrays(torch, bodies, n)
    L = 0.5 * np.linalg.norm(bodies["aabb_max"] - bodies["aabb_min"], axis=1)
    for call in range(2):
        hctx.compute_static(bodies["mesh"], d_b.data_ptr(), sc["ocean"], st, d_w.data_ptr(), stream)
        torch.cuda.synchronize()
        out = d_w.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
        assert np.array_equal(out["position"], ref["position"]), call
        assert np.all(out["status"] == 0), call
        e = scaled_errors(out, ref, L)
        act = ref["position"] != abi.OUTSIDE
        for k, v in e.items():
            assert np.max(v[act]) < 2e-6, (call, k, float(np.max(v[act])))


def test_static_step_rejects_too_many_bodies(hctx):
    torch = pytest.importorskip("torch")
    n = abi.STATIC_MAX_BODIES + 1
    ids = np.full(n, abi.NO_MESH, dtype=np.uint32)
    d = torch.zeros(8, dtype=torch.uint8, device="cuda")
    with pytest.raises(abi.HydroError) as ei:
        hctx.compute_static(ids, d.data_ptr(), scenarios.flat_ocean(), scenarios.settings(), d.data_ptr())
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG


def _static_counts(hctx, mesh_xyz_faces):
    """Tiles of the mesh and chunks per body at the context's chunk size."""
    xyz, faces = mesh_xyz_faces
    n_tiles = abi.tile_order(faces, len(xyz))[1].size - 1
    tpc = -(-4096 // abi.TILE_FACES)            # default chunk of 4096 faces in whole tiles
    return n_tiles, -(-n_tiles // tpc)


def test_static_step_rejects_oversized_work_lists(hctx):
    """More chunks than the static work list holds, and a work list whose
    scratch exceeds the array, are rejected before anything is launched."""
    torch = pytest.importorskip("torch")
    from stonefish_gb300 import meshes
    big = meshes.build_icosphere(1.0, 5)                 # 20480 faces
    mid = hctx.upload_mesh(*big)
    hctx.batch(np.array([mid], dtype=np.uint32)).close()  # grows the device tile table
    n_tiles, cpb = _static_counts(hctx, big)
    assert cpb >= 5, (n_tiles, cpb)
    d = torch.zeros(8, dtype=torch.uint8, device="cuda")
    per_chunk = 16 + 16 + 24 * 8                          # ChunkDesc, ActiveChunk, partial sums
    max_chunks = abi.STATIC_SCRATCH_BYTES // per_chunk
    # chunk count above the work-list limit
    n = abi.STATIC_MAX_BODIES
    assert n * cpb > max_chunks
    with pytest.raises(abi.HydroError) as ei:
        hctx.compute_static(np.full(n, mid, np.uint32), d.data_ptr(), scenarios.flat_ocean(), scenarios.settings(),
                            d.data_ptr())
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG and "chunks" in str(ei.value)
    # within the chunk limit, over the scratch bytes (per body 16 + 128 B)
    n = max_chunks // cpb
    assert n * cpb <= max_chunks and n * 144 + n * cpb * per_chunk > abi.STATIC_SCRATCH_BYTES
    with pytest.raises(abi.HydroError) as ei:
        hctx.compute_static(np.full(n, mid, np.uint32), d.data_ptr(), scenarios.flat_ocean(), scenarios.settings(),
                            d.data_ptr())
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG and "scratch" in str(ei.value)


def test_static_step_after_a_rejected_call_and_a_different_batch(hctx):
    """A large batch, a rejected oversized request, then a smaller batch of
    other meshes: the last call matches hydro_batch_compute_device, so no
    state of the earlier calls in the shared array leaks into it."""
    torch = pytest.importorskip("torch")
    st = scenarios.settings()
    stream = torch.cuda.current_stream().cuda_stream
    large = scenarios.mixed_batch(n_bodies=1024, seed=31, scale_faces=0.2)
    ids = np.array([hctx.upload_mesh(x, f) for x, f in large["meshes"]], dtype=np.uint32)
    lb = large["bodies"].copy()
    lb["mesh"] = ids[large["bodies"]["mesh"]]
    small = scenarios.mixed_batch(n_bodies=96, seed=32, scale_faces=0.05)
    ids2 = np.array([hctx.upload_mesh(x, f) for x, f in small["meshes"]], dtype=np.uint32)
    sb = small["bodies"].copy()
    sb["mesh"] = ids2[small["bodies"]["mesh"]]
    bt = hctx.batch(sb["mesh"])                            # reference result; also grows the tile table
    d_sb, d_ref = _device_arrays(torch, sb, len(sb))
    bt.compute_device(d_sb.data_ptr(), small["ocean"], st, d_ref.data_ptr(), stream)
    torch.cuda.synchronize()
    ref = d_ref.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
    bt.close()
    hctx.batch(lb["mesh"]).close()
    d_lb, d_lw = _device_arrays(torch, lb, len(lb))
    hctx.compute_static(lb["mesh"], d_lb.data_ptr(), large["ocean"], st, d_lw.data_ptr(), stream)
    with pytest.raises(abi.HydroError):
        hctx.compute_static(np.full(abi.STATIC_MAX_BODIES + 1, abi.NO_MESH, np.uint32), d_lb.data_ptr(),
                            large["ocean"], st, d_lw.data_ptr(), stream)
    _, d_sw = _device_arrays(torch, sb, len(sb))
    hctx.compute_static(sb["mesh"], d_sb.data_ptr(), small["ocean"], st, d_sw.data_ptr(), stream)
    torch.cuda.synchronize()
    out = d_sw.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
    assert np.array_equal(out["position"], ref["position"])
    assert np.all(out["status"] == 0)
    L = 0.5 * np.linalg.norm(sb["aabb_max"] - sb["aabb_min"], axis=1)
    act = ref["position"] != abi.OUTSIDE
    for k, v in scaled_errors(out, ref, L).items():
        assert np.max(v[act]) < 2e-6, (k, float(np.max(v[act])))
