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
