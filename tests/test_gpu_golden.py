"""The CUDA path against the committed golden fixtures (through the C ABI)."""
import numpy as np
import pytest

from stonefish_gb300 import abi
from tests.golden_io import initial_io, load, names
from tests.helpers import scaled_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", names())
def test_gpu_matches_golden(hctx, name):
    g = load(name)
    if g["waves"] is not None:
        hctx.set_wave_grid(g["waves"])
    ids = np.array([hctx.upload_mesh(x, f) for x, f in g["meshes"]], dtype=np.uint32)
    bodies = g["bodies"].copy()
    bodies["mesh"] = ids[g["bodies"]["mesh"]]
    bt = hctx.batch(bodies["mesh"])
    io = initial_io(len(bodies))
    bt.compute(bodies, g["ocean"], g["settings"], io)
    bt.close()
    L = 0.5 * np.linalg.norm(bodies["aabb_max"] - bodies["aabb_min"], axis=1)
    mir = g["out"]["mirror32"]
    assert np.array_equal(io["position"], mir["position"])
    act = io["position"] != abi.OUTSIDE
    for k, v in scaled_errors(io, mir, L).items():
        assert np.max(v[act], initial=0.0) < 2e-6, (name, k)
    # the reference's own FP32 arithmetic is no closer to FP64 than the GPU
    e_gpu = scaled_errors(io, g["out"]["ref64"], L)
    e_ref = scaled_errors(g["out"]["ref32"], g["out"]["ref64"], L)
    for k in e_gpu:
        assert np.max(e_gpu[k][act], initial=0.0) <= np.max(e_ref[k][act], initial=0.0) + 2e-6, (name, k)
