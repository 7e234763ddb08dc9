"""GPU checks of the native autotuner: it times every candidate, keeps one
of them, does not change the results beyond the FP32 summation order, and
its cache file is reused for a batch of the same shape."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from stonefish_gb300 import abi, scenarios  # noqa: E402
from tests.helpers import scaled_errors  # noqa: E402

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_caches_it(built_library, tmp_path):
    from stonefish_gb300.hydro import HydroContext

    cache = str(tmp_path / "tune.txt")
    h = HydroContext(0, tune_cache_path=cache)
    sc = scenarios.mixed_batch(n_bodies=64, seed=21, scale_faces=0.05)
    ids = np.asarray([h.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)[sc["bodies"]["mesh"]]
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids
    st = scenarios.settings()
    b = h.batch(ids)
    before = scenarios.new_wrenches(len(bodies))
    b.compute(bodies, sc["ocean"], st, before)
    d_b = torch.from_numpy(bodies.view(np.uint8).copy()).cuda()
    d_s = torch.zeros(len(bodies) * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    r = b.autotune(d_b.data_ptr(), sc["ocean"], st, d_s.data_ptr(), reps=2)
    assert not r["from_cache"]
    assert r["chunk_faces"] in tuple(t * abi.TILE_FACES for t in (2, 4, 8, 11, 16, 24, 32))
    assert r["ctas_per_sm"] in (1, 2)
    assert len(r["candidate_ms"]) == 14 and min(r["candidate_ms"]) == pytest.approx(r["ms_per_step"])
    after = scenarios.new_wrenches(len(bodies))
    b.compute(bodies, sc["ocean"], st, after)
    assert np.array_equal(after["position"], before["position"])
    L = 0.5 * np.linalg.norm(np.maximum(bodies["aabb_max"] - bodies["aabb_min"], 0), axis=1)
    act = before["position"] != abi.OUTSIDE
    for k, v in scaled_errors(after, before, L).items():
        assert np.max(v[act]) < 2e-6, k
    assert os.path.exists(cache) and len(open(cache).read().strip().splitlines()) == 1
    # a second batch of the same shape takes the cached choice without timing
    b2 = h.batch(ids)
    r2 = b2.autotune(d_b.data_ptr(), sc["ocean"], st, d_s.data_ptr(), reps=2)
    assert r2["from_cache"] and r2["chunk_faces"] == r["chunk_faces"] and r2["ctas_per_sm"] == r["ctas_per_sm"]
    again = scenarios.new_wrenches(len(bodies))
    b2.compute(bodies, sc["ocean"], st, again)
    assert again.tobytes() == after.tobytes()
    b.close()
    b2.close()
    h.close()


def test_kernel_timing_events_leave_results_unchanged(built_library):
    from stonefish_gb300.hydro import HydroContext

    h = HydroContext(0)
    sc = scenarios.mixed_batch(n_bodies=48, seed=5, scale_faces=0.05)
    ids = np.asarray([h.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)[sc["bodies"]["mesh"]]
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids
    st = scenarios.settings()
    b = h.batch(ids)
    with pytest.raises(abi.HydroError):
        b.kernel_ms()                       # profiling off
    plain = scenarios.new_wrenches(len(bodies))
    b.compute(bodies, sc["ocean"], st, plain)
    b.profile(True)
    with pytest.raises(abi.HydroError):
        b.kernel_ms()                       # no step recorded yet
    timed = scenarios.new_wrenches(len(bodies))
    b.compute(bodies, sc["ocean"], st, timed)
    t = b.kernel_ms()
    assert t["prep"] > 0 and t["chunk"] > 0 and t["finalize"] > 0
    assert timed.tobytes() == plain.tobytes()
    b.profile(False)
    with pytest.raises(abi.HydroError):
        b.kernel_ms()
    b.close()
    h.close()
