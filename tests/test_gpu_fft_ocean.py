"""GPU FFT ocean (hydro_fft_ocean_*) against the oracle's restatement of the
reference's GL pipeline, and the hydrodynamics reading the field it writes."""
import numpy as np
import pytest

from oracle import MIRROR32, REF32
from stonefish_gb300 import abi, scenarios
from stonefish_gb300.hydro import FftOcean, HydroContext, fft_ocean_params
from tests.helpers import scaled_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("state,t", [(1.0, 0.0), (2.5, 7.3)])
def test_fft_ocean_matches_oracle(oracle, built_library, state, t):
    h = HydroContext(0)
    p = fft_ocean_params(state)
    fo = FftOcean(h, p)
    fo.update(t)
    gpu = fo.read()
    ref = oracle.fft_ocean(p, t)
    for c in range(4):
        scale = np.max(np.abs(ref[:, :, c]))
        # CUDA's and the host's cosf/sinf may differ in the last bit
        assert np.max(np.abs(gpu[:, :, c] - ref[:, :, c])) < 1e-4 * scale, c
    fo.close()
    h.close()


def test_hydrodynamics_on_the_fft_field(oracle, built_library):
    """Depths and a batched step read the field as the reference's
    ComputeWaveHeight does: channels 0 and 1 at grid sizes 893 m and 101 m."""
    h = HydroContext(0)
    p = fft_ocean_params(3.0)
    fo = FftOcean(h, p)
    fo.update(12.5)
    field = fo.read()
    waves = {"data": field, "layers": [(0, 893.0), (1, 101.0)]}
    ocean = scenarios.flat_ocean()
    ocean.waves = 1
    rng = np.random.default_rng(3)
    pts = np.stack([rng.uniform(-1000, 1000, 500), rng.uniform(-1000, 1000, 500), rng.uniform(-2, 2, 500)],
                   axis=1).astype(np.float32)
    d_gpu = h.depth(ocean, pts)
    d_ref = np.array([oracle.depth(ocean, waves, *map(float, q)) for q in pts], dtype=np.float32)
    assert np.array_equal(d_gpu, d_ref)
    sc = scenarios.torpedo_waves(n_bodies=24, faces=2000, grid_n=64)
    sc["waves"] = waves
    sc["ocean"] = ocean
    sc["bodies"]["T_CG"]["origin"][:, :2] = rng.uniform(-500, 500, (24, 2))
    sc["bodies"]["T_C"]["origin"][:, :2] = sc["bodies"]["T_CG"]["origin"][:, :2]
    half = 0.5 * (sc["bodies"]["aabb_max"] - sc["bodies"]["aabb_min"])
    c = sc["bodies"]["T_CG"]["origin"]
    sc["bodies"]["aabb_min"] = c - half
    sc["bodies"]["aabb_max"] = c + half
    mid = h.upload_mesh(*sc["meshes"][0])
    bodies = sc["bodies"].copy()
    bodies["mesh"] = mid
    b = h.batch(bodies["mesh"])
    gpu = scenarios.new_wrenches(24)
    b.compute(bodies, ocean, scenarios.settings(), gpu)
    ref = scenarios.new_wrenches(24)
    oracle.batch(MIRROR32, 4, sc["bodies"], sc["meshes"], ocean, scenarios.settings(), ref, waves=waves)
    assert np.array_equal(gpu["position"], ref["position"])
    L = 0.5 * np.linalg.norm(bodies["aabb_max"] - bodies["aabb_min"], axis=1)
    act = ref["position"] != abi.OUTSIDE
    assert act.sum() >= 5
    for k, v in scaled_errors(gpu, ref, L).items():
        assert np.max(v[act]) < 2e-6, k
    b.close()
    fo.close()
    h.close()
