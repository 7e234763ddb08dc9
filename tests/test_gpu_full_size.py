"""GPU parity at the benchmark's full sizes.

The mixed batch of 4096 bodies (37.8M faces, flat surface) and the 1024
torpedo hulls of 20000 faces on the 1024 x 1024 wave grid are evaluated in
one batched step each and compared, body by body, with the CPU oracle's
MIRROR32 variant (the reference's FP32 face arithmetic with exact sums)
over every body: same fluid positions, pair-scaled wrench errors (Swet and
Vsub against the body's surface and volume) within the same 2e-6 bar as the
small parity tests, and against the all-FP64 REF64 the
errors of the reference's own FP32 arithmetic.  Size-independent properties
are checked on the same runs: a repeated step gives the same bits and
bodies outside the water get zeros.  (With CG depths up to 0.3 m no body of
these workloads lies wholly under water; the INSIDE branch is covered by
the single-sphere tests.)
"""
import numpy as np
import pytest

from oracle import MIRROR32, REF64
from stonefish_gb300 import abi, scenarios
from tests.helpers import scaled_errors

pytestmark = pytest.mark.gpu

TOL_MIRROR = 2e-6


def _lengths(bodies):
    h = np.maximum(bodies["aabb_max"] - bodies["aabb_min"], 0)
    return 0.5 * np.linalg.norm(h, axis=1)


def _gpu_steps(sc, steps=2):
    from stonefish_gb300.hydro import HydroContext
    h = HydroContext()
    try:
        if sc.get("waves") is not None:
            h.set_wave_grid(sc["waves"])
        ids = np.array([h.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)
        bodies = sc["bodies"].copy()
        bodies["mesh"] = ids[sc["bodies"]["mesh"]]
        b = h.batch(bodies["mesh"])
        outs = []
        for _ in range(steps):
            io = scenarios.new_wrenches(len(bodies))
            b.compute(bodies, sc["ocean"], scenarios.settings(), io)
            outs.append(io)
        b.close()
        return outs
    finally:
        h.close()


def _oracle(oracle, variant, sc):
    io = scenarios.new_wrenches(len(sc["bodies"]))
    oracle.batch(variant, oracle.hardware_threads(), sc["bodies"], sc["meshes"], sc["ocean"],
                 scenarios.settings(), io, waves=sc.get("waves"))
    return io


def _check_against_oracle(oracle, sc, gpu, min_active):
    mir = _oracle(oracle, MIRROR32, sc)
    assert np.array_equal(gpu["position"], mir["position"])
    act = (gpu["position"] == abi.CROSSING_SURFACE) | (gpu["position"] == abi.INSIDE)
    assert act.sum() >= min_active
    L = _lengths(sc["bodies"])
    b = sc["bodies"]
    e = scaled_errors(gpu, mir, L, volume=b["volume"], surface=b["surface"])
    for k, v in e.items():
        assert np.max(v[act]) < TOL_MIRROR, (k, float(np.max(v[act])), int(np.argmax(np.where(act, v, 0))))
    r64 = _oracle(oracle, REF64, sc)
    e64 = scaled_errors(gpu, r64, L, volume=b["volume"], surface=b["surface"])
    worst = np.max(np.stack([v for v in e64.values()]), axis=0)[act]
    assert np.median(worst) < 1e-5 and np.percentile(worst, 99) < 1e-3, (np.median(worst), np.percentile(worst, 99))
    assert np.all(gpu["status"] == 0)
    return act


def test_mixed_batch_full_size(oracle, built_library):
    """The 4096-body mixed batch of the benchmark, every body against the oracle."""
    sc = scenarios.mixed_batch(n_bodies=4096, seed=1)
    first, second = _gpu_steps(sc)
    assert first.tobytes() == second.tobytes()
    act = _check_against_oracle(oracle, sc, first, min_active=2000)
    out = first["position"] == abi.OUTSIDE
    assert out.sum() > 500 and (act | out).all()
    for k in abi.WRENCH_VECTORS:
        assert np.all(first[k][out] == 0.0), k
    assert np.all(first["Swet"][out] == 0.0) and np.all(first["Vsub"][out] == 0.0)


def test_torpedo_waves_full_size(oracle, built_library):
    """The 1024 torpedo hulls of 20000 faces on the 1024 x 1024 wave grid."""
    sc = scenarios.torpedo_waves(n_bodies=1024, faces=20000, grid_n=1024)
    first, second = _gpu_steps(sc)
    assert first.tobytes() == second.tobytes()
    _check_against_oracle(oracle, sc, first, min_active=700)
