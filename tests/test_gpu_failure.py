"""Failure detection without a GPU fault: a bounded device wait that nothing
completes reports HYDRO_ERR_TIMEOUT and the context keeps working; host-side
failures (bad arguments, unknown meshes) return status codes without a
launch."""
import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_stays_usable(hctx):
    assert hctx.wait_timeout(20000) == abi.HYDRO_ERR_TIMEOUT
    # the context still computes
    sc = scenarios.single_sphere(steps=8, seed=4)
    mid = hctx.upload_mesh(*sc["meshes"][0])
    b = sc["bodies"].copy()
    b["mesh"] = mid
    bt = hctx.batch(b["mesh"])
    io = scenarios.new_wrenches(len(b))
    bt.compute(b, sc["ocean"], scenarios.settings(), io)
    assert np.all(io["status"] == 0)
    bt.close()


def test_host_side_errors_do_not_launch(hctx, built_library):
    from stonefish_gb300.hydro import HydroContext
    with pytest.raises(abi.HydroError) as ei:
        hctx.wait_timeout(0)
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG
    fresh = HydroContext()
    oc = scenarios.flat_ocean()
    oc.waves = 1          # waves requested but no grid was given
    with pytest.raises(abi.HydroError) as ei:
        fresh.depth(oc, np.zeros((4, 3), np.float32))
    assert ei.value.status == abi.HYDRO_ERR_INVALID_ARG
    fresh.close()
