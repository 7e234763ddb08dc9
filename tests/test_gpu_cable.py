"""GPU parity of CableEntity::ComputeHydrodynamicForces
(CableEntity.cpp:240-376) against the oracle: FP64 per node, within 1e-12 of
each cable's force scale (CUDA's and the host's double-precision sin, cos,
acos and atan may differ in the last bit)."""
import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [(1, 1), (0, 1), (1, 0)])
def test_cables_match_oracle(oracle, hctx, flags):
    sc = scenarios.cable_set(n_cables=96, seed=7)
    st = scenarios.settings(damping=bool(flags[0]), buoyancy=bool(flags[1]))
    n = len(sc["x"])
    gpu = np.zeros(n, dtype=abi.CABLE_FORCES_DTYPE)
    gpu["Fb"] = 9.0                   # the disabled cable keeps it
    ref = gpu.copy()
    hctx.cable_forces(sc["cables"], sc["x"], sc["v"], sc["ocean"], st, gpu)
    oracle.cable_forces(sc["cables"], sc["x"], sc["v"], sc["ocean"], st, ref)
    for c in sc["cables"]:
        sl = slice(int(c["first_node"]), int(c["first_node"] + c["n_nodes"]))
        scale = max(np.abs(ref["Fb"][sl]).max(), np.abs(ref["Fdq"][sl]).max(), np.abs(ref["Fdf"][sl]).max(), 1e-300)
        for k in ("Fb", "Fdq", "Fdf"):
            assert np.max(np.abs(gpu[k][sl] - ref[k][sl])) <= 1e-12 * scale, (k, int(c["first_node"]))
    last = sc["cables"][-1]
    assert np.all(gpu["Fb"][int(last["first_node"]):] == 9.0)


def test_cable_node_range_checked(hctx):
    cables = np.zeros(1, dtype=abi.CABLE_DTYPE)
    cables["n_nodes"] = 5
    cables["radius"] = 0.05
    cables["mode"] = abi.MODE_SUBMERGED
    out = np.zeros(3, dtype=abi.CABLE_FORCES_DTYPE)
    with pytest.raises(abi.HydroError) as ei:
        hctx.cable_forces(cables, np.zeros((3, 3)), np.zeros((3, 3)), scenarios.flat_ocean(), scenarios.settings(),
                          out)
    assert ei.value.status == abi.HYDRO_ERR_INDEX_RANGE
