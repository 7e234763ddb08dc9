"""The CPU oracle reproduces the committed golden fixtures (no GPU).

The fixtures hold the outputs of the reference's own code (``reference``,
compiled from its source tree) and of the oracle's variants on small seeded
cases.  The oracle's REF32 must give the reference's bits, and each variant
its own stored bits.  The FP32 and FP64 arithmetic is plain IEEE (+, -, *,
/, sqrt) and gives the same bits on every host, so the comparison is exact
except where a case uses exp/pow (jet and pipe currents), whose last bit may
differ between C libraries."""
import numpy as np
import pytest

from oracle import MIRROR32, REF32, REF64
from stonefish_gb300 import abi
from tests.golden_io import initial_io, load, names

VARIANTS = {"ref32": REF32, "ref64": REF64, "mirror32": MIRROR32, "reference": REF32}


@pytest.mark.parametrize("name", names())
@pytest.mark.parametrize("tag", sorted(VARIANTS))
def test_oracle_reproduces_golden(oracle, name, tag):
    g = load(name)
    io = initial_io(len(g["bodies"]))
    oracle.batch(VARIANTS[tag], 1, g["bodies"], g["meshes"], g["ocean"], g["settings"], io,
                 waves=g["waves"])
    ref = g["out"][tag]
    assert np.array_equal(io["position"], ref["position"])
    for k in list(abi.WRENCH_VECTORS) + ["Swet", "Vsub"]:
        if name == "currents_jet_pipe":
            np.testing.assert_allclose(io[k], ref[k], rtol=1e-9, atol=1e-12, err_msg=k)
        else:
            assert np.array_equal(io[k], ref[k]), (name, tag, k)


def test_golden_cases_cover_every_branch():
    seen = set()
    for name in names():
        g = load(name)
        seen.update(np.unique(g["out"]["ref32"]["position"]).tolist())
    assert {abi.INSIDE, abi.OUTSIDE, abi.CROSSING_SURFACE} <= seen


@pytest.mark.parametrize("name", names())
def test_reference_outputs_equal_ref32(name):
    """Stored outputs of the reference's code and of REF32, made on one host."""
    g = load(name)
    for k in list(abi.WRENCH_VECTORS) + ["Swet", "Vsub", "position"]:
        assert np.array_equal(g["out"]["reference"][k], g["out"]["ref32"][k]), (name, k)
