"""The debug-geometry fixture (tests/golden/ref_outline.npz) against the
reference itself: the points its DEBUG_HYDRO build records in
ComputeHydrodynamicForcesSurface, regenerated from the reference's code
compiled on this machine (oracle/_ref), must equal the committed ones.
Skipped where the reference's source tree is absent."""
import os

import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios
from tests.golden_io import GOLDEN, load, load_face_patterns
from tests.helpers import body_transform


def _fixture():
    return np.load(os.path.join(GOLDEN, "ref_outline.npz"))


def test_outline_fixture_shape():
    """Every recorded outline is a closed triangle or quad as segments: the
    points come in pairs and each segment starts where the previous one
    ended, within a face's run of 6 or 8 points."""
    z = _fixture()
    for name in ("face_patterns", "sphere_crossing", "waves_small"):
        pts, counts = z[name + "_points"], z[name + "_count"]
        assert pts.dtype == np.float32 and pts.shape[1] == 3
        assert int(counts.sum()) == len(pts) and np.all(counts % 2 == 0)
    # the single-face cases: 0, 6 or 8 points each (one triangle or quad)
    assert set(np.unique(z["face_patterns_count"])) <= {0, 6, 8}
    assert {6, 8} <= set(np.unique(z["face_patterns_count"]))


def test_outline_fixture_equals_reference():
    from oracle.ref import Reference
    if not Reference.available():
        pytest.skip("the reference's source tree is not present")
    ref = Reference()
    z = _fixture()
    st = scenarios.settings()

    def outline(body, mesh, ocean, waves):
        return ref.surface_outline(st, mesh, ocean, body_transform(body, "T_CG"), body_transform(body, "T_C"),
                                   body["v"][0], body["omega"][0], waves=waves)

    fp = load_face_patterns()
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    want = np.split(z["face_patterns_points"], np.cumsum(z["face_patterns_count"])[:-1])
    for i in range(len(fp["xyz"])):
        oc = scenarios.flat_ocean(tuple(fp["current"][i]))
        oc.waves = int(fp["waves_on"][i])
        got = outline(fp["bodies"][i:i + 1], (fp["xyz"][i], faces), oc, fp["waves"] if fp["waves_on"][i] else None)
        assert np.array_equal(got, want[i]), i
    for name in ("sphere_crossing", "waves_small"):
        g = load(name)
        b = g["bodies"]
        want = np.split(z[name + "_points"], np.cumsum(z[name + "_count"])[:-1])
        for j, w in zip(z[name + "_bodies"], want):
            assert g["out"]["reference"]["position"][j] == abi.CROSSING_SURFACE
            got = outline(b[j:j + 1], g["meshes"][int(b["mesh"][j])], g["ocean"], g["waves"])
            assert np.array_equal(got, w), (name, int(j))
