"""The CUDA path against the committed golden fixtures (through the C ABI).

The fixtures hold the reference's own outputs (its SolidEntity code compiled
from source on the CPU) next to the oracle's."""
import numpy as np
import pytest

from stonefish_gb300 import abi, scenarios
from tests.golden_io import initial_io, load, load_face_patterns, names
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
    # against the reference's own outputs: same fluid positions, and per body
    # no further from them than the reference's FP32 sums are from FP64
    ref = g["out"]["reference"]
    assert np.array_equal(io["position"], ref["position"])
    e_vs_ref = scaled_errors(io, ref, L)
    e_ref64 = scaled_errors(ref, g["out"]["ref64"], L)
    for k in e_vs_ref:
        assert np.all(e_vs_ref[k][act] <= e_ref64[k][act] + 2e-6), (name, k)


@pytest.mark.parametrize("packed", [False, True])
def test_gpu_face_terms_equal_reference_single_faces(hctx, packed):
    """Single triangles -- the 27 depth-sign patterns of the waterline clip
    and 200 random ones on flat and wavy surfaces -- through the GPU's face
    code against the reference's ComputeHydrodynamicForcesSurface on the
    same face: with one face the reference's FP32 sums are the face's terms,
    so drag, friction and wetted area must match bit for bit, and so must
    the buoyancy and volume the reference derives from them."""
    fp = load_face_patterns()
    hctx.set_wave_grid(fp["waves"])
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    st = scenarios.settings()
    for i in range(len(fp["xyz"])):
        oc = scenarios.flat_ocean(tuple(fp["current"][i]))
        oc.waves = int(fp["waves_on"][i])
        body = fp["bodies"][i:i + 1].copy()
        body["mesh"] = hctx.upload_mesh(fp["xyz"][i], faces)
        t = hctx.face_terms(body, oc, st, packed=packed)[0]
        r = fp["reference"][i]
        for name, lo in (("Fdq", 6), ("Tdq", 9), ("Fdf", 12), ("Tdf", 15)):
            assert np.array_equal(t[lo:lo + 3].astype(np.float64), r[lo:lo + 3]), (i, name, t[lo:lo + 3], r[lo:lo + 3])
        assert np.float64(t[18]) == r[18], (i, "Swet")
        v6 = t[19]
        if v6 > np.float32(1e-9):      # SolidEntity.cpp:1689: buoyancy only when Vsub > 1e-9f
            assert np.float64(np.float32(v6 / np.float32(6.0))) == r[19], (i, "Vsub")
            if oc.waves:
                k = np.float32(oc.density * oc.gravity)
                assert np.array_equal((t[0:3] * k).astype(np.float64), r[0:3]), (i, "Fb")
                assert np.array_equal((t[3:6] * k).astype(np.float64), r[3:6]), (i, "Tb")
        else:
            assert r[19] == 0.0 and np.all(r[0:6] == 0.0), (i, "stale outputs")


def _outline_fixture():
    import os
    from tests.golden_io import GOLDEN
    return np.load(os.path.join(GOLDEN, "ref_outline.npz"))


def _split(points, counts):
    return np.split(points, np.cumsum(counts)[:-1])


def test_gpu_surface_outline_equals_reference_debug_points(hctx):
    """hydro_debug_surface_outline against the points the reference's
    DEBUG_HYDRO build records in ComputeHydrodynamicForcesSurface
    (tests/golden/ref_outline.npz): the outline of every evaluated submerged
    triangle or quad, faces in mesh order, bit for bit -- the 227 single-face
    cases (every clip case, flat and wavy surfaces, slivers) and whole
    meshes (an icosphere on a flat surface, torpedo hulls on waves)."""
    z = _outline_fixture()
    st = scenarios.settings()
    fp = load_face_patterns()
    hctx.set_wave_grid(fp["waves"])
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    for i, want in enumerate(_split(z["face_patterns_points"], z["face_patterns_count"])):
        oc = scenarios.flat_ocean(tuple(fp["current"][i]))
        oc.waves = int(fp["waves_on"][i])
        body = fp["bodies"][i:i + 1].copy()
        body["mesh"] = hctx.upload_mesh(fp["xyz"][i], faces)
        got = hctx.surface_outline(body, oc, st)
        assert np.array_equal(got, want), i
    for name in ("sphere_crossing", "waves_small"):
        g = load(name)
        if g["waves"] is not None:
            hctx.set_wave_grid(g["waves"])
        ids = [hctx.upload_mesh(x, f) for x, f in g["meshes"]]
        wants = _split(z[name + "_points"], z[name + "_count"])
        assert len(z[name + "_points"]) > 0
        for j, want in zip(z[name + "_bodies"], wants):
            # (a crossing body whose box dips under the surface but none of
            # whose faces does records no points, in the reference too)
            body = g["bodies"][j:j + 1].copy()
            body["mesh"] = ids[int(body["mesh"][0])]
            got = hctx.surface_outline(body, g["ocean"], st)
            assert np.array_equal(got, want), (name, int(j))
