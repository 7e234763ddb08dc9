"""The horizontally centred frame (HYDRO_FRAME_CENTRED) on the GPU.

The centred frame evaluates each body's faces relative to its CG's x and y
(rounded to FP32), which on a level ocean with position-independent currents
is the reference's own FP32 arithmetic applied to the body moved to the
origin.  So its face terms must equal the oracle's MIRROR32 terms of the
moved body bit for bit, its wrenches must match MIRROR32 on the moved bodies
within the usual 2e-6, and its error against the all-FP64 evaluation must
be far below the world frame's for bodies away from the origin."""
import numpy as np
import pytest

from oracle import MIRROR32, REF64
from stonefish_gb300 import abi, scenarios
from stonefish_gb300.hydro import HydroContext
from tests.helpers import body_transform, centred_scene, scaled_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hctx_centred(built_library):
    h = HydroContext(frame=abi.FRAME_CENTRED)
    yield h
    h.close()


def _run(h, sc, bodies=None, waves=None):
    if waves is not None:
        h.set_wave_grid(waves)
    ids = np.array([h.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)
    b = (sc["bodies"] if bodies is None else bodies).copy()
    b["mesh"] = ids[b["mesh"]]
    bt = h.batch(b["mesh"])
    io = scenarios.new_wrenches(len(b))
    bt.compute(b, sc["ocean"], scenarios.settings(), io)
    bt.close()
    return io


def _worst(e, act):
    return np.max(np.stack([v for v in e.values()]), axis=0)[act]


def test_face_terms_equal_oracle_on_the_moved_body(oracle, hctx_centred):
    sc = scenarios.mixed_batch(n_bodies=48, seed=61, scale_faces=0.05)
    moved = centred_scene(sc["bodies"])
    st = scenarios.settings()
    ids = [hctx_centred.upload_mesh(x, f) for x, f in sc["meshes"]]
    checked = 0
    for i in range(len(moved)):
        b = sc["bodies"][i:i + 1].copy()
        b["mesh"] = ids[int(b["mesh"][0])]
        mesh = sc["meshes"][int(sc["bodies"]["mesh"][i])]
        T = body_transform(moved[i:i + 1])
        TC = body_transform(moved[i:i + 1], "T_C")
        cpu = oracle.face_terms(MIRROR32, st, mesh, sc["ocean"], T, TC, moved["v"][i], moved["omega"][i])
        for packed in (False, True):
            gpu = hctx_centred.face_terms(b, sc["ocean"], st, packed=packed)
            assert np.array_equal(gpu, cpu), (i, packed)
        checked += int(np.any(cpu != 0))
    assert checked > 10


def test_wrenches_match_mirror_on_moved_bodies_and_beat_world_frame(oracle, hctx, hctx_centred):
    sc = scenarios.mixed_batch(n_bodies=512, seed=62, scale_faces=0.1)
    cen = _run(hctx_centred, sc)
    wor = _run(hctx, sc)
    moved = centred_scene(sc["bodies"])
    mir = scenarios.new_wrenches(len(moved))
    oracle.batch(MIRROR32, 8, moved, sc["meshes"], sc["ocean"], scenarios.settings(), mir)
    r64 = scenarios.new_wrenches(len(moved))
    oracle.batch(REF64, 8, sc["bodies"], sc["meshes"], sc["ocean"], scenarios.settings(), r64)
    assert np.array_equal(cen["position"], mir["position"])
    assert np.array_equal(cen["position"], wor["position"])
    act = cen["position"] != abi.OUTSIDE
    L = 0.5 * np.linalg.norm(sc["bodies"]["aabb_max"] - sc["bodies"]["aabb_min"], axis=1)
    for k, v in scaled_errors(cen, mir, L).items():
        assert np.max(v[act]) < 2e-6, k
    e_c = _worst(scaled_errors(cen, r64, L), act & (cen["position"] == abi.CROSSING_SURFACE))
    e_w = _worst(scaled_errors(wor, r64, L), act & (cen["position"] == abi.CROSSING_SURFACE))
    assert np.median(e_c) < 0.25 * np.median(e_w), (np.median(e_c), np.median(e_w))
    assert np.percentile(e_c, 99) <= 1e-5 and np.mean(e_c <= 1e-5) >= 0.99, (np.percentile(e_c, 99),
                                                                             np.mean(e_c <= 1e-5))


def test_waves_and_currents_in_the_centred_frame(oracle, hctx, hctx_centred):
    """With waves and a jet and pipe current the offset is added back for the
    wave lookups and the currents: the centred frame stays as close to FP64
    as the world frame (and closer at the median)."""
    sc = scenarios.torpedo_waves(n_bodies=96, seed=63, faces=2000, grid_n=256)
    oc = sc["ocean"]
    oc.n_currents = 2
    c = oc.currents[1]
    c.type, c.enabled = abi.CURRENT_JET, 1
    c.point[:] = (10.0, 10.0, 0.2)
    c.dir[:] = (1.0, 0.0, 0.0)
    c.radius, c.speed = 3.0, 2.0
    cen = _run(hctx_centred, sc, waves=sc["waves"])
    wor = _run(hctx, sc, waves=sc["waves"])
    r64 = scenarios.new_wrenches(len(sc["bodies"]))
    oracle.batch(REF64, 8, sc["bodies"], sc["meshes"], oc, scenarios.settings(), r64, waves=sc["waves"])
    act = (cen["position"] == abi.CROSSING_SURFACE)
    assert act.sum() > 20
    L = 0.5 * np.linalg.norm(sc["bodies"]["aabb_max"] - sc["bodies"]["aabb_min"], axis=1)
    e_c = _worst(scaled_errors(cen, r64, L), act)
    e_w = _worst(scaled_errors(wor, r64, L), act)
    assert np.median(e_c) <= np.median(e_w) and np.percentile(e_c, 99) <= max(2 * np.percentile(e_w, 99), 1e-5)
    assert np.percentile(e_c, 99) < 2e-5


def test_frame_argument_checked(hctx):
    with pytest.raises(abi.HydroError):
        hctx._ck(hctx.lib.hydro_set_frame(hctx.ctx, 7))
