"""GPU checks of the device rigid-body step against its CPU restatement, and
of a graph-captured rollout against the same steps issued one by one."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import rigid  # noqa: E402
from stonefish_gb300 import abi, scenarios  # noqa: E402
from stonefish_gb300 import rollout as RO  # noqa: E402
from stonefish_gb300 import surrogate as S  # noqa: E402

pytestmark = pytest.mark.gpu


def _dev_bytes(a):
    return torch.from_numpy(np.frombuffer(a.tobytes(), dtype=np.uint8).copy()).cuda()


def _host(t, dtype):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=dtype).copy()


@pytest.mark.parametrize("source", ["exact", "body", "none"])
def test_rigid_step_matches_oracle(hctx, source):
    rng = np.random.default_rng(4)
    n = 777
    st = RO.initial_states(rng, n)
    st["v"] = rng.uniform(-1, 1, (n, 3))
    st["w"] = rng.uniform(-0.5, 0.5, (n, 3))
    q = rng.normal(size=(n, 4))
    st["q"] = q / np.linalg.norm(q, axis=1)[:, None]
    bodies = RO.static_bodies(n, 0)
    ex = np.zeros(n, dtype=abi.WRENCH_DTYPE)
    for k in abi.WRENCH_VECTORS:
        ex[k] = rng.normal(size=(n, 3)) * 30.0
    bw = (rng.normal(size=(n, 6)) * 30.0).astype(np.float32)
    d_st, d_b, d_ex, d_bw = _dev_bytes(st), _dev_bytes(bodies), _dev_bytes(ex), torch.from_numpy(bw).cuda()
    dt, g = 0.01, 9.81
    P = RO._ptr
    st_ex = P(d_ex) if source == "exact" else None
    st_bw = P(d_bw) if source == "body" else None
    assert hctx.lib.hydro_rigid_step(hctx.ctx, P(d_st), P(d_b), st_ex, st_bw, n, dt, g, None) == 0
    torch.cuda.synchronize()
    R = rigid.quat_to_rot(st["q"])
    if source == "exact":
        F = ex["Fb"] + ex["Fdq"] + ex["Fdf"]
        T = np.einsum("nji,nj->ni", R, ex["Tb"] + ex["Tdq"] + ex["Tdf"])
    elif source == "body":
        F = np.einsum("nij,nj->ni", R, bw[:, :3].astype(np.float64))
        T = bw[:, 3:].astype(np.float64)
    else:
        F = np.zeros((n, 3))
        T = np.zeros((n, 3))
    ref = rigid.step(st, F, T, dt, g)
    got = _host(d_st, abi.RIGID_DTYPE)
    for k in ("p", "q", "v", "w"):
        assert np.allclose(got[k], ref[k], rtol=1e-12, atol=1e-12), k
    b = _host(d_b, abi.BODY_DTYPE)
    Rr, o, lo, hi = rigid.body_pose(ref)
    assert np.allclose(b["T_CG"]["basis"], Rr, atol=1e-12)
    assert np.allclose(b["T_C"]["origin"], o, atol=1e-12)
    assert np.allclose(b["R_O"], Rr, atol=1e-12)
    assert np.allclose(b["aabb_min"], lo, atol=1e-12) and np.allclose(b["aabb_max"], hi, atol=1e-12)
    assert np.array_equal(b["v"], got["v"]) and np.array_equal(b["omega"], got["w"])
    assert np.all(b["mode"] == abi.MODE_SUBMERGED)   # static fields untouched


def test_graph_rollout_equals_eager_steps(built_library):
    from stonefish_gb300.hydro import HydroContext

    h = HydroContext(0)
    xyz, fc = S.hull_mesh(2000)
    mid = h.upload_mesh(xyz, fc)
    h.set_wave_grid(scenarios.wave_grid(n=256))
    ocean, st = S.wave_ocean(), scenarios.settings()
    n, steps = 512, 30
    init = RO.initial_states(np.random.default_rng(7), n, extent=25.6, surface=RO.surface_z(h, ocean))
    a = RO.Rollout(h, mid, n, ocean, st, "exact")
    a.reset(init)
    for _ in range(steps):
        a.step()
    eager = a.host_states()
    b = RO.Rollout(h, mid, n, ocean, st, "exact")
    b.reset(init)
    kernels = b.capture(steps, snap_every=10)
    b.replay()
    graph = b.host_states()
    assert kernels == steps * 4
    assert graph.tobytes() == eager.tobytes()
    snaps = b.snapshots()
    assert len(snaps) == 3 and snaps[-1].tobytes() == graph.tobytes()
    # hulls moved and stayed finite
    assert np.all(np.isfinite(graph["p"]))
    assert np.max(np.linalg.norm(graph["p"] - init["p"], axis=1)) > 1e-3
    # replay from the same start reproduces the run
    b.reset(init)
    b.replay()
    assert b.host_states().tobytes() == graph.tobytes()
    a.close()
    b.close()
    h.close()
