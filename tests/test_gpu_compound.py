"""GPU parity of the batched Compound::ComputeHydrodynamicForces
(Compound.cpp:291-436) against the oracle (MIRROR32: the same FP32 face
terms with exact sums): per compound within 2e-6 of the force scale."""
import numpy as np
import pytest

from oracle import MIRROR32
from stonefish_gb300 import abi, scenarios
from stonefish_gb300.hydro import CompoundBatch

pytestmark = pytest.mark.gpu
TOL = 2e-6


def oracle_compounds(oracle, sc, settings, ppc=None):
    ppc = sc["parts_per_compound"] if ppc is None else ppc
    first = np.concatenate([[0], np.cumsum(ppc)[:-1]]).astype(int)
    out = scenarios.new_wrenches(len(ppc))
    for c in range(len(ppc)):
        parts = sc["parts"][first[c]:first[c] + int(ppc[c])]
        io = out[c:c + 1].copy()
        oracle.compound_forces(MIRROR32, sc["compounds"][c:c + 1], parts, [sc["meshes"][i] for i in parts["mesh"]],
                               sc["ocean"], settings, io)
        out[c] = io[0]
    return out


def check(gpu, ref, compounds):
    assert np.array_equal(gpu["position"], ref["position"])
    L = 0.5 * np.linalg.norm(compounds["aabb_max"] - compounds["aabb_min"], axis=1)
    S = np.max(np.stack([np.linalg.norm(ref[k], axis=1) for k in ("Fb", "Fdq", "Fdf")]), axis=0)
    act = (ref["position"] != abi.OUTSIDE) & (ref["position"] != abi.SKIPPED) & (S > 0)
    for k in ("Fb", "Fdq", "Fdf"):
        e = np.linalg.norm(gpu[k] - ref[k], axis=1)[act] / S[act]
        assert np.max(e, initial=0) < TOL, k
    for k in ("Tb", "Tdq", "Tdf"):
        e = np.linalg.norm(gpu[k] - ref[k], axis=1)[act] / (S[act] * L[act])
        assert np.max(e, initial=0) < TOL, k
    for k in ("Swet", "Vsub"):
        scale = np.maximum(np.abs(ref[k]), 1e-3)
        assert np.max(np.abs(gpu[k] - ref[k]) / scale) < 1e-5, k
    assert np.all(gpu["status"] == 0)


@pytest.mark.parametrize("flags", [(1, 1), (1, 0), (0, 1)])
def test_compound_batch_matches_oracle(oracle, hctx, flags):
    sc = scenarios.compound_batch(n_compounds=60, seed=21, faces_scale=0.3)
    ids = np.asarray([hctx.upload_mesh(*m) for m in sc["meshes"]], dtype=np.uint32)
    parts = sc["parts"].copy()
    parts["mesh"] = ids[sc["parts"]["mesh"]]
    st = scenarios.settings(damping=bool(flags[0]), buoyancy=bool(flags[1]))
    cb = CompoundBatch(hctx, parts["mesh"], sc["parts_per_compound"])
    gpu = scenarios.new_wrenches(60)
    gpu["Fb"] = 1.5          # untouched by the mode gate, kept by a stale rule
    cb.compute(sc["compounds"], parts, sc["ocean"], st, gpu)
    ref = scenarios.new_wrenches(60)
    ref["Fb"] = 1.5
    first = np.concatenate([[0], np.cumsum(sc["parts_per_compound"])[:-1]]).astype(int)
    for c in range(60):
        p = sc["parts"][first[c]:first[c] + int(sc["parts_per_compound"][c])]
        io = ref[c:c + 1].copy()
        oracle.compound_forces(MIRROR32, sc["compounds"][c:c + 1], p, [sc["meshes"][i] for i in p["mesh"]],
                               sc["ocean"], st, io)
        ref[c] = io[0]
    kinds = set(ref["position"].tolist())
    assert {abi.INSIDE, abi.OUTSIDE, abi.CROSSING_SURFACE, abi.SKIPPED} <= kinds
    check(gpu, ref, sc["compounds"])
    cb.close()


def test_compound_device_entry_and_empty_part_lists(oracle, hctx):
    torch = pytest.importorskip("torch")
    sc = scenarios.compound_batch(n_compounds=24, seed=22, faces_scale=0.3)
    ids = np.asarray([hctx.upload_mesh(*m) for m in sc["meshes"]], dtype=np.uint32)
    # every fourth compound loses its parts
    ppc = sc["parts_per_compound"].copy()
    first = np.concatenate([[0], np.cumsum(ppc)[:-1]]).astype(int)
    keep = np.ones(len(sc["parts"]), bool)
    for c in range(0, 24, 4):
        keep[first[c]:first[c] + ppc[c]] = False
        ppc[c] = 0
    sc = dict(sc, parts=sc["parts"][keep], parts_per_compound=ppc)
    parts = sc["parts"].copy()
    parts["mesh"] = ids[sc["parts"]["mesh"]]
    st = scenarios.settings()
    cb = CompoundBatch(hctx, parts["mesh"], ppc)
    d_c = torch.from_numpy(sc["compounds"].view(np.uint8).copy()).cuda()
    d_p = torch.from_numpy(parts.view(np.uint8).copy()).cuda()
    d_w = torch.zeros(24 * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    cb.compute_device(d_c.data_ptr(), d_p.data_ptr(), sc["ocean"], st, d_w.data_ptr(),
                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gpu = d_w.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
    ref = oracle_compounds(oracle, sc, st, ppc)
    check(gpu, ref, sc["compounds"])
    cb.close()
