"""Generates the golden fixtures in this directory from the CPU oracle.

The reference's own tests hold no active known-answer vectors for the
hydrodynamics path, so these fixtures pin the oracle (its FP32 reference
arithmetic REF32, the all-FP64 REF64 and the GPU-mirror MIRROR32 variants)
on small seeded cases: inputs (meshes, body tables, ocean, wave grid) and
outputs are stored together.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import MIRROR32, REF32, REF64, Oracle  # noqa: E402
from stonefish_gb300 import abi, meshes, scenarios  # noqa: E402


def ocean_array(o: abi.Ocean) -> np.ndarray:
    return np.frombuffer(bytes(o), dtype=np.uint8).copy()


def save(name, sc, settings=None):
    o = Oracle()
    st = settings or scenarios.settings()
    out = {}
    for tag, var in (("ref32", REF32), ("ref64", REF64), ("mirror32", MIRROR32)):
        io = scenarios.new_wrenches(len(sc["bodies"]))
        io["Fb"] = 0.5          # non-zero starting values exercise the stale-output rules
        io["Vsub"] = 0.25
        o.batch(var, 1, sc["bodies"], sc["meshes"], sc["ocean"], st, io, waves=sc.get("waves"))
        out[tag] = io
    arrays = {"bodies": sc["bodies"], "ocean": ocean_array(sc["ocean"]),
              "settings": np.array([st.damping_forces, st.realistic_buoyancy], np.int32)}
    for i, (x, f) in enumerate(sc["meshes"]):
        arrays[f"mesh{i}_xyz"] = x
        arrays[f"mesh{i}_faces"] = f
    if sc.get("waves") is not None:
        arrays["wave_data"] = sc["waves"]["data"]
        arrays["wave_layers"] = np.array(sc["waves"]["layers"], dtype=np.float64)
    for tag, io in out.items():
        arrays[tag] = io
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, {k: v.shape for k, v in arrays.items() if hasattr(v, "shape")})


def main():
    save("sphere_crossing", scenarios.single_sphere(steps=64, seed=101))
    save("sphere_inside", scenarios.single_sphere(steps=24, seed=102, depth=(0.55, 1.5)))
    save("sphere_no_damping", scenarios.single_sphere(steps=24, seed=103),
         scenarios.settings(damping=False))
    mb = scenarios.mixed_batch(n_bodies=12, seed=104, scale_faces=0.02)
    save("mixed_small", mb)
    tw = scenarios.torpedo_waves(n_bodies=12, seed=105, faces=800, grid_n=64)
    save("waves_small", tw)
    sc = scenarios.single_sphere(steps=16, seed=106)
    oc = sc["ocean"]
    oc.n_currents = 3
    c = oc.currents[1]
    c.type, c.enabled = abi.CURRENT_JET, 1
    c.point[:] = (-2.0, 0.0, 0.2)
    c.dir[:] = (1.0, 0.0, 0.0)
    c.radius, c.speed = 0.3, 2.0
    p = oc.currents[2]
    p.type, p.enabled = abi.CURRENT_PIPE, 1
    p.point[:] = (0.0, -2.0, 0.1)
    p.dir[:] = (0.0, 1.0, 0.0)
    p.radius, p.radius2, p.length, p.speed, p.gamma = 0.5, 1.0, 5.0, 1.5, 0.7
    save("currents_jet_pipe", sc)


if __name__ == "__main__":
    main()
