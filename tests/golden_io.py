"""Loading of the golden fixtures in tests/golden (see make_golden.py)."""
import glob
import os

import numpy as np

from stonefish_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith("ref_"))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meshes = []
    i = 0
    while f"mesh{i}_xyz" in z:
        meshes.append((z[f"mesh{i}_xyz"], z[f"mesh{i}_faces"]))
        i += 1
    ocean = abi.Ocean.from_buffer_copy(z["ocean"].tobytes())
    st = abi.Settings(int(z["settings"][0]), int(z["settings"][1]))
    waves = None
    if "wave_data" in z:
        waves = {"data": z["wave_data"], "layers": [(int(c), float(g)) for c, g in z["wave_layers"]]}
    out = {k: z[k] for k in ("ref32", "ref64", "mirror32", "reference")}
    return {"meshes": meshes, "bodies": z["bodies"], "ocean": ocean, "settings": st, "waves": waves,
            "out": out}


def initial_io(n):
    io = np.zeros(n, dtype=abi.WRENCH_DTYPE)
    io["Fb"] = 0.5
    io["Vsub"] = 0.25
    return io


def load_face_patterns():
    """Single-face cases with the reference's outputs: columns Fb Tb Fdq Tdq
    Fdf Tdf (3 each), Swet, Vsub."""
    z = np.load(os.path.join(GOLDEN, "ref_face_patterns.npz"))
    waves = {"data": z["wave_data"], "layers": [(int(c), float(g)) for c, g in z["wave_layers"]]}
    return {"xyz": z["xyz"], "bodies": z["bodies"], "current": z["current"], "waves_on": z["waves"],
            "waves": waves, "reference": z["reference"]}
