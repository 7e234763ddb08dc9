"""Error metrics and small builders shared by the tests."""
from __future__ import annotations

import numpy as np

from stonefish_gb300 import abi

FORCES = ("Fb", "Fdq", "Fdf")
TORQUES = ("Tb", "Tdq", "Tdf")


def scaled_errors(a: np.ndarray, c: np.ndarray, length, volume=None, surface=None) -> dict:
    """Per-body error of wrench array ``a`` against reference ``c``.

    Forces are measured against the body's force scale S = max(|Fb|, |Fdq|,
    |Fdf|) of the reference, torques against S * length (the torque a force
    of that size makes at the body's size); Swet and Vsub relatively, or,
    when the body's ``surface`` and ``volume`` are given, against those (a
    body barely in the water has a tiny Vsub summed from tetrahedra that
    cancel).  This is the pair-scaled relative error: components that cancel
    to ~0 are not divided by their own tiny size."""
    L = np.broadcast_to(np.asarray(length, dtype=np.float64), (len(c),))
    S = np.max(np.stack([np.linalg.norm(c[k], axis=1) for k in FORCES]), axis=0)
    S = np.maximum(S, 1e-300)
    out = {}
    for k in FORCES:
        out[k] = np.linalg.norm(a[k] - c[k], axis=1) / S
    for k in TORQUES:
        out[k] = np.linalg.norm(a[k] - c[k], axis=1) / (S * L)
    for k, ref in (("Swet", surface), ("Vsub", volume)):
        scale = np.abs(c[k]) if ref is None else np.maximum(np.abs(c[k]), np.asarray(ref, dtype=np.float64))
        out[k] = np.abs(a[k] - c[k]) / np.maximum(scale, 1e-300)
    return out


def max_scaled_error(a, c, length, mask=None) -> float:
    e = scaled_errors(a, c, length)
    m = np.ones(len(c), dtype=bool) if mask is None else mask
    return float(max(np.max(v[m]) if m.any() else 0.0 for v in e.values()))


def io_dict() -> dict:
    d = {k: np.zeros(3) for k in ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf")}
    d["Swet"] = np.zeros(1)
    d["Vsub"] = np.zeros(1)
    return d


def body_transform(body, which="T_CG") -> abi.Transform:
    t = abi.Transform()
    for i in range(9):
        t.basis[i] = float(body[which]["basis"][0][i])
    for i in range(3):
        t.origin[i] = float(body[which]["origin"][0][i])
    return t


from oracle.oracle import centred_scene  # noqa: E402,F401  (re-exported for the tests)
