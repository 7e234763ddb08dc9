"""Generates the golden fixtures in this directory.

Each fixture holds a small seeded case -- inputs (meshes, body tables, ocean,
wave grid) and outputs together.  The outputs are those of the reference's
own hydrodynamics code (``reference``: SolidEntity.cpp and the functions it
calls, compiled from the reference's source tree by oracle/build_ref.py)
and of the oracle's variants (REF32, the reference's arithmetic restated;
REF64, all FP64; MIRROR32, the GPU kernel's arithmetic).
``ref_face_patterns.npz`` holds single triangles, one per case of the
waterline clip plus random ones on a flat and a wavy surface, with the
reference's per-face outputs.  Needs the reference's source tree; run from
the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import MIRROR32, REF32, REF64, Oracle  # noqa: E402
from oracle.ref import Reference  # noqa: E402
from stonefish_gb300 import abi, scenarios  # noqa: E402


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
    io = scenarios.new_wrenches(len(sc["bodies"]))
    io["Fb"] = 0.5
    io["Vsub"] = 0.25
    Reference().batch(1, sc["bodies"], sc["meshes"], sc["ocean"], st, io, waves=sc.get("waves"))
    out["reference"] = io
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
    save_face_patterns()
    save_ingest()
    save_outlines()


def ingest_meshes():
    """Synthetic physics meshes for the mass-property and coefficient-setup
    fixtures: sphere, box, capped cylinders along x and y, and a sphere with
    seeded radial noise (distinct principal moments)."""
    from stonefish_gb300 import meshes
    rng = np.random.default_rng(109)
    ico = meshes.build_icosphere(0.7, 3)
    bumpy = (ico[0] * (1.0 + 0.08 * rng.standard_normal((len(ico[0]), 1))).astype(np.float32)
             * np.array([1.0, 0.8, 0.6], np.float32), ico[1])
    cyl = meshes.capped_cylinder_for_faces(0.2, 1.6, 3000)
    ycyl = (np.ascontiguousarray(cyl[0][:, [1, 0, 2]] * np.array([-1.0, 1.0, 1.0], np.float32)), cyl[1])
    return {"sphere": ico, "box": meshes.build_box((0.3, 0.2, 0.5), 2), "cylinder_x": cyl,
            "cylinder_y": ycyl, "bumpy": bumpy}


def save_ingest():
    """The reference's ComputePhysicalProperties (solid and shell) and
    ComputeFluidDynamicsApprox (every approximation, rotated frames) on
    ingest_meshes()."""
    ref = Reference()
    rng = np.random.default_rng(110)
    arrays = {}
    for name, (xyz, faces) in ingest_meshes().items():
        arrays[f"{name}_xyz"] = xyz
        arrays[f"{name}_faces"] = faces
        props = []
        for th in (-1.0, 0.01):
            p = ref.mesh_properties((xyz, faces), th, 900.0)
            props.append(np.concatenate([[p["mass"], p["volume"], p["surface"]], p["CG"], p["Ipri"],
                                         p["Irot"].reshape(-1)]))
        arrays[f"{name}_props"] = np.array(props)
        frames, approx = [], []
        for trial in range(3):
            R1 = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0] if trial else np.eye(3)
            R2 = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))[0] if trial == 2 else np.eye(3)
            o1, o2, pcb = rng.uniform(-0.1, 0.1, 3), rng.uniform(-0.1, 0.1, 3), rng.uniform(-0.05, 0.05, 3)
            frames.append(np.concatenate([R1.reshape(-1), o1, R2.reshape(-1), o2, pcb]))
            t1, t2 = abi.Transform(), abi.Transform()
            for i in range(9):
                t1.basis[i], t2.basis[i] = float(R1.reshape(-1)[i]), float(R2.reshape(-1)[i])
            for i in range(3):
                t1.origin[i], t2.origin[i] = float(o1[i]), float(o2[i])
            for ap in (abi.APPROX_AUTO, abi.APPROX_SPHERE, abi.APPROX_CYLINDER, abi.APPROX_ELLIPSOID):
                a = ref.fluid_approx((xyz, faces), ap, t1, t2, pcb, 1025.0)
                par = np.zeros(3)
                par[:len(a["params"])] = a["params"]
                approx.append(np.concatenate([[ap, a["type"], len(a["params"])], par, a["R_CG2H"].reshape(-1),
                                              a["origin_CG2H"], a["added_mass"], a["added_inertia"], a["Cd"],
                                              a["Cf"]]))
        arrays[f"{name}_frames"] = np.array(frames)
        arrays[f"{name}_approx"] = np.array(approx)
    np.savez_compressed(os.path.join(HERE, "ref_ingest.npz"), **arrays)
    print("ref_ingest", sorted(arrays))


def save_face_patterns():
    """Single-face bodies through the reference's ComputeHydrodynamicForcesSurface:
    the 27 depth-sign patterns of one triangle on a flat surface, then random
    triangles (every 7th a sliver) on a flat surface and on a wave grid."""
    from tests.helpers import body_transform, io_dict
    ref = Reference()
    rng = np.random.default_rng(107)
    waves = scenarios.wave_grid(n=64, n_waves=8, seed=108)
    base = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 1.0, 0.0]], dtype=np.float32)
    levels = (-0.3, 0.0, 0.25)
    xyz, bodies, oceans, wavy = [], [], [], []
    for za in levels:
        for zb in levels:
            for zc in levels:
                p = base.copy()
                p[:, 2] = (za, zb, zc)
                xyz.append(p)
                bodies.append(scenarios.fill_bodies(1, np.eye(3)[None], np.zeros((1, 3)), np.array([[0.3, -0.2, 0.1]]),
                                                    np.array([[0.1, 0.2, -0.3]]), np.ones((1, 3)), 1.0, 1.0, (1, 1, 1),
                                                    (.1, .1, .1), 0))
                oceans.append((0.2, 0.1, -0.3))
                wavy.append(0)
    for t in range(200):
        p = rng.uniform(-1.0, 1.0, (3, 3)).astype(np.float32)
        p[:, 2] = rng.uniform(-0.6, 0.6, 3).astype(np.float32)
        if t % 7 == 0:
            p[2] = p[0] + np.float32(1e-4) * (p[1] - p[0])
        xyz.append(p)
        R = scenarios.quat_to_matrix(scenarios.random_quaternions(rng, 1))
        pos = np.array([[rng.uniform(0, 6.4), rng.uniform(0, 6.4), rng.uniform(-0.3, 0.3)]])
        bodies.append(scenarios.fill_bodies(1, R, pos, rng.uniform(-1, 1, (1, 3)), rng.uniform(-0.5, 0.5, (1, 3)),
                                            np.ones((1, 3)), 1.0, 1.0, (1, 1, 1), (.1, .1, .1), 0))
        oceans.append(tuple(rng.uniform(-0.5, 0.5, 3)))
        wavy.append(t % 2)
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    keys = ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf", "Swet", "Vsub")
    out = np.zeros((len(xyz), 20))
    for i, (p, b) in enumerate(zip(xyz, bodies)):
        oc = scenarios.flat_ocean(oceans[i])
        oc.waves = wavy[i]
        io = io_dict()
        T = body_transform(b)
        ref.surface_forces(scenarios.settings(), (p, faces), oc, T, T, b["v"][0], b["omega"][0], io,
                           waves=waves if wavy[i] else None)
        out[i] = np.concatenate([io[k] for k in keys])
    np.savez_compressed(os.path.join(HERE, "ref_face_patterns.npz"), xyz=np.stack(xyz),
                        bodies=np.concatenate(bodies), current=np.array(oceans), waves=np.array(wavy, np.int32),
                        wave_data=waves["data"], wave_layers=np.array(waves["layers"], dtype=np.float64),
                        reference=out)
    print("ref_face_patterns", len(xyz))


def save_outlines():
    """The points the reference's DEBUG_HYDRO build records in
    ComputeHydrodynamicForcesSurface (outlines of the evaluated submerged
    parts) for bodies of three fixtures: the 227 single-face cases of
    ref_face_patterns.npz, the first four crossing bodies of
    sphere_crossing.npz and the first four of waves_small.npz."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from tests import golden_io
    from tests.helpers import body_transform
    ref = Reference()
    st = scenarios.settings()
    arrays = {}

    def outline(body, mesh, ocean, waves):
        return ref.surface_outline(st, mesh, ocean, body_transform(body, "T_CG"), body_transform(body, "T_C"),
                                   body["v"][0], body["omega"][0], waves=waves)

    fp = golden_io.load_face_patterns()
    faces = np.array([[0, 1, 2]], dtype=np.uint32)
    pts = []
    for i in range(len(fp["xyz"])):
        oc = scenarios.flat_ocean(tuple(fp["current"][i]))
        oc.waves = int(fp["waves_on"][i])
        pts.append(outline(fp["bodies"][i:i + 1], (fp["xyz"][i], faces), oc,
                           fp["waves"] if fp["waves_on"][i] else None))
    arrays["face_patterns_count"] = np.array([len(q) for q in pts], np.int64)
    arrays["face_patterns_points"] = np.concatenate(pts)
    for name in ("sphere_crossing", "waves_small"):
        g = golden_io.load(name)
        b = g["bodies"]
        sel = [i for i in range(len(b)) if g["out"]["reference"]["position"][i] == abi.CROSSING_SURFACE][:4]
        pts = [outline(b[i:i + 1], g["meshes"][int(b["mesh"][i])], g["ocean"], g["waves"]) for i in sel]
        arrays[name + "_bodies"] = np.array(sel, np.int64)
        arrays[name + "_count"] = np.array([len(q) for q in pts], np.int64)
        arrays[name + "_points"] = np.concatenate(pts)
    np.savez_compressed(os.path.join(HERE, "ref_outline.npz"), **arrays)
    print("ref_outline", {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
