"""Seeded synthetic workloads for the hydrodynamics path.

Each builder returns meshes, a body table (``abi.BODY_DTYPE``), an ocean
(``abi.Ocean``) and, for the wave workload, a height grid.  The shapes and
distributions are those of the benchmark workloads:

* ``single_sphere``   one icosphere r=0.5 m (1280 faces), flat surface,
  uniform current (0.2,0,0) m/s, 1000 seeded steps with CG depth
  U(-1.0,+0.3) m (``depth=(0.5,1.5)`` gives the fully submerged variant),
  uniform random orientation, v ~ U(-1,1)^3 m/s, omega ~ U(-0.5,0.5)^3 rad/s;
* ``mixed_batch``     4096 bodies with distinct meshes: icospheres
  (320-20480 faces), boxes (12-49152 faces), capped cylinders 1.6 m x 0.2 m
  (500-50000 faces), about 37M faces in total, poses as above;
* ``torpedo_waves``   1024 torpedo hulls (2 m x 0.25 m, hemispherical caps,
  20000 faces, one shared mesh) over a 1024 x 1024 height grid at 0.1 m
  built from 64 sinusoids with JONSWAP amplitudes (Hs=1 m, Tp=6 s), CG depth
  U(-0.5,+0.2) m.

Body state follows the reference's primitive solids: the physics-mesh frame
is the CG frame (T_CG2C = I, Sphere.cpp:37-40), the origin frame equals the
CG frame, P_CB = 0, and the AABB is Bullet's compound-shape box
centre +- |R| h (3rdparty/BulletCollision/CollisionShapes/btCompoundShape.cpp
:161-181) of the child shape's local half extents h.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi, meshes

RHO_WATER = 1025.0
GRAVITY = 9.81


# ------------------------------------------------------------------ math
def quat_to_matrix(q: np.ndarray) -> np.ndarray:
    """Rotation matrices (n,3,3) of unit quaternions (n,4) ordered (x,y,z,w)."""
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotations (Shoemake's subgroup algorithm)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    return np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                     b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)


def compound_aabb(R: np.ndarray, origin: np.ndarray, half: np.ndarray):
    """btCompoundShape::getAabb with margin 0 and the child box centred at the
    CG: extent = h . |R row|, min/max = origin -+ extent (float64, Bullet's
    left-to-right dot)."""
    A = np.abs(R)
    ext = half[:, None, 0] * A[:, :, 0] + half[:, None, 1] * A[:, :, 1] + half[:, None, 2] * A[:, :, 2]
    return origin - ext, origin + ext


def flat_ocean(current=(0.2, 0.0, 0.0), density=RHO_WATER, gravity=GRAVITY) -> abi.Ocean:
    o = abi.Ocean()
    o.density = density
    o.gravity = gravity
    o.waves = 0
    if current is not None:
        o.currents_enabled = 1
        o.n_currents = 1
        o.currents[0].type = abi.CURRENT_UNIFORM
        o.currents[0].enabled = 1
        for k in range(3):
            o.currents[0].vel[k] = current[k]
    return o


def settings(damping=True, buoyancy=True) -> abi.Settings:
    return abi.Settings(int(damping), int(buoyancy))


def fill_bodies(n: int, R: np.ndarray, pos: np.ndarray, v: np.ndarray, w: np.ndarray,
                half: np.ndarray, volume, surface, Cd, Cf, mesh_ids,
                mode=abi.MODE_SUBMERGED, buoyancy=1) -> np.ndarray:
    b = np.zeros(n, dtype=abi.BODY_DTYPE)
    Rf = R.reshape(n, 9)
    b["T_CG"]["basis"] = Rf
    b["T_CG"]["origin"] = pos
    b["T_C"]["basis"] = Rf
    b["T_C"]["origin"] = pos
    b["R_O"] = Rf
    b["v"] = v
    b["omega"] = w
    b["Cd"] = Cd
    b["Cf"] = Cf
    b["volume"] = volume
    b["surface"] = surface
    mn, mx = compound_aabb(R, pos, half)
    b["aabb_min"] = mn
    b["aabb_max"] = mx
    b["mesh"] = mesh_ids
    b["mode"] = mode
    b["buoyancy"] = buoyancy
    return b


def random_states(rng: np.random.Generator, n: int, depth=(-1.0, 0.3), xy=0.0):
    q = random_quaternions(rng, n)
    R = quat_to_matrix(q)
    pos = np.zeros((n, 3))
    if xy:
        pos[:, 0] = rng.uniform(-xy, xy, n)
        pos[:, 1] = rng.uniform(-xy, xy, n)
    pos[:, 2] = rng.uniform(depth[0], depth[1], n)
    v = rng.uniform(-1.0, 1.0, (n, 3))
    w = rng.uniform(-0.5, 0.5, (n, 3))
    return R, pos, v, w


def new_wrenches(n: int) -> np.ndarray:
    return np.zeros(n, dtype=abi.WRENCH_DTYPE)


# ------------------------------------------------------ single sphere
def single_sphere(steps: int = 1000, seed: int = 0, depth=(-1.0, 0.3), radius=0.5,
                  subdivisions=3):
    """One icosphere stepped through ``steps`` seeded states (one body per step)."""
    rng = np.random.default_rng(seed)
    xyz, faces = meshes.build_icosphere(radius, subdivisions)
    R, pos, v, w = random_states(rng, steps, depth)
    half = np.full((steps, 3), radius)
    vol = 4.0 / 3.0 * math.pi * radius ** 3       # Sphere.cpp:55
    surf = 4.0 * math.pi * radius ** 2            # Sphere.cpp:56
    bodies = fill_bodies(steps, R, pos, v, w, half, vol, surf, (1.0, 1.0, 1.0),
                         (0.1, 0.1, 0.1), 0)      # SolidEntity.cpp:753-755
    return {"meshes": [(xyz, faces)], "bodies": bodies, "ocean": flat_ocean(), "waves": None}


# --------------------------------------------------------- mixed batch
def _cylinder_levels():
    return np.unique(np.round(np.geomspace(500, 50000, 24)).astype(int))


def mixed_batch(n_bodies: int = 4096, seed: int = 1, depth=(-1.0, 0.3), xy=50.0,
                scale_faces: float = 1.0):
    """Batch of bodies with distinct meshes drawn from three families.

    ``scale_faces`` < 1 shrinks every family's face counts (for quick tests)."""
    rng = np.random.default_rng(seed)
    ico_levels = [2, 3, 4, 5]
    box_levels = [0, 1, 2, 3, 4, 5, 6]
    cyl_levels = _cylinder_levels()
    if scale_faces < 1.0:
        ico_levels = [s for s in ico_levels if 20 * 4 ** s <= max(320, 20480 * scale_faces)]
        box_levels = [k for k in box_levels if 12 * 4 ** k <= max(12, 49152 * scale_faces)]
        cyl_levels = [f for f in cyl_levels if f <= max(500, 50000 * scale_faces)]
    ico_cat = {s: meshes.build_icosphere(1.0, s) for s in ico_levels}
    box_cat = {k: meshes.build_box((1.0, 1.0, 1.0), k) for k in box_levels}
    cyl_cat = {int(f): meshes.capped_cylinder_for_faces(0.2, 1.6, int(f)) for f in cyl_levels}

    fam = rng.integers(0, 3, n_bodies)
    R, pos, v, w = random_states(rng, n_bodies, depth, xy)
    half = np.zeros((n_bodies, 3))
    vol = np.zeros(n_bodies)
    surf = np.zeros(n_bodies)
    Cd = np.zeros((n_bodies, 3))
    mesh_list = []
    for i in range(n_bodies):
        if fam[i] == 0:
            s = ico_levels[rng.integers(len(ico_levels))]
            r = rng.uniform(0.3, 0.7)
            xyz, faces = ico_cat[s]
            mesh_list.append(((xyz * np.float32(r)).astype(np.float32), faces))
            half[i] = r
            vol[i] = 4.0 / 3.0 * math.pi * r ** 3
            surf[i] = 4.0 * math.pi * r * r
            Cd[i] = (1.0, 1.0, 1.0)
        elif fam[i] == 1:
            k = box_levels[rng.integers(len(box_levels))]
            h = rng.uniform(0.15, 0.6, 3)
            xyz, faces = box_cat[k]
            mesh_list.append(((xyz * h.astype(np.float32)).astype(np.float32), faces))
            half[i] = h
            vol[i] = 8.0 * h[0] * h[1] * h[2]                                   # Box.cpp:66
            surf[i] = 8.0 * (h[0] * h[1] + h[0] * h[2] + h[1] * h[2])           # Box.cpp:67
            inv = 1.0 / h
            Cd[i] = inv / inv.max()                                             # SolidEntity.cpp:1014-1019
        else:
            f = int(cyl_levels[rng.integers(len(cyl_levels))])
            sc = rng.uniform(0.8, 1.25)
            xyz, faces = cyl_cat[f]
            mesh_list.append(((xyz * np.float32(sc)).astype(np.float32), faces))
            r, L = 0.2 * sc, 1.6 * sc
            half[i] = (0.5 * L + r, r, r)
            vol[i] = meshes.capped_cylinder_volume(r, L)
            surf[i] = meshes.capped_cylinder_surface(r, L)
            Cd[i] = (1.0, 0.5, 0.5)      # cylinder Cd (0.5,0.5,1) with the axis on x, :841-844
    bodies = fill_bodies(n_bodies, R, pos, v, w, half, vol, surf, Cd, 0.1 * Cd,
                         np.arange(n_bodies, dtype=np.uint32))
    return {"meshes": mesh_list, "bodies": bodies, "ocean": flat_ocean(), "waves": None}


# ---------------------------------------------------------------- waves
def jonswap(omega: np.ndarray, hs: float, tp: float, gamma: float = 3.3) -> np.ndarray:
    """JONSWAP spectral density S(omega) [m^2 s] (Hasselmann et al. 1973, in the
    Hs/Tp form with the normalisation A_gamma = 1 - 0.287 ln gamma)."""
    wp = 2.0 * math.pi / tp
    sigma = np.where(omega <= wp, 0.07, 0.09)
    pm = 5.0 / 16.0 * hs * hs * wp ** 4 * omega ** -5.0 * np.exp(-1.25 * (omega / wp) ** -4.0)
    peak = gamma ** np.exp(-((omega - wp) ** 2) / (2.0 * sigma * sigma * wp * wp))
    return (1.0 - 0.287 * math.log(gamma)) * pm * peak


def wave_grid(n: int = 1024, spacing: float = 0.1, n_waves: int = 64, hs: float = 1.0,
              tp: float = 6.0, seed: int = 7) -> dict:
    """Periodic height field h(x,y) (elevation, up positive) sampled at texel
    centres x_i = (i + 0.5) * spacing.  Each of the 64 sinusoids has a random
    direction and phase, an angular frequency spread over [0.5, 3] omega_p and
    amplitude sqrt(2 S(omega) d omega); its wave vector (deep-water dispersion
    k = omega^2 / g) is snapped to the grid's reciprocal lattice so that the
    field is exactly periodic over the n*spacing square."""
    rng = np.random.default_rng(seed)
    L = n * spacing
    wp = 2.0 * math.pi / tp
    edges = np.linspace(0.5 * wp, 3.0 * wp, n_waves + 1)
    om = 0.5 * (edges[1:] + edges[:-1])
    dom = edges[1:] - edges[:-1]
    amp = np.sqrt(2.0 * jonswap(om, hs, tp) * dom)
    theta = rng.uniform(0.0, 2.0 * math.pi, n_waves)
    phase = rng.uniform(0.0, 2.0 * math.pi, n_waves)
    k = om * om / GRAVITY
    dk = 2.0 * math.pi / L
    mx = np.round(k * np.cos(theta) / dk)
    my = np.round(k * np.sin(theta) / dk)
    zero = (mx == 0) & (my == 0)
    mx[zero] = 1.0
    x = (np.arange(n) + 0.5) * spacing
    h = np.zeros((n, n))
    for a, kx, ky, ph in zip(amp, mx * dk, my * dk, phase):
        h += a * np.cos(kx * x[None, :] + ky * x[:, None] + ph)
    return {"data": h.astype(np.float32), "layers": [(0, float(np.float32(L)))]}


def torpedo_waves(n_bodies: int = 1024, seed: int = 2, depth=(-0.5, 0.2), faces=20000,
                  grid_n: int = 1024):
    rng = np.random.default_rng(seed)
    r, L = 0.25, 2.0
    xyz, fc = meshes.capped_cylinder_for_faces(r, L, faces)
    waves = wave_grid(n=grid_n)
    R, pos, v, w = random_states(rng, n_bodies, depth)
    extent = grid_n * 0.1
    pos[:, 0] = rng.uniform(0.0, extent, n_bodies)
    pos[:, 1] = rng.uniform(0.0, extent, n_bodies)
    half = np.tile([0.5 * L + r, r, r], (n_bodies, 1))
    bodies = fill_bodies(n_bodies, R, pos, v, w, half, meshes.capped_cylinder_volume(r, L),
                         meshes.capped_cylinder_surface(r, L), (1.0, 0.5, 0.5),
                         (0.1, 0.05, 0.05), 0)
    ocean = flat_ocean()
    ocean.waves = 1
    return {"meshes": [(xyz, fc)], "bodies": bodies, "ocean": ocean, "waves": waves}


def compound_batch(n_compounds: int = 64, seed: int = 5, depth=(-0.8, 0.8), faces_scale: float = 1.0):
    """Seeded AUV-like compounds for Compound::ComputeHydrodynamicForces
    (Compound.cpp:291-436): an external buoyant hull (capped cylinder), two
    external pontoons (boxes), an internal buoyant ballast block and, on
    every third compound, a part whose mode takes it out of the fluid
    computation.  The compound's origin frame is its CG frame; each part
    sits at a fixed offset (origin) in it.  Returns meshes, compounds
    (hydro_body, one per compound), parts (hydro_compound_part) with mesh
    indices into meshes, parts_per_compound and a flat ocean."""
    rng = np.random.default_rng(seed)
    hull = meshes.capped_cylinder_for_faces(0.2, 1.2, max(200, int(3000 * faces_scale)))
    pontoon = meshes.build_box((0.5, 0.08, 0.06), 2 if faces_scale < 1 else 3)
    ballast = meshes.build_box((0.3, 0.1, 0.05), 1)
    mesh_list = [hull, pontoon, ballast]
    vol = (meshes.capped_cylinder_volume(0.2, 1.2), 8 * 0.5 * 0.08 * 0.06, 8 * 0.3 * 0.1 * 0.05)
    area = (meshes.capped_cylinder_surface(0.2, 1.2), 8 * (0.5 * 0.08 + 0.5 * 0.06 + 0.08 * 0.06),
            8 * (0.3 * 0.1 + 0.3 * 0.05 + 0.1 * 0.05))
    R, pos, v, w = random_states(rng, n_compounds, depth)
    compounds = np.zeros(n_compounds, dtype=abi.BODY_DTYPE)
    half_c = np.array([0.9, 0.45, 0.25])
    parts = []
    counts = []
    for c in range(n_compounds):
        Rc = R[c]
        layout = [  # (mesh, offset, external, buoyant, mode, Cd, Cf)
            (0, (0.0, 0.0, 0.0), 1, 1, abi.MODE_SUBMERGED, (1.0, 0.5, 0.5), (0.1, 0.05, 0.05)),
            (1, (0.0, 0.35, 0.15), 1, 1, abi.MODE_SUBMERGED, (0.3, 1.0, 1.0), (0.03, 0.1, 0.1)),
            (1, (0.0, -0.35, 0.15), 1, 1, abi.MODE_FLOATING, (0.3, 1.0, 1.0), (0.03, 0.1, 0.1)),
            (2, (0.1, 0.0, -0.05), 0, 1, abi.MODE_SUBMERGED, (1.0, 1.0, 1.0), (0.1, 0.1, 0.1)),
        ]
        if c % 3 == 0:
            layout.append((1, (0.0, 0.0, -0.3), 1, 1, abi.MODE_DISABLED, (1.0, 1.0, 1.0), (0.1, 0.1, 0.1)))
        for mi, off, ext, buoy, mode, cd, cf in layout:
            p = np.zeros(1, dtype=abi.COMPOUND_PART_DTYPE)
            p["T_C"]["basis"] = Rc.reshape(9)
            p["T_C"]["origin"] = pos[c] + Rc @ np.asarray(off)
            p["R_O"] = Rc.reshape(9)
            p["Cd"] = cd
            p["Cf"] = cf
            p["mesh"] = mi
            p["mode"] = mode
            p["buoyant"] = buoy
            p["external"] = ext
            parts.append(p)
        counts.append(len(layout))
    compounds["T_CG"]["basis"] = R.reshape(n_compounds, 9)
    compounds["T_CG"]["origin"] = pos
    compounds["T_C"] = compounds["T_CG"]
    compounds["R_O"] = R.reshape(n_compounds, 9)
    compounds["v"] = v
    compounds["omega"] = w
    compounds["volume"] = vol[0] + 2 * vol[1] + vol[2]
    compounds["surface"] = area[0] + 2 * area[1] + area[2]
    compounds["P_CB"] = (0.0, 0.0, 0.02)
    mn, mx = compound_aabb(R, pos, np.tile(half_c, (n_compounds, 1)))
    compounds["aabb_min"] = mn
    compounds["aabb_max"] = mx
    compounds["mesh"] = abi.NO_MESH
    compounds["mode"] = np.where(np.arange(n_compounds) % 11 == 10, abi.MODE_DISABLED, abi.MODE_SUBMERGED)
    compounds["buoyancy"] = 1
    return {"meshes": mesh_list, "compounds": compounds, "parts": np.concatenate(parts),
            "parts_per_compound": np.asarray(counts, dtype=np.uint32), "ocean": flat_ocean()}


def cable_set(n_cables: int = 48, seed: int = 6, max_nodes: int = 120):
    """Seeded cables for CableEntity::ComputeHydrodynamicForces
    (CableEntity.cpp:240-376): sagging catenary-like chains across the
    surface, plus cables built to hit each submersion case exactly -- a
    horizontal cable on the waterline (dz = 0), a vertical one through it
    (dxy = 0), fully submerged and fully dry ones -- and one cable in a mode
    outside the fluid computation.  Returns cables, node positions and
    velocities (FP64) and a flat ocean with a uniform current."""
    rng = np.random.default_rng(seed)
    cables = np.zeros(n_cables, dtype=abi.CABLE_DTYPE)
    xs, vs = [], []
    first = 0
    for c in range(n_cables):
        kind = c % 6
        n = int(rng.integers(2, max_nodes)) if kind not in (1, 2) else int(rng.integers(2, 20))
        t = np.linspace(0.0, 1.0, n)
        x0 = rng.uniform(-5, 5, 3)
        if kind == 1:        # horizontal on the waterline
            pts = np.stack([x0[0] + 3 * t, np.full(n, x0[1]), np.full(n, rng.uniform(-0.02, 0.02))], axis=1)
        elif kind == 2:      # vertical through the surface
            pts = np.stack([np.full(n, x0[0]), np.full(n, x0[1]), -1.0 + 2.5 * t], axis=1)
        elif kind == 3:      # fully submerged
            pts = np.stack([x0[0] + 4 * t, x0[1] + t, 2.0 + np.sin(3 * t)], axis=1)
        elif kind == 4:      # dry
            pts = np.stack([x0[0] + 4 * t, x0[1] - t, -3.0 - t], axis=1)
        else:                # sagging chain across the surface
            span = rng.uniform(2, 10)
            sag = rng.uniform(0.2, 3.0)
            pts = np.stack([x0[0] + span * t, x0[1] + rng.uniform(-1, 1) * t,
                            rng.uniform(-1.0, 0.3) + sag * (1 - (2 * t - 1) ** 2)], axis=1)
        xs.append(pts)
        vs.append(rng.uniform(-1.0, 1.0, (n, 3)))
        cables[c]["first_node"] = first
        cables[c]["n_nodes"] = n
        cables[c]["radius"] = rng.uniform(0.01, 0.08)
        cables[c]["mode"] = abi.MODE_DISABLED if c == n_cables - 1 else (abi.MODE_FLOATING if c % 2 else
                                                                          abi.MODE_SUBMERGED)
        cables[c]["buoyancy"] = 0 if c % 7 == 5 else 1
        first += n
    return {"cables": cables, "x": np.concatenate(xs), "v": np.concatenate(vs),
            "ocean": flat_ocean(current=(0.3, -0.1, 0.0))}
