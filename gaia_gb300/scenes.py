"""Synthetic scenes for the VBD step, written as the reference's inputs.

Plays the role of the reference's ParameterGen scripts
(Simulator/VBDDynamics/ParameterGen/M01_Parameters.py, S0*.py): builds tet
meshes, colors them with the reference's OrderedGreedy algorithm (through the
library's bit-exact implementation), and writes ``.t`` meshes, coloring JSON,
``Models.json`` and ``Parameters.json`` that both this library and the
reference's loader read. All randomness is seeded numpy PCG64; seeds are
stored in the written JSON.
"""
from __future__ import annotations

import json
import os

import numpy as np


def lame(E: float, nu: float) -> tuple[float, float]:
    """Young's modulus / Poisson ratio -> (mu, lambda)."""
    return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))


# Local corner (a, b, c) of a lattice cell -> index a + 2b + 4c.
def _c(a, b, c):
    return a + 2 * b + 4 * c


# 5-tet split of a cube cell. Even cells use the central tet on corners
# {100, 010, 001, 111}; odd cells are the mirror image in x, so that shared
# faces use the same diagonal (a conforming mesh).
_EVEN = [
    (_c(1, 0, 0), _c(0, 1, 0), _c(0, 0, 1), _c(1, 1, 1)),
    (_c(0, 0, 0), _c(1, 0, 0), _c(0, 1, 0), _c(0, 0, 1)),
    (_c(1, 1, 0), _c(1, 0, 0), _c(0, 1, 0), _c(1, 1, 1)),
    (_c(1, 0, 1), _c(1, 0, 0), _c(0, 0, 1), _c(1, 1, 1)),
    (_c(0, 1, 1), _c(0, 1, 0), _c(0, 0, 1), _c(1, 1, 1)),
]
_ODD = [tuple(_c(1 - (k & 1), (k >> 1) & 1, (k >> 2) & 1) for k in t) for t in _EVEN]


def lattice_cube(n: tuple[int, int, int], spacing: float = 0.01, origin=(0.0, 0.0, 0.0),
                 jitter: float = 0.0, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """A vertex lattice of n = (nx, ny, nz) vertices, each cell split into 5 tets.

    Vertex (i, j, k) has index i + nx * (j + ny * k). Tets are positively
    oriented (det(Dm) > 0). Positions are jittered by U(-jitter, +jitter) per
    coordinate from numpy's PCG64 with `seed`.
    """
    nx, ny, nz = n
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    X = np.stack([i.transpose(2, 1, 0).ravel(), j.transpose(2, 1, 0).ravel(), k.transpose(2, 1, 0).ravel()], 1)
    X = X.astype(np.float64) * spacing + np.asarray(origin, np.float64)
    if jitter > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        X = X + rng.uniform(-jitter, jitter, size=X.shape)
    ci, cj, ck = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    ci, cj, ck = ci.transpose(2, 1, 0).ravel(), cj.transpose(2, 1, 0).ravel(), ck.transpose(2, 1, 0).ravel()
    corner = np.stack([(ci + a) + nx * ((cj + b) + ny * (ck + c))
                       for c in (0, 1) for b in (0, 1) for a in (0, 1)], 1)  # index a + 2b + 4c
    parity = (ci + cj + ck) & 1
    tets = np.empty((len(ci), 5, 4), np.int64)
    for t in range(5):
        even = corner[:, list(_EVEN[t])]
        odd = corner[:, list(_ODD[t])]
        tets[:, t, :] = np.where(parity[:, None] == 0, even, odd)
    tets = tets.reshape(-1, 4)
    # orient positively
    d = X[tets[:, 1:]] - X[tets[:, :1]]
    det = np.einsum("ij,ij->i", d[:, 0], np.cross(d[:, 1], d[:, 2]))
    neg = det < 0
    tets[neg, 2], tets[neg, 3] = tets[neg, 3].copy(), tets[neg, 2].copy()
    return X, tets.astype(np.int32)


# Who writes mesh and coloring files: "library" (the product's writers and colorings) or
# "oracle" (plain-Python writers and the oracle's colorings, for the CPU reference arm of
# the benchmark, which must not load the product library).
_WRITER = "library"


def set_writer(name: str) -> None:
    global _WRITER
    if name not in ("library", "oracle"):
        raise ValueError(name)
    _WRITER = name


def _py_write_t(path: str, X: np.ndarray, tets: np.ndarray) -> None:
    """The .t format the library writes ("Vertex id x y z" with %.9g, "Tet id a b c d")."""
    X = np.asarray(X, np.float64)
    with open(path, "w") as f:
        f.writelines("Vertex %d %.9g %.9g %.9g\n" % (i, x[0], x[1], x[2]) for i, x in enumerate(X))
        f.writelines("Tet %d %d %d %d %d\n" % (i, t[0], t[1], t[2], t[3]) for i, t in enumerate(np.asarray(tets)))


def _py_write_categories(path: str, colors: np.ndarray, order: np.ndarray) -> None:
    cats = [[] for _ in range(int(np.max(colors)) + 1)]
    for v in np.asarray(order).tolist():
        cats[int(colors[v])].append(v)
    with open(path, "w") as f:
        f.write("[" + ",".join("[" + ",".join(map(str, c)) + "]" for c in cats) + "]")


def _write_mesh(dirname: str, name: str, X: np.ndarray, tets: np.ndarray, coloring: str = "tool") -> tuple[str, str]:
    """.t mesh plus its vertex coloring file. coloring = "tool": what the reference's
    GraphColoring tool writes by default (MCS, categories balanced to a 1.05 size ratio);
    "mcs" / "greedy": the plain algorithms."""
    os.makedirs(dirname, exist_ok=True)
    tpath = os.path.join(dirname, name + ".t")
    cpath = tpath + ".vertexColoring.json"
    if _WRITER == "oracle":
        from oracle.scene_colorings import tet_coloring

        _py_write_t(tpath, X, tets)
        _py_write_categories(cpath, *tet_coloring(len(X), np.asarray(tets, np.int32), coloring))
        return tpath, cpath
    from .physics import color_greedy, color_mcs, color_tool, write_categories, write_coloring, write_t
    write_t(tpath, X, tets)
    if coloring == "tool":
        colors, order = color_tool(len(X), tets)
        write_categories(cpath, colors, order)
    else:
        colors = color_greedy(len(X), tets) if coloring == "greedy" else color_mcs(len(X), tets)
        write_coloring(cpath, colors)
    return tpath, cpath


def model_entry(path: str, coloring_path: str, E: float = 1e6, nu: float = 0.4, density: float = 1000.0,
                **extra) -> dict:
    mu, lmbd = lame(E, nu)
    m = {
        "path": path,
        "verticesColoringCategoriesPath": coloring_path,
        "materialName": "NeoHookean",
        "miu": mu,
        "lmbd": lmbd,
        "density": density,
        "dampingHydrostatic": 0.0,
        "dampingDeviatoric": 0.0,
        "frictionDynamic": 0.1,
        "frictionEpsV": 0.01,
        "initializationType": 0,
        "scale": [1.0, 1.0, 1.0],
        "translation": [0.0, 0.0, 0.0],
        "rotation": [0.0, 0.0, 0.0],
        "initialVelocity": [0.0, 0.0, 0.0],
        "fixedPoints": [],
    }
    m.update(extra)
    return m


def physics_params(timeStep: float, iterations: int, numSubsteps: int = 1, gravity=(0.0, -9.8, 0.0),
                   ground_y: float | None = None, precision: str = "mixed", **extra) -> dict:
    lo = [-1e7, -1e7, -1e7]
    if ground_y is not None:
        lo[1] = ground_y
    p = {
        "timeStep": timeStep,
        "numSubsteps": numSubsteps,
        "iterations": iterations,
        "gravity": list(gravity),
        "worldBounds": [lo, [1e7, 1e7, 1e7]],
        "usePlaneGround": True,
        "boundaryCollisionStiffness": 1e5,
        "boundaryFrictionDynamic": 0.2,
        "boundaryFrictionEpsV": 1.0,
        "stepSize": 1.0,
        "stepSizeGD": 1e-3,
        "useGPU": True,
        "handleCollision": False,
        "gpuPrecision": precision,
        "checkAndUpdateWorldBounds": False,
        "saveOutputs": False,
    }
    p.update(extra)
    return p


# CollisionParams of scenes without contact between meshes (contact detection off)
NO_CONTACT = {"allowCCD": False, "allowDCD": False}


def _write_json(dirname: str, models: list[dict], params: dict, deformers: list[dict] | None = None,
                meta: dict | None = None, collision: dict | None = None) -> tuple[str, str]:
    mp = os.path.join(dirname, "Models.json")
    pp = os.path.join(dirname, "Parameters.json")
    with open(mp, "w") as f:
        json.dump({"Models": models}, f, indent=1)
    P = {"PhysicsParams": params, "CollisionParams": dict(collision or {}), "ViewerParams": {"enableViewer": False}}
    if deformers:
        P["Deformers"] = deformers
    if meta:
        P["SceneInfo"] = meta
    with open(pp, "w") as f:
        json.dump(P, f, indent=1)
    return mp, pp


def drop_cube(dirname: str, n: int = 10, precision: str = "mixed", iterations: int = 20, seed: int = 1,
              spacing: float = 0.01, height: float = 0.2, coloring: str = "tool",
              collision: dict | None = None) -> tuple[str, str]:
    """Plain VBD drop: an n^3 vertex lattice cube (spacing 1 cm, jitter 1e-4, seed 1),
    Neo-Hookean E=1e6, nu=0.4, rho=1000, bottom at `height` above a ground plane at
    y=0 (stiffness 1e5, friction 0.2), dt=1/300, `iterations` per step. `coloring` as in
    _write_mesh; `collision` = CollisionParams (None: the reference's defaults, tet-mesh
    contact detection on)."""
    half = 0.5 * spacing * (n - 1)
    X, T = lattice_cube((n, n, n), spacing, (-half, height, -half), jitter=1e-4, seed=seed)
    tp, cp = _write_mesh(dirname, f"cube{n}", X, T, coloring=coloring)
    models = [model_entry(tp, cp)]
    params = physics_params(1.0 / 300.0, iterations, ground_y=0.0, precision=precision)
    return _write_json(dirname, models, params, meta={"workload": f"drop_cube_{n}", "seed": seed},
                       collision=collision)


def stack_drop(dirname: str, n_lower: int = 6, n_upper: int = 5, spacing: float = 0.01, gap: float = 0.004,
               speed: float = 1.5, precision: str = "mixed", iterations: int = 10, timeStep: float = 1.0 / 300.0,
               numSubsteps: int = 1, collision_stiffness: float = 1e5, offset=(0.013, 0.0, 0.011),
               seed: int = 3, **extra) -> tuple[str, str]:
    """Tet-mesh contact: a cube (n_upper^3 lattice) moving down at `speed` m/s onto
    another (n_lower^3) resting on the ground plane y = 0, `gap` above it and shifted
    by `offset` in x/z so that edges and vertices also meet faces. Both cubes are
    Neo-Hookean E=1e6, nu=0.4; contact through the tet-surface CCD and the v-f
    penalty (collisionStiffness)."""
    Xa, Ta = lattice_cube((n_lower,) * 3, spacing, (0.0, 0.0, 0.0), jitter=1e-4, seed=seed)
    top = spacing * (n_lower - 1)
    Xb, Tb = lattice_cube((n_upper,) * 3, spacing * 0.97, (offset[0], top + gap, offset[2]), jitter=1e-4,
                          seed=seed + 1)
    ta, ca = _write_mesh(dirname, "lower", Xa, Ta, coloring="greedy")
    tb, cb = _write_mesh(dirname, "upper", Xb, Tb, coloring="mcs")
    models = [model_entry(ta, ca, frictionDynamic=0.2, frictionEpsV=0.01),
              model_entry(tb, cb, density=800.0, frictionDynamic=0.3, frictionEpsV=0.02,
                          initialVelocity=[0.0, -speed, 0.0])]
    params = physics_params(timeStep, iterations, numSubsteps=numSubsteps, ground_y=0.0, precision=precision,
                            collisionStiffness=collision_stiffness, **extra)
    return _write_json(dirname, models, params)


def twist_cube(dirname: str, n: int = 100, precision: str = "mixed", iterations: int = 50, seed: int = 1,
               spacing: float = 0.01, omega: float = 2.0) -> tuple[str, str]:
    """Twist test: an n^3 lattice cube with its long (x) axis on the world x axis;
    both x-end faces are Dirichlet and the x-max face rotates at `omega` rad/s about
    the x axis (Rotator deformer). Same material, dt=1/300, `iterations` per step.
    A single body without contact: CollisionParams turn contact detection off."""
    half = 0.5 * spacing * (n - 1)
    X, T = lattice_cube((n, n, n), spacing, (0.0, -half, -half), jitter=1e-4, seed=seed)
    tp, cp = _write_mesh(dirname, f"twist{n}", X, T)
    idx = np.arange(n * n * n)
    ii = idx % n
    left = idx[ii == 0].tolist()
    right = idx[ii == n - 1].tolist()
    models = [model_entry(tp, cp, fixedPoints=left + right)]
    params = physics_params(1.0 / 300.0, iterations, precision=precision)
    deformers = [{"DeformerName": "Rotator", "center": [0.0, 0.0, 0.0], "axis": [1.0, 0.0, 0.0],
                  "angularVelocity": omega, "selectedMeshes": [0], "selectedVertices": [right]}]
    return _write_json(dirname, models, params, deformers, meta={"workload": f"twist_cube_{n}", "seed": seed},
                       collision=NO_CONTACT)


def batch_cubes(dirname: str, n_scenes: int = 512, side_range=(4, 24), precision: str = "mixed",
                iterations: int = 20, seed: int = 7, spacing: float = 0.01) -> tuple[str, str]:
    """Batching form: `n_scenes` independent lattice cubes, side drawn uniformly from
    side_range (vertices per edge), E ~ U(1e5, 1e7), nu ~ U(0.3, 0.45), laid out on a
    grid above one ground plane (no inter-object contact, contact detection off), dt=1/300."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sides = rng.integers(side_range[0], side_range[1] + 1, size=n_scenes)
    Es = rng.uniform(1e5, 1e7, size=n_scenes)
    nus = rng.uniform(0.3, 0.45, size=n_scenes)
    files = {}
    models = []
    g = int(np.ceil(np.sqrt(n_scenes)))
    pitch = spacing * side_range[1] + 0.1
    for s in range(n_scenes):
        n = int(sides[s])
        if n not in files:
            X, T = lattice_cube((n, n, n), spacing, (0.0, 0.0, 0.0), jitter=1e-4, seed=seed + n)
            files[n] = _write_mesh(dirname, f"cube{n}", X, T)
        tp, cp = files[n]
        tx, tz = (s % g) * pitch, (s // g) * pitch
        models.append(model_entry(tp, cp, E=float(Es[s]), nu=float(nus[s]), translation=[tx, 0.1, tz]))
    params = physics_params(1.0 / 300.0, iterations, ground_y=0.0, precision=precision)
    return _write_json(dirname, models, params,
                       meta={"workload": f"batch_cubes_{n_scenes}", "seed": seed, "sides": sides.tolist()},
                       collision=NO_CONTACT)


def lattice_ball(radius: float, spacing: float, jitter: float = 0.0, seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """A tetrahedralised ball: the cells of a 5-tet lattice (see lattice_cube) whose
    centres lie within `radius` of the origin, unused vertices dropped."""
    n = int(np.ceil(2 * radius / spacing)) + 2
    X, T = lattice_cube((n, n, n), spacing, (-(n - 1) * spacing / 2,) * 3, jitter=jitter, seed=seed)
    c = X[T].mean(axis=1)
    # a cell's 5 tets share its centre; keep cells, not single tets, so the surface stays manifold
    cell_c = c.reshape(-1, 5, 3).mean(axis=1)
    keep = np.repeat(np.linalg.norm(cell_c, axis=1) <= radius, 5)
    T = T[keep]
    used = np.unique(T)
    remap = -np.ones(len(X), np.int64)
    remap[used] = np.arange(len(used))
    return X[used], remap[T].astype(np.int32)


def collision_drop(dirname: str, n_objects: int = 32, precision: str = "mixed", iterations: int = 30,
                   seed: int = 5, cube_sides=(8, 20), ball_radii=(0.05, 0.15), ball_tets=(5000, 40000),
                   cube_spacing: float = 0.008, box: float = 1.0) -> tuple[str, str]:
    """Collision-heavy drop: `n_objects` tet meshes, half lattice cubes (side drawn from
    cube_sides vertices, `cube_spacing` apart) and half tetrahedralised balls (radius from
    ball_radii, lattice spacing chosen for a tet count in ball_tets), at seeded random,
    non-overlapping positions and random orientations in a `box`-metre world box with
    walls, Neo-Hookean E=1e6, nu=0.4, rho=1000, gravity -9.8, dt=1/300, `iterations` per
    step; vertex-face contact between and within objects (CCD and DCD)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    os.makedirs(dirname, exist_ok=True)
    shapes = []
    for k in range(n_objects):
        if k % 2 == 0:
            n = int(rng.integers(cube_sides[0], cube_sides[1] + 1))
            X, T = lattice_cube((n, n, n), cube_spacing, (0.0, 0.0, 0.0), jitter=1e-4, seed=seed + k)
            X = X - X.mean(axis=0)
            name = f"cube{k}"
        else:
            r = float(rng.uniform(*ball_radii))
            ntet = float(rng.uniform(*ball_tets))
            h = (4.0 / 3.0 * np.pi * r ** 3 / (ntet / 5.0)) ** (1.0 / 3.0)
            X, T = lattice_ball(r, h, jitter=1e-4 * h / 0.01, seed=seed + k)
            name = f"ball{k}"
        shapes.append((name, X, T, float(np.linalg.norm(X, axis=1).max())))
    # place: largest first, rejection-sampled centres inside the box, no bounding-sphere overlap
    order = sorted(range(n_objects), key=lambda k: -shapes[k][3])
    centres = [None] * n_objects
    placed = []
    for k in order:
        R = shapes[k][3]
        for _ in range(20000):
            c = rng.uniform(R + 0.01, box - R - 0.01, size=3)
            if all(np.linalg.norm(c - pc) > R + pr + 0.01 for pc, pr in placed):
                break
        else:
            raise RuntimeError("could not place all objects in the box")
        centres[k] = c
        placed.append((c, R))
    models = []
    for k, (name, X, T, R) in enumerate(shapes):
        tp, cp = _write_mesh(dirname, name, X, T)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        angle = float(rng.uniform(0, np.pi))
        models.append(model_entry(tp, cp, rotation=(axis * angle).tolist(), translation=centres[k].tolist()))
    params = physics_params(1.0 / 300.0, iterations, precision=precision,
                            worldBounds=[[0.0, 0.0, 0.0], [box, box, box]], collisionStiffness=1e5)
    nv = int(sum(len(s[1]) for s in shapes))
    return _write_json(dirname, models, params,
                       meta={"workload": f"collision_drop_{n_objects}", "seed": seed, "vertices": nv})


def contact_cluster(dirname: str, precision: str = "mixed", iterations: int = 30, seed: int = 11,
                    spacing: float = 0.025, gap: float = 0.004, speed: float = 0.8,
                    sizes=(4, 0.045, 3, 0.04)) -> tuple[str, str]:
    """The collision-heavy drop at test size: two lattice cubes (`sizes` vertices per side)
    and two tetrahedralised balls (`sizes` radii) stacked in a column with `gap` between
    neighbours, seeded random orientations, the upper three moving down at `speed` m/s
    onto the lowest cube, which rests on the floor of a 0.5 m world box. Same material and
    contact settings as collision_drop (CCD and DCD, contact stiffness 1e5); cells of
    2.5 cm keep |6V| of every tet above the 1e-5 below which the reference's discrete test
    rejects a tet, so both kinds of contact occur."""
    rng = np.random.Generator(np.random.PCG64(seed))
    os.makedirs(dirname, exist_ok=True)
    shapes = []
    for k, (kind, size) in enumerate(zip(("cube", "ball", "cube", "ball"), sizes)):
        if kind == "cube":
            X, T = lattice_cube((size,) * 3, spacing, (0.0, 0.0, 0.0), jitter=1e-4, seed=seed + k)
        else:
            X, T = lattice_ball(size, spacing, jitter=1e-4 * spacing / 0.01, seed=seed + k)
        X = X - X.mean(axis=0)
        shapes.append((f"{kind}{k}", X, T))
    models = []
    y = 0.0
    for k, (name, X, T) in enumerate(shapes):
        tp, cp = _write_mesh(dirname, name, X, T)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        angle = float(rng.uniform(0, np.pi)) if k else 0.0
        R = float(np.linalg.norm(X, axis=1).max()) if k else float(-X[:, 1].min())
        y += R if k else R + 1e-4
        shift = rng.uniform(-0.3, 0.3, size=2) * spacing
        models.append(model_entry(tp, cp, rotation=(axis * angle).tolist(),
                                  translation=[0.25 + shift[0], y, 0.25 + shift[1]],
                                  initialVelocity=[0.0, -speed if k else 0.0, 0.0]))
        y += R + gap
    params = physics_params(1.0 / 300.0, iterations, precision=precision,
                            worldBounds=[[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]], collisionStiffness=1e5)
    return _write_json(dirname, models, params, meta={"workload": "contact_cluster_4", "seed": seed})


def set_precision(params_json: str, precision: str, out_path: str | None = None, **overrides) -> str:
    """Copy of a Parameters.json with gpuPrecision (and other PhysicsParams) replaced."""
    with open(params_json) as f:
        P = json.load(f)
    P["PhysicsParams"]["gpuPrecision"] = precision
    P["PhysicsParams"].update(overrides)
    out = out_path or params_json.replace(".json", f".{precision}.json")
    with open(out, "w") as f:
        json.dump(P, f, indent=1)
    return out


# ---------------------------------------------------------------- cloth scenes
def write_obj(path: str, X: np.ndarray, faces: np.ndarray) -> None:
    """Wavefront .obj with 1-based faces (the reference's cloth and collider format)."""
    with open(path, "w") as f:
        for x in np.asarray(X, np.float64):
            f.write(f"v {x[0]:.9g} {x[1]:.9g} {x[2]:.9g}\n")
        for t in np.asarray(faces, np.int64):
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def cloth_grid(n: int, side: float = 1.0, height: float = 0.0, noise: float = 0.0, seed: int = 1):
    """A square cloth of n x n vertices in the xz plane at y = height, centred on the y
    axis; each cell split into two triangles along alternating diagonals, faces wound
    so their normals point up (+y). Vertex (i, j) has index i + n * j. Heights get
    U(-noise, +noise) from numpy's PCG64 with `seed`."""
    h = side / (n - 1)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    X = np.stack([i.ravel() * h - 0.5 * side, np.full(n * n, height), j.ravel() * h - 0.5 * side], 1)
    if noise > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        X[:, 1] += rng.uniform(-noise, noise, size=n * n)
    ci, cj = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    a = ci + n * cj
    b = a + 1
    c = a + n
    d = c + 1
    even = ((ci + cj) & 1) == 0
    # winding (a, c, b) has normal +y for this layout (x right, z down the rows)
    t1 = np.where(even[:, None], np.stack([a, c, d], 1), np.stack([a, c, b], 1))
    t2 = np.where(even[:, None], np.stack([a, d, b], 1), np.stack([b, c, d], 1))
    F = np.concatenate([t1, t2], 0).astype(np.int32)
    return X, F


def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Subdivided icosahedron with outward-wound faces."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.asarray(v, np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[k] = len(V) - 1
            return cache[k]

        F2 = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    X = np.asarray(V) * radius + np.asarray(center, np.float64)
    return X, np.asarray(F, np.int32)


def cloth_params(timeStep: float, iterations: int, contact_radius: float, max_query: float,
                 contact_stiffness: float = 1e5, gravity=(0.0, -9.8, 0.0), precision: str = "fp32", **extra) -> dict:
    p = {
        "timeStep": timeStep, "numSubsteps": 1, "iterations": iterations, "gravity": list(gravity),
        "worldBounds": [[-1e7, -1e7, -1e7], [1e7, 1e7, 1e7]], "boundaryFrictionDynamic": 0.1,
        "handleCollision": True, "contactStiffness": contact_stiffness, "contactRadius": contact_radius,
        "thickness": 0.0, "conservativeStepRelaxation": 0.45, "useNewton": False, "useLineSearch": False,
        "evaluateConvergence": False, "gpuPrecision": precision, "saveOutputs": False,
    }
    p.update(extra)
    return p


def cloth_on_sphere(dirname: str, n: int = 512, side: float = 1.0, sphere_radius: float = 0.3, sphere_level: int = 5,
                    gap: float = 0.01, iterations: int = 20, dt: float = 1.0 / 600.0, contact_radius: float = 2e-3,
                    max_query: float | None = None, noise: float = 1e-3, seed: int = 1, precision: str = "fp32",
                    mu: float = 1e4, lmbd: float = 1e4, bending: float = 1e-5, density: float = 0.2,
                    contact_stiffness: float = 1e5, friction: float = 0.1, init_type: int = 2,
                    **param_overrides) -> tuple[str, str]:
    """Cloth drape: an n x n vertex cloth (`side` metres, StVK mu/lambda, quadratic bending,
    areal density) `gap` above a static icosphere collider of `sphere_radius` centred at the
    origin; heights jittered by U(+-noise) (PCG64, `seed`); self and cloth-sphere VF/EE
    contact at `contact_radius`, query radius `max_query` (default 1.5 x contact radius)."""
    os.makedirs(dirname, exist_ok=True)
    X, F = cloth_grid(n, side, sphere_radius + gap, noise, seed)
    cpath = os.path.join(dirname, f"cloth{n}.obj")
    write_obj(cpath, X, F)
    colpath = cpath + ".vertexColoring.json"
    if _WRITER == "oracle":
        from oracle.scene_colorings import trimesh_coloring

        _py_write_categories(colpath, *trimesh_coloring(len(X), np.asarray(F, np.int32)))
    else:
        from .cloth import color_trimesh_tool
        from .physics import write_categories

        write_categories(colpath, *color_trimesh_tool(len(X), F))  # the coloring tool's default
    SX, SF = icosphere(sphere_level, sphere_radius)
    spath = os.path.join(dirname, f"sphere{sphere_level}.obj")
    write_obj(spath, SX, SF)
    model = {"path": cpath, "verticesColoringCategoriesPath": colpath, "materialName": "StVK_triMesh",
             "miu": mu, "lambda": lmbd, "bendingStiffness": bending, "density": density, "frictionDynamic": friction,
             "frictionEpsV": 0.01, "initializationType": init_type, "fixedPoints": []}
    mq = max_query if max_query is not None else 1.5 * contact_radius
    params = cloth_params(dt, iterations, contact_radius, mq, contact_stiffness, precision=precision, **param_overrides)
    mp = os.path.join(dirname, "Models.json")
    pp = os.path.join(dirname, "Parameters.json")
    with open(mp, "w") as f:
        json.dump({"Models": [model]}, f, indent=1)
    P = {"PhysicsParams": params, "ContactDetectorParams": {"maxQueryDis": mq},
         "ColliderParams": {"ColliderMeshes": [{"colliderType": "TriMeshSequence", "meshFiles": [spath],
                                                "frictionDynamic": friction, "frictionEpsV": 0.01}]},
         "SceneInfo": {"workload": f"cloth_on_sphere_{n}", "seed": seed}}
    with open(pp, "w") as f:
        json.dump(P, f, indent=1)
    return mp, pp
