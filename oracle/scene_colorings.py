"""Vertex colorings of the benchmark's large meshes for the CPU reference arm — TEST
INFRASTRUCTURE ONLY.

The reference arm of bench.py times the oracle and must build its scenes without the
product library. Scene files carry a vertex coloring (Models.json
verticesColoringCategoriesPath, as the reference's inputs do); for meshes up to
ORACLE_MAX_VERTICES the oracle computes it with its restatement of the reference's
GraphColoring tool (O(V^2), as the reference's mcs.cpp / gready.cpp are written), and for
the larger ones (the 100^3 twist lattice, the 512 x 512 cloth) it is read from
scene_colorings.npz, written by ``python -m oracle.scene_colorings`` from the colorings the
scene writer produces (the library's O(E log V) implementation of the same tool, which
tests/test_coloring.py pins bit for bit to the reference's own coloring code).
Entries are keyed by a hash of the mesh's connectivity and the coloring kind.
"""
from __future__ import annotations

import hashlib
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
STORE = os.path.join(HERE, "scene_colorings.npz")
ORACLE_MAX_VERTICES = 30000
_cache: dict | None = None


def key(nv: int, elems: np.ndarray, kind: str) -> str:
    h = hashlib.sha1()
    h.update(f"{kind}:{nv}:".encode())
    h.update(np.ascontiguousarray(elems, np.int32).tobytes())
    return h.hexdigest()[:20]


def _load() -> dict:
    global _cache
    if _cache is None:
        _cache = dict(np.load(STORE)) if os.path.exists(STORE) else {}
    return _cache


def stored(nv: int, elems: np.ndarray, kind: str):
    """(colors, order) stored for this mesh and kind, or None."""
    d = _load()
    k = key(nv, elems, kind)
    if k + "__colors" not in d:
        return None
    colors = d[k + "__colors"].astype(np.int32)
    order = np.cumsum(d[k + "__order_delta"].astype(np.int64)).astype(np.int32)
    return colors, order


def tet_coloring(nv: int, tets: np.ndarray, kind: str):
    """(colors, category order) of a tet mesh: kind "tool" (MCS + balancing, the tool's
    default), "mcs" or "greedy" (plain, categories in ascending vertex order)."""
    s = stored(nv, tets, "tet_" + kind)
    if s is not None:
        return s
    if nv > ORACLE_MAX_VERTICES:
        raise RuntimeError(f"no stored coloring for a {nv}-vertex tet mesh ({kind}); run python -m "
                           "oracle.scene_colorings where the product library is built")
    from . import oracle as orc

    if kind == "tool":
        return orc.color_tool(nv, tets)
    colors = orc.color_mcs(nv, tets) if kind == "mcs" else orc.color_greedy(nv, tets)
    order = np.concatenate([np.flatnonzero(colors == c) for c in range(int(colors.max()) + 1)]).astype(np.int32)
    return colors, order


def trimesh_coloring(nv: int, faces: np.ndarray):
    """(colors, category order) the coloring tool writes for a triangle mesh (stored only)."""
    s = stored(nv, faces, "tri_tool")
    if s is None:
        raise RuntimeError(f"no stored coloring for a {nv}-vertex triangle mesh")
    return s


def main() -> None:
    """Write scene_colorings.npz: the tool colorings of the benchmark's large meshes."""
    import sys

    sys.path.insert(0, os.path.dirname(HERE))
    from gaia_gb300 import physics, scenes
    from gaia_gb300.cloth import color_trimesh_tool

    out = {}

    def put(nv, elems, kind, colors, order):
        k = key(nv, elems, kind)
        out[k + "__colors"] = np.asarray(colors, np.uint8)
        out[k + "__order_delta"] = np.diff(np.asarray(order, np.int64), prepend=0).astype(np.int32)

    n = 100
    half = 0.5 * 0.01 * (n - 1)
    X, T = scenes.lattice_cube((n, n, n), 0.01, (0.0, -half, -half), jitter=1e-4, seed=1)
    put(len(X), T, "tet_tool", *physics.color_tool(len(X), T))
    with tempfile.TemporaryDirectory():
        Xc, F = scenes.cloth_grid(512, 1.0, 0.3 + 0.01, 1e-3, 1)
        put(len(Xc), F, "tri_tool", *color_trimesh_tool(len(Xc), F))
    np.savez_compressed(STORE, **out)
    print(f"wrote {STORE} ({os.path.getsize(STORE) / 1e6:.2f} MB, {len(out) // 2} meshes)")


if __name__ == "__main__":
    main()
