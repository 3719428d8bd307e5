"""Generate tests/golden/coloring_fixtures.npz from the reference's shipped data.

The reference ships vertex colorings produced by its GraphColoring tool (MCS,
GraphColoring/GraphColoring.cpp:157-196) next to the .t meshes they color
(Data/mesh_models/**/*.t.vertexColoring.json). This script stores, for the
small meshes (<= 1000 vertices), the tet index list and the coloring, so that
parity can be checked where the reference tree is not available. Larger
meshes are checked directly from the reference tree when it is present.

Usage: python tests/golden/make_fixtures.py /path/to/reference/Data/mesh_models
"""
import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_t(path):
    ids, tets = [], []
    with open(path) as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "Vertex":
                ids.append(int(p[1]))
            elif p[0] == "Tet":
                tets.append([int(p[2]), int(p[3]), int(p[4]), int(p[5])])
    lut = {v: i for i, v in enumerate(ids)}
    return len(ids), np.array([[lut[a] for a in t] for t in tets], np.int32)


def main(root):
    out = {}
    names = []
    for f in sorted(glob.glob(os.path.join(root, "**", "*.t.vertexColoring.json"), recursive=True)):
        t = f[: -len(".vertexColoring.json")]
        if not os.path.exists(t):
            continue
        nv, tets = load_t(t)
        if nv > 1000:
            continue
        cats = json.load(open(f))
        colors = np.full(nv, -1, np.int32)
        for c, verts in enumerate(cats):
            colors[np.asarray(verts, np.int64)] = c
        key = os.path.relpath(t, root).replace("/", "__")
        names.append(key)
        out[key + "__tets"] = tets
        out[key + "__colors"] = colors
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "coloring_fixtures.npz"), **out)
    print(f"wrote {len(names)} fixtures")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        from oracle.oracle import reference_root

        root = reference_root()
        if not root:
            sys.exit("the reference tree is not present (set GAIA_REFERENCE_ROOT or pass the mesh_models folder)")
        main(os.path.join(root, "Data", "mesh_models"))
