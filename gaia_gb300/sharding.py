"""Scene sharding across GPUs (one process per GPU, no collective on the data path).

Independent scenes (separate meshes without contact) partition across ranks:
the reference runs all meshes in one VBDPhysics and merges their colors into
parallel groups (VBD/VBDPhysics.cpp:235-274); across GPUs each rank runs its
own VBDPhysics over its share of the meshes. Shares are balanced by vertex
count with a deterministic greedy bin-pack (largest scene first, to the least
loaded rank, lowest rank on ties), so every rank computes the same partition
without communicating.
"""
from __future__ import annotations

import json
import os


def partition_scenes(vertex_counts: list[int], world: int) -> list[list[int]]:
    """Indices of the scenes each rank owns."""
    if world <= 0:
        raise ValueError("world must be positive")
    order = sorted(range(len(vertex_counts)), key=lambda i: (-vertex_counts[i], i))
    load = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += vertex_counts[i]
    return [sorted(p) for p in parts]


def write_shard(models_json: str, params_json: str, scene_ids: list[int], out_dir: str) -> tuple[str, str]:
    """Models.json / Parameters.json holding only `scene_ids` (deformers re-indexed,
    deformers of other scenes dropped)."""
    with open(models_json) as f:
        M = json.load(f)
    with open(params_json) as f:
        P = json.load(f)
    remap = {old: new for new, old in enumerate(scene_ids)}
    M["Models"] = [M["Models"][i] for i in scene_ids]
    defs = []
    for d in P.get("Deformers", []):
        keep = [(remap[m], v) for m, v in zip(d["selectedMeshes"], d["selectedVertices"]) if m in remap]
        if keep:
            d = dict(d)
            d["selectedMeshes"] = [k[0] for k in keep]
            d["selectedVertices"] = [k[1] for k in keep]
            defs.append(d)
    if "Deformers" in P:
        P["Deformers"] = defs
    os.makedirs(out_dir, exist_ok=True)
    mp = os.path.join(out_dir, "Models.json")
    pp = os.path.join(out_dir, "Parameters.json")
    with open(mp, "w") as f:
        json.dump(M, f, indent=1)
    with open(pp, "w") as f:
        json.dump(P, f, indent=1)
    return mp, pp
