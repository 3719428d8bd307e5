"""Benchmark of the GB300 VBD step: vertex-solves/s and steps/s.

Default workload (the headline configuration): the 100^3-vertex lattice cube
twist test (1.0 M vertices, 4.85 M tets, both x faces Dirichlet, one rotating at
2 rad/s), dt = 1/300 s, 50 VBD iterations per step, synthetic seeded inputs.

One JSON line on rank 0 with:
  value   = vertex-solves/s of the fastest FP32-compute mode (fp32, dfhi, mixed) whose
            error is within --tolerance (1e-5), inputs resident in HBM, device-timed with
            CUDA events on the library's stream;
  e2e     = the same metric through the public C ABI with host buffers
            (per step: H2D of positions+velocities, the step, D2H of both);
  fp64    = the plain FP64 engine on the same workload (same kernels in FP64);
  error   = relative position error of that mode vs the FP64 engine after
            --error-steps steps from the same initial state;
  roofline, cpu_baseline, clocks, gpu_launches;
  other_workloads = (twist on one GPU, unless --no-extra) the other configurations'
            default runs (drop, batch, collide, cloth), each in a child process,
            summarised: value, step time, precision, error and speed-up vs FP64.

``--impl reference`` times the CPU restatement of the reference's VBD path (the
oracle, all host threads) on bounded samples of the same workload.
Multi-GPU (torchrun): one independent replica per rank (weak scaling, no
collective on the data path); rank 0 reports the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "VBD vertex-solves/s & steps/s, FP32-mixed vs plain FP64 at <=1e-5 rel pos err"
# dram__bytes_read.sum + dram__bytes_write.sum per solved incidence of k_solve, measured by
# ncu: FP32 on 8 color launches of the 100^3 twist (4.8 M incidences each), double-float on
# colors 0-2 of the 60^3 twist (3 x ~1.01 M incidences); see profiles/
TRAFFIC_BYTES_PER_INCIDENCE = {"fp32": 54.4, "mixed": 59.9}
# DRAM bytes (read + write) of one k_sweep_scenes launch per solved incidence and iteration:
# 44.65 GB over 20 iterations of the 512-cube batch's 38.95 M incidences (FP32, mesh frames)
SCENES_TRAFFIC_BYTES_PER_INCIDENCE_ITERATION = 57.3


def load_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_scene(workload: str, d: str, precision: str, size: int, iterations: int):
    from gaia_gb300 import scenes

    if workload == "twist":
        return scenes.twist_cube(d, n=size, iterations=iterations, precision=precision)
    if workload == "drop":
        # the plain VBD drop: no contact detection, the reference's greedy coloring
        return scenes.drop_cube(d, n=size, iterations=iterations, precision=precision, coloring="greedy",
                                collision=scenes.NO_CONTACT)
    if workload == "batch":
        return scenes.batch_cubes(d, n_scenes=512, iterations=iterations, precision=precision)
    if workload == "collide":
        return scenes.collision_drop(d, n_objects=32, iterations=iterations, precision=precision)
    raise ValueError(workload)


def cpu_sample(mp: str, pp: str, iters: int, reps: int, precision: int = 32, nthreads: int = 0) -> dict:
    """Oracle (CPU restatement of the reference VBD step, all host threads; precision 32 =
    the reference's FloatingType, float): `reps` samples of one substep with `iters`
    iterations each."""
    from oracle import oracle as orc
    from oracle import scene_io

    sc = scene_io.load_scene(mp, pp)
    o = orc.OracleScene(sc, precision=precision, nthreads=nthreads)
    nact = sum(int(len(m["fixed"]) - m["fixed"].sum()) for m in sc["meshes"])
    t0 = time.perf_counter()
    for _ in range(reps):
        o.substep_sample(iters)
    dt = time.perf_counter() - t0
    cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    return {"vertex_solves_per_s": nact * iters * reps / dt, "seconds": dt, "cores": cores,
            "active_vertices": nact, "iterations": iters, "reps": reps}


def run_reference(args, world, rank):
    """The reference arm: the oracle (CPU restatement of the reference's VBD step in float,
    the reference's FloatingType) on all host threads, on the same scene files as the GPU
    arm, written without the product library (scene writer "oracle": plain-Python .t and
    coloring files, the oracle's or stored colorings). Each step is one substep of the
    configuration with as many of its iterations as fit the time budget (all of them when
    they fit); warm-up steps run one iteration each."""
    if rank != 0:
        return
    from gaia_gb300 import scenes
    from oracle import oracle as orc
    from oracle import scene_io

    scenes.set_writer("oracle")
    with tempfile.TemporaryDirectory() as d:
        mp, pp = make_scene(args.workload, d, "fp32", args.size, args.iterations)
        sc = scene_io.load_scene(mp, pp)
        o = orc.OracleScene(sc, precision=32, nthreads=0)
        nact = sum(int(len(m["fixed"]) - m["fixed"].sum()) for m in sc["meshes"])
        t_it = None
        for _ in range(max(args.warmup, 1)):
            t0 = time.perf_counter()
            o.substep_sample(1)
            t_it = time.perf_counter() - t0
        iters = args.iterations
        if args.ref_iters > 0:
            iters = min(iters, args.ref_iters)
        else:
            iters = max(1, min(iters, int(args.ref_budget / max(args.steps, 1) / max(t_it, 1e-9))))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            o.substep_sample(iters)
        dt = time.perf_counter() - t0
    v = nact * iters * args.steps / dt
    cores = os.cpu_count() or 1
    sample = (f"each step = one substep with {iters} of the configuration's {args.iterations} iterations over "
              f"{nact} active vertices (float oracle, {cores} threads); warm-up steps 1 iteration each")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "vertex-solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "steps_per_s_extrapolated": v / (nact * args.iterations),
        "config": {"workload": workload_name(args), "vertices_active": nact, "iterations_per_sample": iters,
                   "sample": sample},
        "cpu_baseline": {"value": v, "unit": "vertex-solves/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "vertex-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_name(args) -> str:
    if args.workload == "batch":
        return f"batch_cubes_512 (sides 4..24), {args.iterations} iterations/step, dt=1/300"
    if args.workload == "collide":
        return (f"collision_drop_32 (16 lattice cubes of 8..20 vertices per side, 16 tet balls r 0.05..0.15 m, "
                f"1 m box, tet-surface CCD + DCD every substep), {args.iterations} iterations/step, dt=1/300")
    if args.workload == "drop":
        return (f"drop_cube_{args.size}^3 (ground plane, no contact detection, greedy coloring), "
                f"{args.iterations} iterations/step, dt=1/300")
    return f"{args.workload}_cube_{args.size}^3, {args.iterations} iterations/step, dt=1/300"


def l2_bytes(local: int) -> int:
    try:
        import torch

        return int(torch.cuda.get_device_properties(local).L2_cache_size) or 129 << 20
    except Exception:
        return 129 << 20


def other_workloads(timeout_s: float = 900.0) -> dict:
    """The other configurations, each its own default bench run in a child process (so this
    line carries their numbers too): value, step time, precision, error vs the FP64 engine,
    speed-up over it, end-to-end rate, roofline fraction, and per workload its own figure
    (the batch's scene-steps/s and its speed-up over a per-scene loop, the cloth's floors)."""
    import subprocess
    import sys

    out = {}
    for w in ("drop", "batch", "collide", "cloth"):
        try:
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--workload", w, "--no-extra"],
                               capture_output=True, text=True, timeout=timeout_s)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                out[w] = {"error": f"exit {r.returncode}: {r.stderr.strip().splitlines()[-1:] or ''}"}
                continue
            d = json.loads(lines[-1])
        except Exception as ex:  # a failed child leaves the headline intact
            out[w] = {"error": str(ex)}
            continue
        e = d.get("error_vs_fp64") or {}
        summary = {"workload": d["config"].get("workload"), "value": d["value"], "unit": d["unit"],
                   "ms_per_step": d["ms_per_step"], "precision": d["config"].get("precision", "fp32"),
                   "error_vs_fp64": e.get("rel"),
                   "speedup_over_fp64": (d.get("fp64") or {}).get("speedup_over_fp64"),
                   "e2e": (d.get("e2e") or {}).get("value"), "roofline_frac": (d.get("roofline") or {}).get("frac"),
                   "cpu_baseline": (d.get("cpu_baseline") or {}).get("value"),
                   "schedule": (d["config"].get("schedule") or {}).get("sweep_mode"),
                   "clocks": d.get("clocks")}
        if d.get("batching"):
            summary["scenes_steps_per_s"] = d["batching"]["scenes_steps_per_s"]
            summary["speedup_over_per_scene_loop"] = d["batching"]["speedup_over_loop"]
        if "fp64_vs_fp64_summation_order" in e:
            summary["fp64_vs_fp64_summation_order"] = e["fp64_vs_fp64_summation_order"]
            summary["without_friction"] = e.get("without_friction")
        out[w] = summary
    return out


def timed_steps(phys, steps: int, local: int, rewind=None) -> tuple[float, float | None, str]:
    """Device time of `steps` steps, the time of their solve sweeps, and how L2 was handled.
    The steps are timed as runStep runs them (one graph per substep, timed as a whole); the
    sweep time, for the roofline, comes from the same steps run again from the same state
    (`rewind()` brings the handle back to it; no sweep time without it) with the substep's
    initial step, sweeps and velocity update as three graphs and CUDA events around every
    sweep. Scenes whose device data is under 4x L2 run each timed step alone after writing a
    buffer of 2x L2 (L2 flushed between timed steps); larger scenes run the steps back to
    back."""
    import torch

    l2 = l2_bytes(local)
    data = phys.stats()["device_bytes"]
    apart = data < 4 * l2
    buf = torch.empty(2 * l2 // 4, dtype=torch.float32, device=f"cuda:{local}") if apart else None

    def region(name: str, sweeps: bool) -> tuple[float, float | None]:
        # an NVTX range around each timed region, so that a profiler can select its launches
        # (ncu --nvtx --nvtx-include "timed_steps/")
        torch.cuda.nvtx.range_push(name)
        if not apart:
            tot, sw = phys.run_steps_timed(steps, sweeps)
        else:
            tot, sw = 0.0, (0.0 if sweeps else None)
            for _ in range(steps):
                buf.fill_(1.0)
                torch.cuda.synchronize()
                t, s = phys.run_steps_timed(1, sweeps)
                tot += t
                if sweeps:
                    sw += s
        torch.cuda.nvtx.range_pop()
        return tot, sw

    tot, _ = region("timed_steps", False)
    sw = None
    if rewind is not None:
        rewind()
        _, sw = region("timed_sweeps", True)
    del buf
    if not apart:
        return tot, sw, f"inputs larger than L2 ({data / 1e6:.0f} MB of device data, L2 {l2 / 1e6:.0f} MB)"
    return tot, sw, (f"L2 flushed before every timed step ({2 * l2 / 1e6:.0f} MB write; {data / 1e6:.0f} MB of "
                     f"device data), steps timed one at a time")


def measure_mode(args, mp, pp, precision, overrides, world, local, xref=None):
    """Device-timed steps, e2e steps through the C ABI, stats and the position error vs
    the FP64 reference trajectory (xref) for one precision mode."""
    import numpy as np
    import torch

    from gaia_gb300 import VBDPhysics, scenes

    ppm = scenes.set_precision(pp, precision, **overrides)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, ppm)
    phys.initialize()
    st = phys.stats()
    ccfg = phys.colorConfigs()
    nact, ninc, n = st["num_active_vertices"], st["num_incidences"], st["num_vertices"]
    x0 = np.concatenate([phys.positions(m) for m in range(phys.numMeshes())])
    err = None
    if xref is not None:
        phys.runStep(args.error_steps)
        x = np.concatenate([phys.positions(m) for m in range(phys.numMeshes())])
        err = {"steps": args.error_steps, "rel": float(np.linalg.norm(x - xref) / np.linalg.norm(xref - x0)),
               "max_abs_m": float(np.abs(x - xref).max()), "reference": "fp64 engine, same kernels"}

    def rewind():
        # the state the timed steps start from: the initial state and the warm-up steps
        phys.reset()
        for _ in range(args.warmup):
            phys.runStep(1)
        phys.synchronize()

    rewind()
    clk = ClockSampler(local)
    clk.start()
    barrier(world)
    total_ms, sweep_ms, l2_how = timed_steps(phys, args.steps, local, rewind)
    clocks = clk.stop()
    total_ms = allmax(world, total_ms)
    sweep_ms = allmax(world, sweep_ms)
    st = phys.stats()
    # e2e through the C ABI with page-locked host buffers, from the state the timed steps
    # started from: per step H2D of positions and velocities, the step, D2H of both
    rewind()
    xh = torch.empty(3 * n, dtype=torch.float32, pin_memory=True)
    vh = torch.empty(3 * n, dtype=torch.float32, pin_memory=True)
    phys.get_positions_f32(xh.data_ptr())
    phys.get_velocities_f32(vh.data_ptr())
    e2e_steps = max(3, args.steps // 2)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        phys.set_state_f32(xh.data_ptr(), vh.data_ptr())
        phys.runStep(1)
        phys.get_positions_f32(xh.data_ptr())
        phys.get_velocities_f32(vh.data_ptr())
    e2e_s = allmax(world, time.perf_counter() - t0)
    phys.close()
    solves = nact * args.iterations
    return {
        "precision": precision, "value": world * solves * args.steps / (total_ms / 1e3),
        "steps_per_s": args.steps / (total_ms / 1e3), "ms_per_step": total_ms / args.steps, "sweep_ms": sweep_ms,
        "e2e_value": world * solves * e2e_steps / e2e_s, "e2e_steps": e2e_steps, "error": err, "clocks": clocks,
        "stats": st, "nact": nact, "ninc": ninc, "n": n, "ccfg": ccfg, "l2": l2_how,
    }


def measure_scene_loop(args, mp, pp, precision, d):
    """The batching comparison: every scene of the batch as its own handle (its own
    layout, graphs and stream), stepped one after another in a host loop. Returns
    scenes-steps/s over `args.loop_steps` steps, timed on the host around a full
    device synchronisation."""
    from gaia_gb300 import VBDPhysics, scenes

    models = json.load(open(mp))["Models"]
    params = json.load(open(pp))["PhysicsParams"]
    params = dict(params, gpuPrecision=precision, autotune=False)
    handles = []
    for i, m in enumerate(models):
        sd = os.path.join(d, f"scene{i}")
        os.makedirs(sd, exist_ok=True)
        smp, spp = scenes._write_json(sd, [m], params)
        h = VBDPhysics()
        h.loadRunningparameters(smp, spp)
        h.initialize()
        handles.append(h)
    for _ in range(args.warmup):
        for h in handles:
            h.runStep(1)
    for h in handles:
        h.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.loop_steps):
        for h in handles:
            h.runStep(1)
    for h in handles:
        h.synchronize()
    dt = time.perf_counter() - t0
    for h in handles:
        h.close()
    return {"scenes_steps_per_s": len(models) * args.loop_steps / dt, "ms_per_step": 1e3 * dt / args.loop_steps,
            "steps": args.loop_steps, "scenes": len(models),
            "how": "one handle per scene (own graphs and stream, fixed lanes/block, no autotune), "
                   "stepped in a host loop; host-timed around a full synchronisation"}


# ---------------------------------------------------------------- cloth workload
CLOTH_METRIC = "cloth VBD vertex-solves/s & steps/s (StVK + bending + VF/EE contact), FP32 vs plain FP64"


def cloth_scene(args, d: str, precision: str):
    from gaia_gb300 import scenes

    extra = {"lanesPerVertex": args.lanes} if args.lanes else {}
    return scenes.cloth_on_sphere(d, n=args.size, iterations=args.iterations, precision=precision, **extra)


def cloth_algorithmic_bytes(c) -> tuple[float, dict]:
    """Algorithmic HBM bytes of one sweep of the cloth solve (all colors), FP32 layout:
    per vertex 89 B (x, x_prev, y, x_next 16 B each, mass 4, fixed 1, mesh/local ids 8,
    three CSR offsets 12, VF contact count 4), per face incidence 48 B (list entry 8, face
    ids 16, DmInv 16, area 4, FV link count 4), per bending incidence 40 B (list entry 8,
    edge ids 16, row of Q 16), per edge incidence 12 B (list entry 8, EE count 4).
    Positions of neighbours are L2-resident and not counted."""
    e6, fe = c.topology(0)
    nv, nf, ne = c.numVertices(0), c.numFaces(0), c.numEdges(0)
    interior = int((e6[:, 5] >= 0).sum())
    # bending incidences: the two vertices on each interior edge plus the two across it
    b = nv * 89.0 + 3 * nf * 48.0 + 4 * interior * 40.0 + 2 * ne * 12.0
    return b, {"vertices": nv, "faces": nf, "edges": ne, "interior_edges": interior}


def cloth_engine(mp, pp, precision, **overrides):
    from gaia_gb300 import VBDClothSimulationFramework, scenes

    c = VBDClothSimulationFramework()
    c.loadRunningparameters(mp, scenes.set_precision(pp, precision, out_path=pp + f".{precision}.{len(overrides)}.json",
                                                     **overrides))
    c.initialize()
    return c


def cloth_cpu_sample(mp, pp, iters: int, reps: int) -> dict:
    """The cloth oracle (FP64 solve, FP32 contact detection, all host threads) on
    `reps` samples of one substep with `iters` iterations (contact detection included)."""
    from oracle import cloth as oc

    sc = oc.load_scene(mp, pp)
    sc["params"]["iterations"] = iters
    sc["params"]["numSubsteps"] = 1
    o = oc.ClothOracle(sc, nthreads=0)
    nv = len(sc["meshes"][0]["X"])
    t0 = time.perf_counter()
    o.step(reps)
    dt = time.perf_counter() - t0
    return {"value": nv * iters * reps / dt, "seconds": dt, "cores": os.cpu_count() or 1, "vertices": nv}


def run_cloth(args, world, rank, local):
    import numpy as np

    peak, peak_kind = load_peaks()
    tmp = tempfile.TemporaryDirectory()
    d = tmp.name
    mp, pp = cloth_scene(args, d, "fp32")
    # plain FP64 engine: the reference trajectory for the error, and its speed
    fp64, xref = None, None
    if not args.no_fp64:
        c64 = cloth_engine(mp, pp, "fp64")
        x0 = c64.positions(0)
        c64.runStep(args.error_steps)
        xref = c64.positions(0)
        t64 = c64.run_steps_timed(args.fp64_steps)
        st64 = c64.stats()
        c64.close()
        fp64 = {"value": st64["num_sim_vertices"] * args.iterations * args.fp64_steps / (t64 / 1e3),
                "unit": "vertex-solves/s", "ms_per_step": t64 / args.fp64_steps}
    err = None
    if xref is not None:
        xm = {}
        for prec in ("fp32", "mixed"):
            ce = cloth_engine(mp, pp, prec)
            ce.runStep(args.error_steps)
            xm[prec] = ce.positions(0)
            ce.close()
        x = xm["fp32"]
        # the divergence floor of the drape: two FP64 runs that differ only in summation order
        # (one and two lanes per vertex, all else equal); a precision mode cannot get closer
        # to an FP64 run than two FP64 runs get to each other
        floor = []
        for lanes in (1, 2):
            cf = cloth_engine(mp, pp, "fp64", lanesPerVertex=lanes)
            cf.runStep(args.error_steps)
            floor.append(cf.positions(0))
            cf.close()
        err = {"steps": args.error_steps, "rel": float(np.linalg.norm(x - xref) / np.linalg.norm(xref - x0)),
               "max_abs_m": float(np.abs(x - xref).max()), "reference": "fp64 engine, same kernels",
               "mixed_rel": float(np.linalg.norm(xm["mixed"] - xref) / np.linalg.norm(xref - x0)),
               "fp64_vs_fp64_summation_order": float(np.linalg.norm(floor[0] - floor[1]) /
                                                     np.linalg.norm(xref - x0))}
        # the same drape without friction: the friction Hessian's jump at zero tangential
        # displacement (an exact zero in one summation order, a rounding residual in another)
        # is the drape's main discontinuity; without it the floor is that of the truncations
        from gaia_gb300 import scenes as _sc

        dnf = os.path.join(d, "no_friction")
        extra = {"lanesPerVertex": args.lanes} if args.lanes else {}
        mpf, ppf = _sc.cloth_on_sphere(dnf, n=args.size, iterations=args.iterations, precision="fp32", friction=0.0,
                                       **extra)
        xs, x1 = {}, {}
        for key, prec, over in (("fp64", "fp64", {"lanesPerVertex": 1}), ("fp64_l2", "fp64", {"lanesPerVertex": 2}),
                                ("fp32", "fp32", {}), ("mixed", "mixed", {})):
            cf = cloth_engine(mpf, ppf, prec, **over)
            if key == "fp64":
                xf0 = cf.positions(0)
            cf.runStep(1)
            x1[key] = cf.positions(0)  # after one step: before the first truncation flip
            cf.runStep(args.error_steps - 1)
            xs[key] = cf.positions(0)
            cf.close()
        den = np.linalg.norm(xs["fp64"] - xf0)
        den1 = np.linalg.norm(x1["fp64"] - xf0)
        err["without_friction"] = {
            "steps": args.error_steps, "rel": float(np.linalg.norm(xs["fp32"] - xs["fp64"]) / den),
            "mixed_rel": float(np.linalg.norm(xs["mixed"] - xs["fp64"]) / den),
            "fp64_vs_fp64_summation_order": float(np.linalg.norm(xs["fp64_l2"] - xs["fp64"]) / den),
            "after_1_step": {k: float(np.linalg.norm(x1[k] - x1["fp64"]) / den1) for k in ("fp32", "mixed", "fp64_l2")}}
    c = cloth_engine(mp, pp, "fp32")
    nv = c.numVertices(0)
    for _ in range(args.warmup):
        c.runStep(1)
    if not args.lanes:
        c.autotune()  # lanes per vertex re-timed on a state with the drape's contacts
    c.runStep(1)
    c.synchronize()
    clk = ClockSampler(local)
    clk.start()
    barrier(world)
    total_ms = c.run_steps_timed(args.steps)
    clocks = clk.stop()
    total_ms = allmax(world, total_ms)
    st = c.stats()
    sweep_ms = c.time_solve(5)
    lanes = c.groupLanes()
    alg, counts = cloth_algorithmic_bytes(c)
    # e2e through the C ABI with host buffers: per step the positions and velocities of
    # the cloth go host -> device, the step runs, positions and velocities come back
    xh, vh = c.positions(0), c.velocities(0)
    e2e_steps = max(3, args.steps // 3)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        c.setPositions(0, xh)
        c.setVelocities(0, vh)
        c.runStep(1)
        xh = c.positions(0)
        vh = c.velocities(0)
    e2e_s = allmax(world, time.perf_counter() - t0)
    c.close()
    # the double-float mode's rate on the same drape
    cmx = cloth_engine(mp, pp, "mixed")
    for _ in range(args.warmup):
        cmx.runStep(1)
    if not args.lanes:
        cmx.autotune()
    cmx.runStep(1)
    cmx.synchronize()
    mixed_ms = allmax(world, cmx.run_steps_timed(args.steps))
    cmx.close()
    cpu = None
    if rank == 0 and not args.no_cpu:
        s = cloth_cpu_sample(mp, pp, args.cpu_iters, args.cpu_reps)
        cpu = {"value": s["value"], "unit": "vertex-solves/s", "cores": s["cores"], "kind": "port",
               "sample": f"{args.cpu_reps} x one substep with {args.cpu_iters} iterations (contact detection "
                         f"included) over {s['vertices']} vertices ({s['seconds']:.1f} s), CPU restatement of the "
                         "reference cloth step"}
    tmp.cleanup()
    if rank != 0:
        return
    solves = world * nv * args.iterations
    ngroups = st["num_groups"]
    achieved = alg / (sweep_ms / 1e3) / 1e9
    line = {
        "metric": CLOTH_METRIC, "value": solves * args.steps / (total_ms / 1e3), "unit": "vertex-solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "steps_per_s": args.steps / (total_ms / 1e3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64 height noise)",
        "config": {"workload": f"cloth_on_sphere {args.size}x{args.size} (1 m, icosphere r=0.3 collider), "
                               f"{args.iterations} iterations/step, dt=1/600, contact radius 2e-3",
                   **counts, "colors": ngroups, "lanes_per_color": lanes, "detections": st["detections"],
                   "truncations": st["truncations"],
                   "l2": "inputs larger than L2 (per-sweep records %.0f MB)" % (alg / 1e6)},
        "e2e": {"value": solves * e2e_steps / e2e_s, "unit": "vertex-solves/s", "h2d_bytes_per_step": 48 * nv,
                "d2h_bytes_per_step": 48 * nv, "steps": e2e_steps},
        "error_vs_fp64": err, "fp64": fp64,
        "modes": {"fp32": {"value": solves * args.steps / (total_ms / 1e3), "ms_per_step": total_ms / args.steps,
                           "error_vs_fp64": err["rel"] if err else None},
                  "mixed": {"value": solves * args.steps / (mixed_ms / 1e3), "ms_per_step": mixed_ms / args.steps,
                            "error_vs_fp64": err["mixed_rel"] if err else None}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind, "kernel": "cloth k_solve + k_commit (all colors)",
                     "algorithmic_bytes_per_launch": alg / max(ngroups, 1),
                     "avg_launch_us": 1e3 * sweep_ms / max(ngroups, 1)},
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": st["kernel_launches_per_step"] * args.steps,
        "fp64_fallback_solves": st["fp64_fallback_solves"], "failed_solves": st["failed_solves"],
        "overflow": {k: st[k] for k in ("vf_overflow", "ee_overflow", "fv_overflow", "candidate_overflow",
                                        "stack_overflow")},
    }
    if fp64:
        fp64["speedup_over_fp64"] = line["value"] / fp64["value"]
    print(json.dumps(line), flush=True)


def run_cloth_reference(args, world, rank):
    """The cloth reference arm: the cloth oracle (FP64 solve, FP32 detection) on all host
    threads, on scene files written without the product library; each step is one substep
    with as many of the configuration's iterations as fit the time budget."""
    if rank != 0:
        return
    from gaia_gb300 import scenes

    scenes.set_writer("oracle")
    with tempfile.TemporaryDirectory() as d:
        mp, pp = cloth_scene(args, d, "fp64")
        w = cloth_cpu_sample(mp, pp, 1, max(args.warmup, 1))
        t_it = w["seconds"] / max(args.warmup, 1)
        iters = args.ref_iters if args.ref_iters > 0 else max(1, min(args.iterations, int(
            args.ref_budget / max(args.steps, 1) / max(t_it, 1e-9))))
        s = cloth_cpu_sample(mp, pp, iters, args.steps)
    args.ref_iters = iters
    v = s["value"]
    line = {
        "impl": "reference", "metric": CLOTH_METRIC, "value": v, "unit": "vertex-solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * s["seconds"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"cloth_on_sphere {args.size}x{args.size}", "vertices": s["vertices"],
                   "sample": f"each step = one substep with {args.ref_iters} iterations"},
        "cpu_baseline": {"value": v, "unit": "vertex-solves/s", "cores": s["cores"], "kind": "port",
                         "sample": f"{args.steps} samples of one substep x {args.ref_iters} iterations"},
        "e2e": {"value": v, "unit": "vertex-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gaia", choices=["gaia", "reference"])
    ap.add_argument("--workload", default="twist", choices=["twist", "drop", "batch", "cloth", "collide"])
    ap.add_argument("--size", type=int, default=0,
                    help="vertices per cube edge (0 = the workload's own: twist 100, drop 10)")
    ap.add_argument("--iterations", type=int, default=0,
                    help="VBD iterations per step (0 = the workload's own: twist 50, drop 20, batch 20)")
    ap.add_argument("--loop-steps", type=int, default=5,
                    help="batch workload: steps of the one-handle-per-scene loop it is compared with")
    ap.add_argument("--error-steps", type=int, default=100)
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--ref-iters", type=int, default=0,
                    help="iterations per CPU sample (0 = as many of the configuration's as fit the budget)")
    ap.add_argument("--ref-budget", type=float, default=120.0,
                    help="seconds of timed CPU work the reference arm aims at")
    ap.add_argument("--cpu-reps", type=int, default=2)
    ap.add_argument("--cpu-iters", type=int, default=2, help="iterations per cpu_baseline sample of the GPU arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--precision", default="auto", choices=["auto", "mixed", "dfhi", "fp32", "fp64"],
                    help="auto: measure fp32, dfhi and mixed, report the fastest within the 1e-5 error bound")
    ap.add_argument("--tolerance", type=float, default=1e-5)
    ap.add_argument("--lanes", type=int, default=0, help="lanes per vertex (0 = autotune)")
    ap.add_argument("--block", type=int, default=0, help="solve block size (0 = autotune)")
    ap.add_argument("--param", action="append", default=[],
                    help="PhysicsParams override key=json_value (e.g. usePDL=false)")
    ap.add_argument("--no-extra", action="store_true",
                    help="twist on 1 GPU: do not also run the other workloads (drop, batch, collide, cloth) "
                         "and summarise them in the line's other_workloads")
    args = ap.parse_args()
    if args.iterations <= 0:
        args.iterations = {"twist": 50, "collide": 30}.get(args.workload, 20)
    if args.workload == "collide" and args.error_steps == 100:
        args.error_steps = 20  # contact sets change discretely; long horizons diverge chaotically
    if args.size <= 0:
        args.size = {"drop": 10, "cloth": 512}.get(args.workload, 100)
    world, rank, local = dist_setup()
    if args.workload == "cloth":
        if args.error_steps == 100:
            args.error_steps = 30
        if args.impl == "reference":
            run_cloth_reference(args, world, rank)
        else:
            run_cloth(args, world, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import numpy as np

    from gaia_gb300 import VBDPhysics, scenes

    peak, peak_kind = load_peaks()
    tmp = tempfile.TemporaryDirectory()
    d = tmp.name
    mp, pp = make_scene(args.workload, d, "mixed", args.size, args.iterations)
    if args.workload == "batch" and world > 1:
        # independent scenes: each rank simulates its share (no collective on the data path)
        from gaia_gb300.sharding import partition_scenes, write_shard

        sides = json.load(open(pp))["SceneInfo"]["sides"]
        part = partition_scenes([s ** 3 for s in sides], world)[rank]
        mp, pp = write_shard(mp, pp, part, os.path.join(d, f"rank{rank}"))
    overrides = {}
    if args.lanes or args.block:
        overrides.update(lanesPerVertex=args.lanes, blockSize=args.block, autotune=False)
    for kv in args.param:
        k, v = kv.split("=", 1)
        overrides[k] = json.loads(v)

    # ---- plain FP64 engine: timing and the reference trajectory for the error ------------
    fp64, xref = None, None
    if not args.no_fp64:
        p64 = VBDPhysics()
        p64.loadRunningparameters(mp, scenes.set_precision(pp, "fp64", **overrides))
        p64.initialize()
        if args.error_steps > 0:
            p64.runStep(args.error_steps)
            xref = np.concatenate([p64.positions(m) for m in range(p64.numMeshes())])
            p64.reset()

        def rewind64():
            # the state the FP32-compute engines' timed steps start from too
            p64.reset()
            for _ in range(args.warmup):
                p64.runStep(1)
            p64.synchronize()

        rewind64()
        t64, _, _ = timed_steps(p64, args.fp64_steps, local)
        nact64 = p64.stats()["num_active_vertices"]
        p64.close()
        fp64 = {"value": world * nact64 * args.iterations * args.fp64_steps / (allmax(world, t64) / 1e3),
                "unit": "vertex-solves/s", "ms_per_step": t64 / args.fp64_steps}

    # ---- FP32-compute engines ------------------------------------------------------------
    modes = ["fp32", "dfhi", "mixed"] if args.precision == "auto" else [args.precision]
    runs = [measure_mode(args, mp, pp, m, overrides, world, local, xref) for m in modes]
    ok = [r for r in runs if r["error"] is None or r["error"]["rel"] <= args.tolerance]
    head = max(ok, key=lambda r: r["value"]) if ok else min(runs, key=lambda r: r["error"]["rel"])

    # ---- batching: the merged step against one handle per scene in a host loop -----------
    batching = None
    if args.workload == "batch" and args.loop_steps > 0:
        nsc = len(json.load(open(mp))["Models"])
        loop = measure_scene_loop(args, mp, pp, head["precision"], d)
        merged = world * nsc * head["steps_per_s"]
        batching = {"scenes_steps_per_s": merged, "scenes": world * nsc,
                    "per_scene_loop": dict(loop, scenes_steps_per_s=world * loop["scenes_steps_per_s"]),
                    "speedup_over_loop": merged / (world * loop["scenes_steps_per_s"])}

    # ---- CPU baseline: the oracle on a bounded sample of the same workload ------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        s = cpu_sample(mp, pp, iters=args.cpu_iters, reps=args.cpu_reps, precision=32)
        s64 = cpu_sample(mp, pp, iters=args.cpu_iters, reps=1, precision=64)
        cpu = {"value": s["vertex_solves_per_s"], "unit": "vertex-solves/s", "cores": s["cores"], "kind": "port",
               "sample": f"{s['reps']} x one substep with {s['iterations']} iterations over {s['active_vertices']} "
                         f"active vertices ({s['seconds']:.1f} s), float CPU restatement of the reference step "
                         "(the reference's FloatingType)",
               "fp64_value": s64["vertex_solves_per_s"]}
    tmp.cleanup()

    if rank == 0:
        st = head["stats"]
        nact, ninc, n = head["nact"], head["ninc"], head["n"]
        # roofline of the solve kernel: algorithmic bytes per iteration 64 B/vertex + 61 B/incidence;
        # the persistent schedules run a substep's iterations in one launch
        alg_bytes_iter = 64.0 * nact + 61.0 * ninc
        sweep_mode = st.get("sweep_mode", 0)
        if sweep_mode == 0:
            launches_solve, kernel, per_launch = st["num_groups"] * args.iterations * args.steps, "k_solve", \
                alg_bytes_iter / st["num_groups"]
        else:
            launches_solve = args.steps * head.get("substeps", 1)
            kernel = {1: "k_sweep_scenes", 2: "k_sweep_cluster", 3: "k_sweep_grid"}[sweep_mode]
            per_launch = alg_bytes_iter * args.iterations
        achieved = alg_bytes_iter * args.iterations * args.steps / (head["sweep_ms"] / 1e3) / 1e9
        # DRAM bytes per solved incidence (records + per-vertex data) from the ncu captures
        # (TRAFFIC_BYTES_PER_INCIDENCE), scaled to one average launch here
        per_inc = TRAFFIC_BYTES_PER_INCIDENCE.get(head["precision"])
        traffic, source = None, None
        if per_inc and sweep_mode == 0:
            traffic = per_inc * ninc / st["num_groups"]
            source = ("ncu DRAM bytes per incidence (FP32: 100^3 twist launches; double-float: 60^3 twist), times "
                      "this launch's incidences")
        elif sweep_mode == 1 and head["precision"] == "fp32":
            traffic = SCENES_TRAFFIC_BYTES_PER_INCIDENCE_ITERATION * ninc * args.iterations
            source = ("ncu DRAM bytes of the scene-major sweep per incidence and iteration (512-cube batch, FP32), "
                      "times this launch's incidences and iterations")
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic, "traffic_source": source,
                    "peak_kind": peak_kind, "kernel": kernel,
                    "algorithmic_bytes_per_launch": per_launch,
                    "avg_launch_us": 1e3 * head["sweep_ms"] / launches_solve}
        if fp64:
            fp64["speedup_over_fp64"] = head["value"] / fp64["value"]
        extra = None
        if args.workload == "twist" and world == 1 and not args.no_extra:
            extra = other_workloads()
        line = {
            "metric": METRIC, "value": head["value"], "unit": "vertex-solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "steps_per_s": head["steps_per_s"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "mixed": "f32 (double-float state)",
                      "dfhi": "f32 (double-float state, FP32 neighbour reads)"}.get(head["precision"], "f64"),
            "data": "synthetic (seeded PCG64 lattice)",
            "config": {"workload": workload_name(args), "vertices": n, "solved_incidences": ninc,
                       "precision": head["precision"], "colors": st["num_groups"],
                       "lanes_per_vertex": st["lanes_per_vertex"], "block": st["block_size"],
                       "solve_variant": st.get("solve_variant"), "overrides": overrides,
                       "color_configs": [[c["lanes"], c["block"], c["variant"]] for c in head["ccfg"]],
                       "schedule": {"sweep_mode": ["merged", "scenes", "cluster", "grid"][sweep_mode],
                                    "cluster_size": st.get("cluster_size", 0),
                                    "autotuned_ms_per_iteration": {k: st.get(f"sweep_ms_{k}", 0.0) for k in
                                                                   ("merged", "scenes", "cluster", "grid")}},
                       "l2": head["l2"],
                       "timing": ("value: the timed steps launched as runStep launches them (one CUDA graph per "
                                  "substep), CUDA events around the steps; roofline: the same steps from the same "
                                  "state with CUDA events around each substep's sweep graph")},
            "e2e": {"value": head["e2e_value"], "unit": "vertex-solves/s", "h2d_bytes_per_step": 24 * n,
                    "d2h_bytes_per_step": 24 * n, "steps": head["e2e_steps"]},
            "error_vs_fp64": head["error"], "fp64": fp64, "batching": batching,
            "modes": {r["precision"]: {"value": r["value"], "ms_per_step": r["ms_per_step"],
                                       "error_vs_fp64": r["error"]["rel"] if r["error"] else None,
                                       "e2e": r["e2e_value"]} for r in runs},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": head["clocks"],
            "gpu_launches": st["kernel_launches_per_step"] * args.steps,
            "fp64_fallback_solves": st["fp64_fallback_solves"], "failed_solves": st["failed_solves"],
        }
        if st.get("contact_detections"):
            # tet-mesh contact detection of the timed engine (cumulative over its life)
            line["contact"] = {k: st[k] for k in ("contact_detections", "contact_stack_overflow",
                                                   "contact_traverse_bounds")}
        if extra is not None:
            line["other_workloads"] = extra
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
