"""The vbd_dynamics command-line runner (VBDDynamics/main.cpp + BasePhysicFramework::simulate
and writeOutputs).

CPU: argument handling and failures before any device work (usage, unknown option,
unreadable parameter file, missing model file).
GPU: a contact scene run for 6 frames writes the frame files and recovery states the
reference's writeOutputs names; the last recovery state equals the positions the Python
API reaches after the same 6 steps; a run recovered from frame 3 (-r) reaches the same
frame 6, and "${REPO_ROOT}" paths with -R resolve.
"""
import json
import os
import subprocess

import numpy as np
import pytest


def _cli(gaia_lib):
    from gaia_gb300 import build as gb

    assert os.access(gb.CLI, os.X_OK)
    return gb.CLI


def _run(exe, *args):
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)


def test_usage_and_options(gaia_lib, tmp_path):
    exe = _cli(gaia_lib)
    r = _run(exe)
    assert r.returncode == 2 and "usage" in r.stderr
    r = _run(exe, "m.json", "p.json", str(tmp_path / "out"), "-x", "1")
    assert r.returncode == 2 and "unknown option -x" in r.stderr


def test_unreadable_inputs_fail_before_device_work(gaia_lib, tmp_path):
    exe = _cli(gaia_lib)
    r = _run(exe, "m.json", str(tmp_path / "missing.json"), str(tmp_path / "out"))
    assert r.returncode == 1 and "loadRunningparameters" in r.stderr
    pp = tmp_path / "p.json"
    pp.write_text(json.dumps({"PhysicsParams": {"numFrames": 1}}))
    r = _run(exe, str(tmp_path / "missing_models.json"), str(pp), str(tmp_path / "out"))
    assert r.returncode == 1 and "loadRunningparameters" in r.stderr
    assert not (tmp_path / "out").exists()
    r = _run(exe, "m.json", "p.json", str(tmp_path / "out"), "-R")
    assert r.returncode == 2 and "needs a value" in r.stderr


FACADE_PROBE = r"""
#include <cstdio>
#include "gaia_vbd.hpp"
int main(int argc, char** argv) {
    gaia::VBDPhysics p;
    try {
        p.initialize();
    } catch (const gaia::VBDError& e) {
        std::printf("before load: %s\n", e.what());
    }
    p.loadRunningparameters(argv[1], argv[2], "${REPO_ROOT}/out", argv[3]);
    const gaia_vbd_output_params o = p.outputParams();
    std::printf("%d %d %d %s %d %d %d %d %d %s\n", p.numMeshes(), o.num_frames, o.save_outputs, o.output_ext,
                o.binary_mode_visualization_steps, o.output_recovery_state, o.output_recovery_state_step,
                o.output_recovery_state_binary, o.save_all_models_together, p.outputFolder.c_str());
    return 0;
}
"""


def test_cpp_facade_loads_and_reads_output_params(gaia_lib, tmp_path):
    """The header-only gaia::VBDPhysics facade, host side: errors before loading, the
    output settings of Parameters.json (reference defaults where absent), ${REPO_ROOT}."""
    import shutil

    from gaia_gb300 import build as gb
    from gaia_gb300 import scenes

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "probe.cpp"
    src.write_text(FACADE_PROBE)
    exe = tmp_path / "probe"
    inc = os.path.join(os.path.dirname(gb.HERE), "include")
    r = subprocess.run([cxx, "-std=c++17", "-O1", str(src), "-o", str(exe), "-I", inc, "-L", gb.HERE, "-lgaia_vbd",
                        "-Wl,-rpath," + gb.HERE], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    mp, pp = scenes.stack_drop(str(tmp_path / "s"), spacing=0.03)
    P = json.load(open(pp))
    P["PhysicsParams"].pop("saveOutputs", None)
    P["PhysicsParams"].update(numFrames=7, outputExt="bin", outputRecoveryStateStep=3)
    json.dump(P, open(pp, "w"))
    r = subprocess.run([str(exe), mp, pp, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0].startswith("before load: ") and "loadRunningparameters" in lines[0]
    assert lines[1].split() == ["2", "7", "1", "bin", "100", "1", "3", "1", "1", str(tmp_path) + "/out"]


def _scene(tmp_path, **params):
    from gaia_gb300 import scenes

    mp, pp = scenes.stack_drop(str(tmp_path), spacing=0.03, gap=0.01, speed=1.0, precision="fp64")
    P = json.load(open(pp))
    P["PhysicsParams"].update(saveOutputs=True, **params)
    json.dump(P, open(pp, "w"))
    return mp, pp


def _state_positions(path):
    S = json.load(open(path))
    return S["frameId"], [np.asarray(m["position"], np.float64).reshape(-1, 3) for m in S["meshesState"]]


@pytest.mark.gpu
def test_frames_and_states_match_api(gaia_lib, tmp_path):
    from gaia_gb300 import VBDPhysics

    exe = _cli(gaia_lib)
    mp, pp = _scene(tmp_path, numFrames=6, outputExt="ply", saveAllModelsTogether=True, outputRecoveryState=True,
                    outputRecoveryStateStep=3, outputRecoveryStateBinary=False)
    out = tmp_path / "out"
    r = _run(exe, mp, pp, str(out))
    assert r.returncode == 0, r.stderr
    assert "6 frames" in r.stdout
    assert sorted(os.listdir(out / "RecoveryStates")) == ["A00000000.json", "A00000003.json", "A00000006.json"]
    assert json.load(open(out / "RecoveryStates" / "A00000003.json"))["format"] == "text"
    assert all((out / f"A{f:08d}.ply").exists() for f in range(7))
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    phys.initialize()
    phys.runStep(6)
    frame, X = _state_positions(out / "RecoveryStates" / "A00000006.json")
    assert frame == 6
    for m in range(2):  # the state holds FP32 positions
        ref = phys.positions(m)
        assert np.abs(X[m] - ref).max() <= 6e-8 * max(1.0, np.abs(ref).max())
    phys.close()

    # recovery from frame 3 reaches the same frame 6
    out2 = tmp_path / "out2"
    r = _run(exe, mp, pp, str(out2), "-r", str(out / "RecoveryStates" / "A00000003.json"))
    assert r.returncode == 0, r.stderr
    assert "3 frames" in r.stdout
    assert not (out2 / "A00000001.ply").exists() and (out2 / "A00000006.ply").exists()
    frame2, X2 = _state_positions(out2 / "RecoveryStates" / "A00000006.json")
    assert frame2 == 6
    for m in range(2):  # restarted from the FP32-rounded frame-3 state
        assert np.abs(X2[m] - X[m]).max() <= 1e-6


@pytest.mark.gpu
def test_binary_output_and_repo_root(gaia_lib, tmp_path):
    exe = _cli(gaia_lib)
    mp, pp = _scene(tmp_path, numFrames=4, outputExt="bin", binaryModeVisualizationSteps=2, outputRecoveryState=True,
                    outputRecoveryStateStep=4, outputRecoveryStateBinary=True)
    out = "${REPO_ROOT}/outbin"
    r = _run(exe, os.path.basename(mp).join(["${REPO_ROOT}/", ""]), os.path.basename(pp).join(["${REPO_ROOT}/", ""]),
             out, "-R", str(tmp_path))
    assert r.returncode == 0, r.stderr
    o = tmp_path / "outbin"
    # the template is written one file per model (writeAllToPLY(..., false, true))
    assert sorted(p.name for p in (o / "TemplateMesh").glob("*.ply")) == [
        "TemplateMesh_Model_000000_lower.ply", "TemplateMesh_Model_000001_upper.ply"]
    assert all((o / f"A{f:08d}.bin").exists() for f in range(5))
    assert sorted(p.name for p in o.glob("A*.ply")) == ["A00000000.ply", "A00000002.ply", "A00000004.ply"]
    assert sorted(p.name for p in (o / "RecoveryStates").glob("*.json")) == ["A00000000.json", "A00000004.json"]
    assert (o / "RecoveryStates" / "A00000004.pos").exists()
    # the bin frame holds the surface vertices of both meshes as FP32 xyz
    from gaia_gb300 import VBDPhysics

    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    ns = sum(len(phys.surface(m)[1]) for m in range(2))
    assert os.path.getsize(o / "A00000004.bin") == 12 * ns


def test_python_output_params(gaia_lib, tmp_path):
    from gaia_gb300 import VBDPhysics, scenes

    mp, pp = scenes.stack_drop(str(tmp_path), spacing=0.03)
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp)
    o = phys.outputParams()
    assert o["num_frames"] == 5000 and o["output_ext"] == "ply" and o["save_outputs"] == 0
    assert o["output_recovery_state_step"] == 10 and o["binary_mode_visualization_steps"] == 100


@pytest.mark.gpu
def test_python_simulate_writes_frames(gaia_lib, tmp_path):
    from gaia_gb300 import VBDPhysics

    mp, pp = _scene(tmp_path, numFrames=4, outputExt="ply", outputRecoveryStateStep=2,
                    outputRecoveryStateBinary=False)
    out = tmp_path / "pyout"
    phys = VBDPhysics()
    phys.loadRunningparameters(mp, pp, str(out))
    phys.initialize()
    assert phys.simulate() == 4 and phys.frameId == 4
    assert all((out / f"A{f:08d}.ply").exists() for f in range(5))
    assert sorted(p.name for p in (out / "RecoveryStates").glob("*.json")) == [
        "A00000000.json", "A00000002.json", "A00000004.json"]
    frame, X = _state_positions(out / "RecoveryStates" / "A00000004.json")
    assert frame == 4
    assert np.abs(X[1] - phys.positions(1)).max() <= 6e-8
    phys.close()
