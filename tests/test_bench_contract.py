"""The benchmark's reference arm on the host (no GPU needed): the CPU restatement of the
reference's step timed on a bounded sample, printed as one JSON line with the keys the
benchmark contract names, from scene files written without the product library, so that
the process maps the oracle's library and not the product's.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RUN = r"""
import contextlib, io, json, sys
sys.argv = ["bench.py", "--impl", "reference"] + sys.argv[1:]
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"out": buf.getvalue(), "product": "libgaia_vbd" in maps, "oracle": "liboracle" in maps}))
"""


def _reference_line(*args):
    r = subprocess.run([sys.executable, "-c", _RUN, *args], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    lines = [ln for ln in res["out"].splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res["out"]
    return json.loads(lines[0]), res


@pytest.mark.skipif(not os.path.exists("/proc/self/maps"), reason="needs /proc/self/maps")
def test_reference_arm_line_and_libraries(oracle_lib):
    line, res = _reference_line("--workload", "drop", "--size", "4", "--iterations", "3", "--steps", "2",
                                "--warmup", "1", "--ref-budget", "2")
    assert line["impl"] == "reference"
    assert line["unit"] == "vertex-solves/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["dtype"] == "f32" and line["data"] == "synthetic"
    assert line["config"]["workload"].startswith("drop_cube_4^3")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the scene files come from the oracle's writers: the product library is never mapped
    assert res["oracle"] and not res["product"]


def test_reference_arm_other_ranks_print_nothing(oracle_lib):
    """Under a multi-process launch only rank 0 runs the CPU sample and prints the line: a
    process whose RANK is not 0 exits 0 without output (WORLD_SIZE stays 1 here, so that no
    process group is formed on a host without a GPU)."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "drop",
                        "--size", "4", "--iterations", "2", "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
