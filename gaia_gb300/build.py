"""Build libgaia_vbd.so in-tree with nvcc for sm_103a.

Translation units compiled in parallel (host scene code, the tet and cloth
engines, the cloth contact detector), one -gencode, no cmake. Outputs:
gaia_gb300/libgaia_vbd.so and the command-line runner gaia_gb300/vbd_dynamics
(Models.json Parameters.json outFolder [-R repoRoot] [-r recoveryState]),
linked against the library with an $ORIGIN rpath.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgaia_vbd.so")
CLI = os.path.join(HERE, "vbd_dynamics")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["scene.cpp", "state_io.cpp", "vbd_engine.cu", "vbd_engine_f32.cu", "vbd_engine_df.cu", "vbd_engine_dfh.cu",
           "vbd_engine_f64.cu", "vbd_energy_noalloc.cu", "tet_cd.cu", "coloring_gpu.cu", "cloth_scene.cpp", "cloth_cd.cu",
           "cloth_engine.cu"]
# every header of csrc/ is a dependency of every translation unit
HEADERS = sorted(f for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h")))
PUBLIC_HEADERS = ["gaia_vbd.h", "gaia_cloth.h"]
# The contact detector's predicates must round like the CPU restatement: no FMA contraction.
EXTRA_FLAGS = {"cloth_cd.cu": ["--fmad=false"], "tet_cd.cu": ["--fmad=false"]}


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; set NVCC or put the CUDA toolkit on PATH")
    return cand


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    deps = ([os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] +
            [os.path.join(INCLUDE, h) for h in PUBLIC_HEADERS])
    if not _stale(obj, deps) and not verbose_ptxas:
        return obj
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, *ARCH]
    if src.endswith(".cu"):
        cmd += ["--expt-relaxed-constexpr", "-Xptxas", "-O3", *EXTRA_FLAGS.get(src, [])]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB, *objs, *ARCH, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "vbd_dynamics.cpp")
    cli_deps = [cli_src, LIB, os.path.join(INCLUDE, "gaia_vbd.h"), os.path.join(INCLUDE, "gaia_vbd.hpp")]
    if force or _stale(CLI, cli_deps):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-o", CLI, cli_src, "-I", INCLUDE, "-L", HERE,
               "-lgaia_vbd", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"vbd_dynamics build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
