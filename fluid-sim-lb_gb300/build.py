"""Build recipe for libfsim.so (CUDA, sm_103a) and the oracle library.

No cmake: each translation unit is compiled by nvcc in parallel, then linked
with ``nvcc -shared``.  The oracle (test infrastructure, under ``oracle/``) is
built with g++ in strict IEEE mode (-O2 -ffp-contract=off, no fast-math).
Outputs are in-tree and git-ignored:
  fluid-sim-lb_gb300/lib/libfsim.so
  oracle/build/liboracle_fsim.so
  fluid-sim-lb_gb300/lib/fsim_demo          (C++ facade example binary)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-prec-div=true", "-prec-sqrt=true",
              "-fmad=false"]
SOURCES = ["fsim_api.cu", "k_topology.cu", "k_grid.cu", "k_pcg.cu", "k_g2p.cu", "k_noalloc.cu", "k_adjoint.cu", "scene.cu", "k_levelset.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    return "nvcc"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} {cmd[-1]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_fsim(force: bool = False, verbose: bool = False) -> Path:
    LIB.mkdir(parents=True, exist_ok=True)
    obj_dir = LIB / "obj"
    obj_dir.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [INCLUDE / "fsim.h"]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = obj_dir / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    so = LIB / "libfsim.so"
    if force or jobs or _stale(so, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(so), *map(str, objs), "-lcudart"])
    return so


def build_oracle(force: bool = False) -> Path:
    out_dir = ORACLE / "build"
    out_dir.mkdir(parents=True, exist_ok=True)
    so = out_dir / "liboracle_fsim.so"
    src = ORACLE / "oracle.cc"
    if force or _stale(so, [src, ORACLE / "oracle.h"]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
              "-fno-fast-math", "-Wall", "-o", str(so), str(src)])
    return so


def build_demo(force: bool = False) -> Path | None:
    """C++ program that drives the reference-named facade over the C ABI."""
    src = PKG / "host" / "flip_demo.cc"
    if not src.exists():
        return None
    out = LIB / "fsim_demo"
    deps = [src, LIB / "libfsim.so"] + list((PKG / "host").glob("*.h"))
    if force or _stale(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), "-I", str(PKG / "host"),
              "-o", str(out), str(src), "-L", str(LIB), "-lfsim", f"-Wl,-rpath,{LIB}"])
    return out


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_fsim, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()
    build_demo(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB / "libfsim.so")
