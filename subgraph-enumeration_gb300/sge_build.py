"""Builds libsge.so (CUDA engine + host planner/IO), the graph_mining_system CLI,
and the oracle library, in-tree under ``_build/`` directories.

The CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host translation units are
compiled with g++ in parallel so a clean build takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
INC = REPO / "include"
OUT = PKG / "_build"
ORACLE = REPO / "oracle"
ORACLE_OUT = ORACLE / "_build"

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SRCS = ["planner.cpp", "graph_io.cpp", "generators.cpp"]
CU_SRCS = ["engine.cu", "mlp.cu", "relation.cu", "ingest.cu"]


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_sge(verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = [INC / "sge.h", CSRC / "common.hpp", CSRC / "device_util.hpp"]
    jobs = []
    objs = []
    for s in CU_SRCS:
        o = OUT / (Path(s).stem + ".cu.o")
        objs.append(o)
        if _stale(o, [CSRC / s] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3",
                         f"-I{INC}", f"-I{CSRC}", "-c", str(CSRC / s), "-o", str(o)])
    for s in HOST_SRCS:
        o = OUT / (Path(s).stem + ".o")
        objs.append(o)
        if _stale(o, [CSRC / s] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wno-unused-function",
                         f"-I{INC}", f"-I{CSRC}", "-c", str(CSRC / s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    lib = OUT / "libsge.so"
    if _stale(lib, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lpthread"])
    cli = OUT / "graph_mining_system"
    if _stale(cli, [lib, CSRC / "cli_main.cpp", INC / "sge.h"]):
        _run(["g++", "-O2", "-std=c++17", f"-I{INC}", str(CSRC / "cli_main.cpp"), "-o", str(cli),
              f"-L{OUT}", "-lsge", "-Wl,-rpath,$ORIGIN"])
    return lib


def build_oracle() -> Path:
    ORACLE_OUT.mkdir(parents=True, exist_ok=True)
    so = ORACLE_OUT / "liboracle.so"
    src = ORACLE / "sge_oracle.c"
    if _stale(so, [src, INC / "sge.h"]):
        _run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(so), "-lm"])
    return so


def build_reference(ref: Path | None = None) -> Path | None:
    """Compiles the reference executor from its sources into oracle/_ref (only
    where a reference checkout is named, by argument or by the SGE_REFERENCE
    environment variable; the result is never committed)."""
    if ref is None:
        env = os.environ.get("SGE_REFERENCE")
        if not env:
            return None
        ref = Path(env)
    if not (ref / "main.cpp").exists() or shutil.which("make") is None:
        return None
    _run(["make", "-f", str(ORACLE / "ref.mk"), f"REF={ref}", f"OUT={ORACLE / '_ref'}",
          f"-j{os.cpu_count() or 4}"], cwd=REPO)
    return ORACLE / "_ref" / "graph_mining_system"


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_sge, verbose)
        f2 = ex.submit(build_oracle)
        f1.result()
        f2.result()
    build_reference()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", OUT / "libsge.so")
