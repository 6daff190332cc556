"""Build the native libraries in-tree.

Outputs (all git-ignored):
  vertexsurge_gb300/libvsgb300.so  CUDA kernels + the C ABI (include/vertexsurge_gb300.h)
  vertexsurge_gb300/libvsgen.so    synthetic graph generators (host C++/OpenMP)
  vertexsurge_gb300/libvsops.so    C++ operator layer over the C ABI (VExpand, HashJoin, ...)
  vertexsurge_gb300/vs_ops_test    operator-level known-answer tests (C++)
  oracle/build/liboracle.so        CPU oracle (test infrastructure)

Every CUDA translation unit is compiled for sm_103a only, in parallel.
Sources are rebuilt only when newer than their outputs.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "build"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fno-strict-aliasing", "-I", str(ROOT / "include")]
CXX_FLAGS = ["-O3", "-std=c++20", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["api.cu", "expand.cu", "matrix.cu", "join.cu", "intersect.cu", "picker.cu", "consumers.cu",
              "filter.cu"]

LIB = PKG / "libvsgb300.so"
GEN_LIB = PKG / "libvsgen.so"
OPS_LIB = PKG / "libvsops.so"
OPS_TEST = PKG / "vs_ops_test"
ORACLE_LIB = ORACLE / "build" / "liboracle.so"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "vertexsurge_gb300.h"]


def build_cuda(jobs: int = 8) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    objs = []
    todo = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            todo.append([nvcc()] + NVCC_FLAGS + ["-c", str(s), "-o", str(o)])
    if todo:
        with ThreadPoolExecutor(max_workers=max(1, min(jobs, len(todo)))) as ex:
            for f in [ex.submit(_run, c) for c in todo]:
                f.result()
    if _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs])
    return LIB


def build_gen() -> Path:
    src = CSRC / "host" / "graphgen.cpp"
    if _stale(GEN_LIB, [src, CSRC / "host" / "graphgen.h"]):
        _run(["g++"] + CXX_FLAGS + ["-shared", str(src), "-o", str(GEN_LIB)])
    return GEN_LIB


def build_ops() -> Path:
    srcs = [PKG / "cpp" / "vs_operators.cpp", PKG / "cpp" / "graph_dir.cpp", PKG / "cpp" / "vql.cpp"]
    hdrs = [PKG / "cpp" / "vs_operators.hh", PKG / "cpp" / "vql.hh", ROOT / "include" / "vertexsurge_gb300.h"]
    if not srcs[0].exists():
        return OPS_LIB
    if _stale(OPS_LIB, srcs + hdrs + [LIB]):
        _run(["g++"] + CXX_FLAGS + ["-shared", "-I", str(ROOT / "include")] + [str(s) for s in srcs]
             + ["-L", str(PKG), "-lvsgb300", "-Wl,-rpath,$ORIGIN", "-o", str(OPS_LIB)])
    test_src = PKG / "cpp" / "vs_ops_test.cpp"
    if test_src.exists() and _stale(OPS_TEST, [test_src, OPS_LIB] + hdrs):
        _run(["g++"] + CXX_FLAGS + ["-I", str(ROOT / "include"), str(test_src),
              "-L", str(PKG), "-lvsops", "-lvsgb300", "-Wl,-rpath,$ORIGIN", "-o", str(OPS_TEST)])
    return OPS_LIB


def build_oracle() -> Path:
    src = ORACLE / "oracle.cpp"
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if _stale(ORACLE_LIB, [src, ORACLE / "oracle.h"]):
        _run(["g++"] + CXX_FLAGS + ["-shared", str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_all(jobs: int = 8) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        fs = [ex.submit(build_cuda, jobs), ex.submit(build_gen), ex.submit(build_oracle)]
        for f in fs:
            f.result()
    build_ops()


if __name__ == "__main__":
    build_all()
    print("built", LIB, GEN_LIB, ORACLE_LIB)
