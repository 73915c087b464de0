"""Build recipe for librtr.so (sm_103a only).

Each CUDA translation unit is compiled by nvcc in parallel, host sources by
g++, and everything is linked into ``realtime_robot_gb300/librtr.so``.  A unit
is rebuilt when it or any header is newer than its object file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "librtr.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(INCLUDE)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir() -> Path:
    nv = Path(_nvcc()).resolve().parent.parent
    for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (nv / d / "libcudart_static.a").exists():
            return nv / d
    return nv / "lib64"


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, hdr_mtime: float, extra: list[str]) -> tuple[Path, str]:
    obj = BUILD / (src.name + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return obj, ""
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hm = _headers_mtime()
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    if ptxas_verbose:
        hm = float("inf")  # force a rebuild to get the report
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, hm, extra), srcs))
    objs = [o for o, _ in results]
    if verbose or ptxas_verbose:
        for (o, log) in results:
            if log:
                sys.stderr.write(f"--- {o.name}\n{log}\n")
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
               "-L", str(_cuda_lib_dir()), "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_demo()
    return LIB


CPP = PKG / "cpp"
DEMO = PKG / "realtime_robot_demo"


def build_demo() -> Path:
    """The C++ mirror of the reference's entry points (cpp/realtime_robot.hpp)
    exercised by its driver (cpp/realtime_robot_demo.cpp), linked to librtr.so."""
    src = CPP / "realtime_robot_demo.cpp"
    deps = [src, CPP / "realtime_robot.hpp", INCLUDE / "rtr.h", LIB]
    if DEMO.exists() and DEMO.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return DEMO
    cuda_inc = Path(_nvcc()).resolve().parent.parent / "include"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", str(INCLUDE), "-I", str(CPP), "-I", str(cuda_inc), str(src),
           "-o", str(DEMO), "-L", str(PKG), "-lrtr", "-L", str(_cuda_lib_dir()), "-lcudart_static", "-ldl", "-lrt",
           "-lpthread", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"demo build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return DEMO


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
