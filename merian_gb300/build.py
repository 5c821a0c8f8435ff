"""Builds the in-tree native library ``merian_gb300/libgbpt.so`` for sm_103a.

The CUDA translation units go through ``nvcc -gencode arch=compute_103a,code=sm_103a``; the host
translation units through the host C++ compiler. All objects are compiled in parallel and linked
with the static CUDA runtime, so the library needs only the driver at run time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
INCLUDE = ROOT / "include"
BUILD = HERE / "_build"
LIB = HERE / "libgbpt.so"

CUDA_SOURCES = ["wavefront.cu", "kernels.cu", "nodes.cu", "debug_kernels.cu"]
HOST_SOURCES = ["api.cpp", "server.cpp", "bvh.cpp", "scenegen.cpp", "image_io.cpp", "pbrt_loader.cpp", "gltf_loader.cpp", "png.cpp", "graph.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    if proc.stdout.strip():
        sys.stderr.write(proc.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False,
          defines: tuple[str, ...] = (), lib: Path = LIB, build_dir: Path = BUILD) -> Path:
    """Compiles the library. `defines` (NAME=VALUE) override the kernels' tuning constants; a
    variant goes to its own `lib` and `build_dir`."""
    cuda = _cuda_home()
    BUILD = Path(build_dir)
    LIB = Path(lib)
    nvcc = str(cuda / "bin" / "nvcc")
    cxx = os.environ.get("CXX", "g++")
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "gbpt.h"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   *[f"-D{d}" for d in defines],
                   "-Xcompiler", "-fvisibility=hidden", "-I", str(INCLUDE), "-I", str(CSRC),
                   "-c", str(CSRC / src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in HOST_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            # no FMA contraction on the host: scene generation and BVH quantisation give the
            # same bits on x86-64 and aarch64
            jobs.append([cxx, "-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall",
                         "-ffp-contract=off", *[f"-D{d}" for d in defines],
                         "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(cuda / "include"),
                         "-c", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for fut in [ex.submit(_run, j) for j in jobs]:
                fut.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
