"""Build recipes for the native libraries of the package.

  libnavba.so    the product: CUDA sm_103a kernels + C ABI (include/nav_ba.h)
  libnavsynth.so the seeded synthetic-problem generator (include/nav_ba_synth.h), host only

Everything is compiled in-tree into nav24_gb300/_build/ with nvcc / g++ directly (no cmake),
translation units in parallel.  Objects are rebuilt only when a source or header is newer.
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
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction (-ffp-contract=off) so that the synthetic
# problems and every host-side floating-point result are the same on x86-64 and aarch64 (gcc fuses
# a*b+c into an FMA by default on aarch64 only).
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]

PRODUCT_CU = ["nav_ba_api.cu", "window_engine.cu", "grid_engine.cu", "noalloc.cu", "pose_engine.cu", "twoview.cu", "undistort.cu"]
PRODUCT_CPP = ["structure.cpp"]
SYNTH_CPP = ["synth.cpp"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    # this file is a dependency too: a change of flags rebuilds everything
    return (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + sorted(INCLUDE.glob("*.h")) +
            [Path(__file__).resolve()])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_product(verbose: bool = False) -> Path:
    """Compile libnavba.so (CUDA sm_103a) and return its path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = str(cuda_home() / "bin" / "nvcc")
    hdrs = _headers()
    jobs, objs = [], []
    for src in PRODUCT_CU:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    for src in PRODUCT_CPP:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(cuda_home() / "include"),
                         "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd))
        list(ex.map(_run, jobs))
    lib = BUILD / "libnavba.so"
    if _newer(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lpthread"])
    return lib


def build_synth() -> Path:
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libnavsynth.so"
    srcs = [CSRC / s for s in SYNTH_CPP]
    if _newer(lib, srcs + _headers()):
        _run(["g++", *CXX_FLAGS, "-shared", "-I", str(INCLUDE), "-o", str(lib), *map(str, srcs)])
    return lib


def build_all(verbose: bool = False) -> dict:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_product, verbose)
        f2 = ex.submit(build_synth)
        return {"navba": f1.result(), "synth": f2.result()}


if __name__ == "__main__":
    print(build_all(verbose=True))
