"""Build recipe of the CPU oracle (test infrastructure): oracle/_build/libnavba_oracle.so.

The oracle is plain C++17 with no dependencies; it is compiled with g++ directly.  The
reference's whole BA path cannot be compiled here (it needs g2o, Eigen, OpenCV, Boost and glog,
none of which exist in this environment); its edge and camera-model code is, against stand-in
headers, by oracle/ref_build.py into oracle/_ref.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"


def build() -> Path:
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libnavba_oracle.so"
    srcs = [HERE / "ba_oracle.cpp"]
    deps = srcs + [HERE / "ba_oracle.h", HERE.parent / "include" / "nav_ba.h", Path(__file__).resolve()]
    if not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
        # no FMA contraction: the same results on x86-64 and aarch64
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-Wall", "-Wextra", "-pthread",
               "-o", str(lib), *map(str, srcs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return lib


if __name__ == "__main__":
    print(build())
