"""Build recipe of oracle/_ref/libnav24ref.so: nav24's own edge, camera-model and calibration code,
compiled from the reference tree's unmodified sources (TEST INFRASTRUCTURE).

The reference cannot be built with its own CMake project here (it needs g2o, Eigen, OpenCV, Boost
and glog, none of which are installed).  Its BA edge arithmetic, though, lives in a handful of
files that touch only a few fixed-size Eigen types, g2o's edge/vertex containers and SE3Quat, and
OpenCV value types.  This recipe compiles those files as they are, with g++, against the stand-in
headers under oracle/ref_shim (our own minimal implementations of those library names), plus
oracle/ref_harness.cpp, which exposes C entry points, and ref_shim/ref_parameter.cpp (the
parameter tree's member definitions; see that file for why the reference's own Parameter.cpp is
not used).  Nothing from the reference tree is copied:
the sources are read in place, and the objects and the library go to oracle/_ref/ (git-ignored).

The reference tree exists only in the build container; on a machine without it, build() returns
None and the tests that need the library use the vectors committed under tests/golden/.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
REFERENCE = Path(os.environ.get("NAV24_REFERENCE", "/root/reference"))

# reference sources compiled as they are (paths within the reference tree)
SOURCES = [
    "core/dataTypes/optimization/OptimizableTypes.cpp",
    "core/sensor/camera/Calibration.cpp",
    "core/sensor/camera/models/Pinhole.cpp",
    "core/sensor/camera/models/PinholeRadTan.cpp",
    "core/sensor/camera/models/KannalaBrandt8.cpp",
    "core/sensorData/observation/Point2D.cpp",
    "core/scene/worldObject/Point3D.cpp",
    "core/scene/worldObject/WorldObject.cpp",
]
# reference header directories (nav24 includes its headers by bare name)
INCLUDE_DIRS = [
    "core/dataTypes", "core/dataTypes/optimization", "core/sensor/camera", "core/sensor/camera/models",
    "core/tools/parameters", "core/sensorData/observation", "core/scene/worldObject",
]
# -ffp-contract=off: no FMA contraction, as in the oracle (the same results on x86-64 and aarch64)
# C++17: the reference's Parameter.hpp declares constructors with template-ids, which g++ 13 rejects
# in C++20 mode; its Parameter.cpp (std::map::contains, C++20) is replaced by ref_shim/ref_parameter.cpp
# (-include string: WorldObject.hpp names std::string and relies on a transitive include)
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-w", "-include", "string"]


def available() -> bool:
    return all((REFERENCE / s).exists() for s in SOURCES)


def _includes() -> list[str]:
    inc = ["-I", str(SHIM / "inc")]
    for d in INCLUDE_DIRS:
        inc += ["-I", str(REFERENCE / d)]
    return inc


def _compile(src: Path, obj: Path) -> None:
    cmd = ["g++", *FLAGS, *_includes(), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build() -> Path | None:
    """Compile oracle/_ref/libnav24ref.so from the reference's sources; None if the reference tree
    is absent (the GPU host).  Rebuilt when a source, stand-in header or this recipe is newer."""
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libnav24ref.so"
    shim = sorted(p for p in SHIM.rglob("*") if p.is_file())
    deps = [REFERENCE / s for s in SOURCES] + shim + [HERE / "ref_harness.cpp", Path(__file__).resolve(),
                                                      ROOT / "include" / "nav_ba.h"]
    if lib.exists() and all(d.stat().st_mtime <= lib.stat().st_mtime for d in deps):
        return lib
    units = [(REFERENCE / s, OUT / (s.replace("/", "_") + ".o")) for s in SOURCES]
    units.append((SHIM / "ref_parameter.cpp", OUT / "ref_parameter.o"))
    units.append((HERE / "ref_harness.cpp", OUT / "ref_harness.o"))
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(lambda u: _compile(*u), units))
    cmd = ["g++", "-shared", "-o", str(lib), *[str(o) for _, o in units]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed:\n" + r.stdout + r.stderr)
    return lib


if __name__ == "__main__":
    print(build())
