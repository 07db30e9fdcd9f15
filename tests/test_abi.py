"""CPU tests of the C ABI boundary: libnavba.so builds, loads, exports every entry point that
include/nav_ba.h declares, and its structs have the layout the Python binding assumes.  No call
here launches device work."""
import ctypes as C
import re
import subprocess
from pathlib import Path

from nav24_gb300 import _lib, abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "nav_ba.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nav_ba_[a-z_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(product_lib):
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    nm = subprocess.run(["nm", "-D", "--defined-only", str(product_lib)], capture_output=True, text=True).stdout
    for name in declared_functions():
        assert re.search(rf"\bT {name}\b", nm), name


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(f"""
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
#include "{ROOT / 'include' / 'nav_ba_synth.h'}"
int main(void) {{
  printf("%zu %zu %zu %zu\\n", sizeof(nav_ba_problem), sizeof(nav_ba_options), sizeof(nav_ba_result),
         sizeof(nav_synth_params));
  printf("%zu %zu %zu %zu\\n", offsetof(nav_ba_problem, intrinsics), offsetof(nav_ba_options, pcg_tolerance),
         offsetof(nav_ba_result, status), offsetof(nav_synth_params, min_points));
  printf("%zu %zu %zu %zu %zu\\n", sizeof(nav_ba_schedule), sizeof(nav_ba_cotangent), sizeof(nav_ba_grads),
         offsetof(nav_ba_schedule, lambda), offsetof(nav_ba_grads, cam_tangent));
  printf("%zu %zu %zu %zu\\n", sizeof(nav_ba_pose_problem), sizeof(nav_ba_pose_result),
         offsetof(nav_ba_pose_problem, intrinsics), offsetof(nav_ba_pose_result, status));
  printf("%zu %zu %zu\\n", sizeof(nav_ba_twoview), sizeof(nav_ba_twoview_result),
         offsetof(nav_ba_twoview, min_triangulated));
  return 0;
}}
""")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    got = list(map(int, out))
    want = [C.sizeof(abi.nav_ba_problem), C.sizeof(abi.nav_ba_options), C.sizeof(abi.nav_ba_result),
            C.sizeof(abi.nav_synth_params), abi.nav_ba_problem.intrinsics.offset,
            abi.nav_ba_options.pcg_tolerance.offset, abi.nav_ba_result.status.offset,
            abi.nav_synth_params.min_points.offset,
            C.sizeof(abi.nav_ba_schedule), C.sizeof(abi.nav_ba_cotangent), C.sizeof(abi.nav_ba_grads),
            abi.nav_ba_schedule.lam.offset, abi.nav_ba_grads.cam_tangent.offset,
            C.sizeof(abi.nav_ba_pose_problem), C.sizeof(abi.nav_ba_pose_result),
            abi.nav_ba_pose_problem.intrinsics.offset, abi.nav_ba_pose_result.status.offset,
            C.sizeof(abi.nav_ba_twoview), C.sizeof(abi.nav_ba_twoview_result),
            abi.nav_ba_twoview.min_triangulated.offset]
    assert got == want


def test_option_defaults_match_binding(product_lib):
    L = _lib.load()
    o = abi.nav_ba_options()
    L.nav_ba_options_default(C.byref(o))
    d = abi.default_options()
    for name, _ in abi.nav_ba_options._fields_:
        if name == "reserved":
            continue
        assert getattr(o, name) == getattr(d, name), name
    assert L.nav_ba_abi_version() == 2
    assert L.nav_ba_status_string(abi.ERR_UNSUPPORTED).decode() == "unsupported size or option"


def test_null_arguments_are_rejected_without_a_device(product_lib):
    L = _lib.load()
    assert L.nav_ba_solve(None, None, None, None) == abi.ERR_ARGUMENT
    assert L.nav_ba_create(None, 0) == abi.ERR_ARGUMENT
    assert L.nav_ba_last_error(None).decode() == ""


def test_missing_library_fails_loudly(tmp_path):
    import pytest
    with pytest.raises(_lib.NativeLibraryMissing):
        _lib.load(tmp_path / "libnavba.so")
