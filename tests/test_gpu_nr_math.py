"""Error bounds of the FP64 Newton-Raphson reciprocal and reciprocal square root that the kernels use
in place of the IEEE divide and square root (recip_nr / recip<double> for 1/z of the depths, rsqrt_nr
for the two-view rotations; nav24_gb300/csrc/ba_math.cuh).  Each refines an FP32 estimate with two
Newton steps.  Measured on the device over 2^21 inputs log-uniform in magnitude over [1e-20, 1e20]
(both signs for the reciprocal) plus powers of two and the edges of the FP32-estimate range, against
the correctly rounded results (an FP64 divide; 1/sqrt in extended precision on the host): the reciprocal is within
1 ulp, the reciprocal square root within 2 ulps, and the device's IEEE operations agree with the
host's reference."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from nav24_gb300.build import ARCH, INCLUDE, cuda_home

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent / "gpu_math"


@pytest.fixture(scope="module")
def nr_lib():
    out = HERE / "_build"
    out.mkdir(exist_ok=True)
    lib = out / "libnr_check.so"
    src = HERE / "nr_check.cu"
    subprocess.run([str(cuda_home() / "bin" / "nvcc"), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                    "-I", str(INCLUDE), str(src), "-o", str(lib)], check=True, capture_output=True)
    L = C.CDLL(str(lib))
    L.nr_eval.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]
    L.nr_eval.restype = C.c_int
    return L


def ulps(a, b):
    """Distance in units in the last place between doubles of the same sign."""
    ia = np.ascontiguousarray(a).view(np.int64)
    ib = np.ascontiguousarray(b).view(np.int64)
    return np.abs(ia - ib)  # in int64: the bit patterns exceed FP64's exact integer range


def inputs():
    rng = np.random.default_rng(2024)
    mag = 10.0 ** rng.uniform(-20.0, 20.0, 1 << 21)
    sign = np.where(rng.random(mag.size) < 0.5, -1.0, 1.0)
    pow2 = 2.0 ** np.arange(-66, 67, dtype=np.float64)
    edges = np.array([1.0000001e-30, 9.999999e29, 1e-30, 1e30, 3.0, 1.0 / 3.0, 7.0, np.pi])
    return np.concatenate([mag * sign, pow2, -pow2, edges])


def test_newton_raphson_reciprocals_within_ulps(nr_lib):
    z = np.ascontiguousarray(inputs())
    out = np.zeros((z.size, 4))
    assert nr_lib.nr_eval(z.ctypes.data_as(C.POINTER(C.c_double)), z.size,
                          out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    recip_ref = 1.0 / z  # an IEEE FP64 divide: correctly rounded
    # 1/sqrt in extended precision (IEEE quad on aarch64), rounded once to FP64
    rsqrt_ref = (np.longdouble(1) / np.sqrt(np.abs(z).astype(np.longdouble))).astype(np.float64)
    # the device's IEEE operations are the correctly rounded results (sanity of the reference)
    assert np.array_equal(out[:, 1], recip_ref)
    assert ulps(out[:, 3], rsqrt_ref).max() <= 1
    d_recip = ulps(out[:, 0], recip_ref)
    d_rsqrt = ulps(out[:, 2], rsqrt_ref)
    assert d_recip.max() <= 1, (d_recip.max(), z[np.argmax(d_recip)])
    assert d_rsqrt.max() <= 2, (d_rsqrt.max(), z[np.argmax(d_rsqrt)])
