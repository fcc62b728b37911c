"""The deterministic FP32 sin/cos/acos used by the FP32-storage path, against
FP64 libm (numpy), within a few ulp over the argument ranges the moves use;
and the 32-bit-conversion fixed-point rounding of trilinear weights against
llrint(w * 2^40) for every binary32 weight in [0, 1]."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

HDR = Path(__file__).resolve().parents[1] / "chromo_gb300" / "csrc" / "cg_math32.h"


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("m32")
    src = d / "m32.c"
    src.write_text(f'#include "{HDR}"\n'
                   "void sc(const float* x, float* s, float* c, int n)"
                   "{ for (int i = 0; i < n; i++) cgm_sincosf(x[i], s + i, c + i); }\n"
                   "void ac(const float* x, float* y, int n) { for (int i = 0; i < n; i++) y[i] = cgm_acosf(x[i]); }\n"
                   "#include <string.h>\n"
                   "long long q40_bad(unsigned lo, unsigned hi) { long long bad = 0;"
                   " for (unsigned b = lo; ; b++) { float w; memcpy(&w, &b, 4);"
                   " if (cgm_q40f(w) != llrint((double)w * 1099511627776.0)) bad++;"
                   " if (b == hi) break; } return bad; }\n")
    so = d / "m32.so"
    subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off", "-o", str(so), str(src), "-lm"])
    L = ctypes.CDLL(str(so))
    L.sc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.ac.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    L.q40_bad.argtypes = [ctypes.c_uint, ctypes.c_uint]
    L.q40_bad.restype = ctypes.c_longlong
    return L


def ulp_err(got, ref):
    ref32 = ref.astype(np.float32)
    spacing = np.spacing(np.abs(ref32).astype(np.float32)).astype(np.float64)
    spacing = np.maximum(spacing, np.spacing(np.float32(1e-30)))
    return np.abs(got.astype(np.float64) - ref) / spacing


def test_sincos_accuracy(lib):
    x = np.concatenate([np.linspace(-2 * np.pi, 2.5 * np.pi, 400001),
                        np.random.default_rng(1).uniform(-40, 40, 200000)]).astype(np.float32)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib.sc(x.ctypes.data, s.ctypes.data, c.ctypes.data, len(x))
    xd = x.astype(np.float64)
    assert np.max(np.abs(s - np.sin(xd))) < 3e-7
    assert np.max(np.abs(c - np.cos(xd))) < 3e-7
    big = np.abs(np.sin(xd)) > 1e-3
    assert np.max(ulp_err(s[big], np.sin(xd[big]))) <= 4


def test_acos_accuracy(lib):
    x = np.concatenate([np.linspace(-1, 1, 400001), [-1.0, 1.0, 0.5, -0.5]]).astype(np.float32)
    y = np.empty_like(x)
    lib.ac(x.ctypes.data, y.ctypes.data, len(x))
    ref = np.arccos(x.astype(np.float64))
    assert np.max(np.abs(y - ref)) < 5e-7
    assert y[-4] == 0.0 or abs(y[-4] - np.pi) < 1e-6


def test_fixed_point_weights_exhaustive(lib):
    """cgm_q40f(w) == llrint(w * 2^40) for all 1,065,353,217 binary32 values
    in [0, 1] (0x00000000 .. 0x3F800000): the GPU deposits weights with
    32-bit conversions only and must produce the oracle's int64 grid."""
    assert lib.q40_bad(0, 0x3F800000) == 0
