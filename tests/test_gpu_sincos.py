"""The double-float sine and cosine of the one-pose kernel (df_sincos, on the
FP32 pipe) against FP64, through mmo_diag_sincos: absolute error at most
1e-14 + |x| 1e-16 (double-float operations carry about 2^-46 each; the
reduction's pi / 2 is rounded to double, 6e-17 per quadrant), hi + lo a
normalised pair, and the FP64 library value for |x| >= 1e5."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eval(gpu_lib, x):
    from mmo_gb300 import lib as L

    h = C.c_void_p()
    assert gpu_lib.mmo_ctx_create(0, C.byref(h)) == L.OK
    try:
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty((len(x), 4), np.float32)
        rc = gpu_lib.mmo_diag_sincos(h, len(x), x.ctypes.data_as(C.POINTER(C.c_float)),
                                     out.ctypes.data_as(C.POINTER(C.c_float)))
        assert rc == L.OK, gpu_lib.mmo_last_error(h)
    finally:
        gpu_lib.mmo_ctx_destroy(h)
    return x, out


def test_df_sincos_error_bound(gpu_lib):
    rng = np.random.default_rng(11)
    q = np.pi / 4
    x = np.concatenate([
        rng.uniform(-7.0, 7.0, 20000),
        rng.uniform(-100.0, 100.0, 20000),
        rng.uniform(-1e4, 1e4, 5000),
        # around the reduction's quadrant edges and the multiples of pi / 2
        np.array([np.nextafter(np.float32(k * q), np.float32(s * np.inf))
                  for k in range(-40, 41) for s in (-1, 1)], np.float32),
        np.arange(-40, 41) * np.float32(np.pi / 2),
        [0.0, -0.0, 1e-30, -1e-30, 1e-8, 3.0e-4],
    ]).astype(np.float32)
    x, out = _eval(gpu_lib, x)
    xd = x.astype(np.float64)
    s = out[:, 0].astype(np.float64) + out[:, 1].astype(np.float64)
    c = out[:, 2].astype(np.float64) + out[:, 3].astype(np.float64)
    bound = 1e-14 + np.abs(xd) * 1e-16
    assert np.all(np.abs(s - np.sin(xd)) <= bound), float(np.max(np.abs(s - np.sin(xd)) / bound))
    assert np.all(np.abs(c - np.cos(xd)) <= bound), float(np.max(np.abs(c - np.cos(xd)) / bound))
    # normalised pairs: |lo| <= ulp(hi) / 2
    for h_, l_ in ((out[:, 0], out[:, 1]), (out[:, 2], out[:, 3])):
        ulp = np.spacing(np.abs(h_)).astype(np.float64)
        assert np.all(np.abs(l_.astype(np.float64)) <= ulp / 2 + 1e-45)


def test_df_sincos_large_arguments_take_the_library(gpu_lib):
    x = np.array([1e5, -2.5e5, 3.0e7, 1e30], np.float32)
    x, out = _eval(gpu_lib, x)
    xd = x.astype(np.float64)
    s = out[:, 0].astype(np.float64) + out[:, 1].astype(np.float64)
    c = out[:, 2].astype(np.float64) + out[:, 3].astype(np.float64)
    assert np.all(np.abs(s - np.sin(xd)) <= 1e-14)
    assert np.all(np.abs(c - np.cos(xd)) <= 1e-14)
