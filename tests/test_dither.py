"""The dithered FP32 constants of the mixed precision passes (cfgpu_dither_versions, host only).

Each constant exists in V = 64 versions cycled one per nonlinear evaluation, so that the rounding of a fixed
operator does not repeat every step.  Properties:
* every version is one of the two floats that bracket x;
* the mean of the V versions is x to 1/(2V) of the float spacing, with no bias over many constants;
* constants that are floats (powers of two among them) are exact in every version;
* version 0 is round-to-nearest except within 1/(2V) of a spacing of the midpoint.
"""

import ctypes as C

import numpy as np
import pytest

V = 64


@pytest.fixture(scope="module")
def versions():
    from channelflow_gb300 import _lib as L
    from channelflow_gb300 import build
    build.build()
    lib = L.load()
    buf = (C.c_float * V)()

    def get(x):
        L.check(lib.cfgpu_dither_versions(float(x), buf))
        return np.frombuffer(buf, dtype=np.float32).copy()
    return get


def _spacing(x):
    lo = np.float32(x)
    if float(lo) > x:
        lo = np.nextafter(lo, np.float32(-np.inf))
    return float(np.nextafter(lo, np.float32(np.inf))) - float(lo), float(lo)


def test_versions_bracket_and_average(versions):
    rng = np.random.default_rng(0)
    xs = rng.standard_normal(3000) * 10.0 ** rng.uniform(-6, 6, 3000)
    errs = []
    for x in xs:
        v = versions(x).astype(np.float64)
        sp, lo = _spacing(x)
        assert np.all((v == lo) | (v == lo + sp)), x
        errs.append((v.mean() - x) / sp)
    errs = np.array(errs)
    assert np.abs(errs).max() <= 1.0 / (2 * V) + 1e-12
    assert abs(errs.mean()) <= 0.002           # unbiased over many constants


@pytest.mark.parametrize("x", [1.0, -1.0, 0.5, 2.0 ** -14, 4.0, 9216.0, 0.0, 0.75, -3.0])
def test_float_constants_exact(versions, x):
    assert np.all(versions(x) == np.float32(x))


def test_version0_nearest(versions):
    rng = np.random.default_rng(1)
    xs = rng.uniform(-100, 100, 2000)
    same = np.mean([versions(x)[0] == np.float32(x) for x in xs])
    assert same >= 0.9


def test_null_argument_rejected():
    from channelflow_gb300 import _lib as L
    from channelflow_gb300 import build
    build.build()
    with pytest.raises(L.CfgpuError):
        L.check(L.load().cfgpu_dither_versions(1.0, None))
