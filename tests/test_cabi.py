"""The C-ABI library loads and exports every function declared in include/cfgpu.h (no GPU needed)."""

import ctypes

import pytest

from channelflow_gb300 import _lib as L
from channelflow_gb300 import DNSFlags


@pytest.fixture(scope="module")
def lib():
    from channelflow_gb300 import build
    build.build()
    return L.load()


def test_exports_every_header_symbol(lib):
    names = L.header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_flags_default_matches_reference_defaults(lib):
    f = L.Flags()
    assert lib.cfgpu_flags_default(ctypes.byref(f)) == 0
    d = DNSFlags()
    for k in ("nu", "dt", "baseflow", "constraint", "timestepping", "initstepping", "nonlinearity", "dealiasing"):
        assert getattr(f, k) == getattr(d, k), k
    assert f.taucorrection == 1


def test_version_and_errors(lib):
    assert lib.cfgpu_version().startswith(b"cfgpu")
    assert lib.cfgpu_flags_default(None) == L.CFGPU_EINVAL
    assert b"null" in lib.cfgpu_last_error()
