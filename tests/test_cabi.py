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


def test_argument_errors_need_no_gpu(lib):
    """Argument checks run before any CUDA call, so they return EINVAL on a machine without a GPU."""
    import ctypes as C
    g = L.Grid(16, 17, 16, 1.0, 1.0, -1.0, 1.0)
    f = L.Flags()
    lib.cfgpu_flags_default(C.byref(f))
    h = C.c_void_p()
    assert lib.cfgpu_ensemble_create(C.byref(g), C.byref(f), 0, L.CFGPU_FP64, C.byref(h)) == L.CFGPU_EINVAL
    assert lib.cfgpu_ensemble_create(C.byref(g), C.byref(f), 2, 7, C.byref(h)) == L.CFGPU_EINVAL
    assert lib.cfgpu_ensemble_set_field(None, 0, None, None) == L.CFGPU_EINVAL
    assert lib.cfgpu_dns_create(C.byref(g), C.byref(f), None, None, None, 9, C.byref(h)) == L.CFGPU_EINVAL
    assert lib.cfgpu_tau_solve_batched(4, 1, None, None, 1.0, 1.0, -1.0, 1.0, 1.0, 1.0, 1,
                                       None, None, None, None, None, None, None) == L.CFGPU_EINVAL
    assert lib.cfgpu_host_register(None, 8) == L.CFGPU_EINVAL
    buf = C.create_string_buffer(64)
    assert lib.cfgpu_host_register(C.cast(buf, C.c_void_p), 0) == L.CFGPU_EINVAL
    assert lib.cfgpu_host_unregister(None) == L.CFGPU_EINVAL
    # form switches: host-side state only (no CUDA call); out-of-range modes refused
    assert lib.cfgpu_set_fused_xz(3) == L.CFGPU_EINVAL
    assert lib.cfgpu_set_fused_xz(-1) == L.CFGPU_EINVAL
    for fn in ("cfgpu_set_fused_xz", "cfgpu_set_pdl", "cfgpu_set_register_zpass"):
        assert getattr(lib, fn)(0) == L.CFGPU_OK
        assert getattr(lib, fn)(1) == L.CFGPU_OK
