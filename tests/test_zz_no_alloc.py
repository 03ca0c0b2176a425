"""The allocation-free batched tau solve agrees with the allocating one.

cfgpu_tau_solve_batched_noalloc serves callers that must not allocate GPU
memory (their GPU memory is fully reserved by another allocator, or they run
latency-sensitive loops): it takes all device working memory from a static
16 MiB array inside the library.  This file is collected last on purpose.
"""

import ctypes as C

import numpy as np
import pytest

from channelflow_gb300 import _lib as L
from tests.test_oracle_golden import tau_case

pytestmark = pytest.mark.gpu
TOL = 1e-12  # same tolerance as the batched tau parity test


@pytest.fixture(scope="module")
def lib():
    from channelflow_gb300 import build
    build.build()
    return L.load()


def _solve(lib, fn, N, kx, kz, c, R):
    outs = [np.zeros((kx.shape[0], N), dtype=np.complex128) for _ in range(4)]
    L.check(getattr(lib, fn)(int(N), int(kx.shape[0]), L.iptr(kx), L.iptr(kz), c["Lx"], c["Lz"], c["a"], c["b"],
                             c["lam_t"], c["nu"], 1, *[L.dptr(r) for r in R], *[L.dptr(o) for o in outs]))
    return outs


def test_noalloc_matches_allocating_entry_point_twice(lib):
    rng = np.random.default_rng(99)
    for call in range(2):
        c = tau_case(rng)
        N = c["N"]
        nm = 40 + 17 * call
        kx = rng.integers(-20, 21, nm).astype(np.int32)
        kz = rng.integers(0, 21, nm).astype(np.int32)
        kx[0], kz[0] = 0, 0
        R = [np.ascontiguousarray(np.stack([c[k] * (1 + 0.1 * j) for j in range(nm)])) for k in ("Rx", "Ry", "Rz")]
        ref = _solve(lib, "cfgpu_tau_solve_batched", N, kx, kz, c, R)
        got = _solve(lib, "cfgpu_tau_solve_batched_noalloc", N, kx, kz, c, R)
        for a, b in zip(got, ref):
            assert np.abs(a - b).max() <= TOL * max(1.0, np.abs(b).max())


def _free_device_bytes():
    cudart = None
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            cudart = C.CDLL(name)
            break
        except OSError:
            continue
    assert cudart is not None, "CUDA runtime library not found"
    free, total = C.c_size_t(), C.c_size_t()
    assert cudart.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def test_noalloc_call_leaves_device_memory_unchanged(lib):
    """After the first call (which may reserve the static array), further calls take no device memory."""
    rng = np.random.default_rng(5)
    c = tau_case(rng)
    N, nm = c["N"], 24
    kx = rng.integers(-8, 9, nm).astype(np.int32)
    kz = rng.integers(0, 9, nm).astype(np.int32)
    R = [np.ascontiguousarray(np.stack([c[k]] * nm)) for k in ("Rx", "Ry", "Rz")]
    first = _solve(lib, "cfgpu_tau_solve_batched_noalloc", N, kx, kz, c, R)
    before = _free_device_bytes()
    second = _solve(lib, "cfgpu_tau_solve_batched_noalloc", N, kx, kz, c, R)
    after = _free_device_bytes()
    assert after == before
    for a, b in zip(first, second):
        assert np.array_equal(a, b)


def test_noalloc_rejects_oversize_request(lib):
    N, nm = 97, 400
    kx = np.zeros(nm, np.int32)
    kz = np.zeros(nm, np.int32)
    R = [np.zeros((nm, N), np.complex128) for _ in range(3)]
    outs = [np.zeros((nm, N), np.complex128) for _ in range(4)]
    code = lib.cfgpu_tau_solve_batched_noalloc(N, nm, L.iptr(kx), L.iptr(kz), 1.0, 1.0, -1.0, 1.0, 1.0, 1e-3, 1,
                                               *[L.dptr(r) for r in R], *[L.dptr(o) for o in outs])
    assert code == L.CFGPU_EINVAL
    assert b"static working array" in lib.cfgpu_last_error()
