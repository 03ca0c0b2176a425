"""FlowField::makePhysical / makeSpectral and their halves on the GPU against the oracle.

Reference: channelflow/flowfield.cpp:1850-2020 (the xz FFTs with the 1/(Nx Nz) forward scale, the y
Chebyshev transform with the chebyfft/ichebyfft scaling of chebyshev.cpp:262-303, makeState).  Oracle:
``make_physical`` / ``make_spectral`` (numpy/scipy FFTs and DCT-I) on the same fields.  FP64 throughout:
relative max-norm differences within 1e-13.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-13

# radices 2, 3, 4, 5 and prime factors 7, 11, 13 (direct-DFT stages)
GRIDS = [(32, 33, 32), (48, 49, 36), (24, 17, 40), (128, 97, 128), (10, 9, 6), (28, 17, 22), (14, 9, 26)]


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def random_spectral(g, Nd, rng, hermitian=True):
    """Spectral coefficients of a real field (random physical values transformed by the oracle), or raw
    random complex data (every mode, Nyquist included)."""
    if hermitian:
        p = rng.standard_normal((Nd, g.Ny, g.Nx, g.Nz))
        return O.make_spectral(p, g)
    return rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz)) + 1j * rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz))


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("grid", GRIDS, ids=["%dx%dx%d" % g for g in GRIDS])
def test_make_physical_matches_oracle(grid):
    from channelflow_gb300.flowfield import FlowField, Physical
    g = O.Grid(*grid, 2.0, 1.0)
    rng = np.random.default_rng(sum(grid))
    for hermitian in (True, False):
        u = random_spectral(g, 3, rng, hermitian)
        f = FlowField(g.Nx, g.Ny, g.Nz, 3, g.Lx, g.Lz)
        f.set_spectral(u)
        f.makePhysical()
        assert f.state() == (Physical, Physical)
        assert rel(f.physical(), O.make_physical(u, g)) <= TOL


@pytest.mark.parametrize("grid", GRIDS, ids=["%dx%dx%d" % g for g in GRIDS])
def test_make_spectral_matches_oracle(grid):
    from channelflow_gb300.flowfield import FlowField, Spectral
    g = O.Grid(*grid, 2.0, 1.0)
    rng = np.random.default_rng(7 + sum(grid))
    p = rng.standard_normal((1, g.Ny, g.Nx, g.Nz))
    f = FlowField(g.Nx, g.Ny, g.Nz, 1, g.Lx, g.Lz)
    f.set_physical(p)
    f.makeSpectral()
    assert f.state() == (Spectral, Spectral)
    assert rel(f.spectral(), O.make_spectral(p, g)) <= TOL
    # and back
    f.makePhysical()
    assert rel(f.physical(), p) <= TOL


def test_half_transforms_and_make_state():
    """makeSpectral_xz / makePhysical_y etc. and the mixed states of makeState."""
    from channelflow_gb300.flowfield import FlowField, Physical, Spectral
    g = O.Grid(24, 25, 30, 3.0, 2.0)
    rng = np.random.default_rng(3)
    p = rng.standard_normal((3, g.Ny, g.Nx, g.Nz))
    f = FlowField(g.Nx, g.Ny, g.Nz, 3, g.Lx, g.Lz)
    f.set_physical(p)
    f.makeSpectral_xz()  # (Spectral, Physical): xz FFT only
    assert f.state() == (Spectral, Physical)
    xz = np.fft.rfft2(p, axes=(2, 3)) / (g.Nx * g.Nz)
    assert rel(f.spectral(), xz) <= TOL
    f.makeSpectral_y()
    assert rel(f.spectral(), O.chebyfft(xz, axis=1)) <= TOL
    f.makeState(Spectral, Physical)  # y back to physical: the xz coefficients again
    assert f.state() == (Spectral, Physical)
    assert rel(f.spectral(), xz) <= TOL
    f.makeState(Physical, Spectral)  # spectral_y then physical_xz
    assert f.state() == (Physical, Spectral)
    assert rel(f.physical(), O.chebyfft(p, axis=1)) <= TOL
    f.makeSpectral_xz()
    f.makeSpectral_xz()  # no-op in the current state
    f.makePhysical()
    assert f.state() == (Physical, Physical)
    assert rel(f.physical(), p) <= TOL


def test_transforms_match_dns_field_layout():
    """A DNS velocity field from the seeded generator: its physical values on the GPU equal the oracle's,
    and the field is real (the spectral round trip is the identity)."""
    from channelflow_gb300.fields import random_divfree_field
    from channelflow_gb300.flowfield import FlowField
    g = O.Grid(32, 33, 32, 2.0, 1.0)
    u = random_divfree_field(g.Nx, g.Ny, g.Nz, g.Lx, g.Lz, seed=4, norm=0.2)
    f = FlowField(g.Nx, g.Ny, g.Nz, 3, g.Lx, g.Lz)
    f.set_spectral(u)
    f.makePhysical()
    assert rel(f.physical(), O.make_physical(u, g)) <= TOL
    f.makeSpectral()
    assert np.abs(f.spectral() - u).max() <= 1e-14 * np.abs(u).max()


def test_bad_sizes_rejected():
    from channelflow_gb300 import _lib as L
    from channelflow_gb300.flowfield import FlowField
    with pytest.raises(L.CfgpuError):
        FlowField(262, 9, 8, 1, 1.0, 1.0)  # 262 = 2 x 131: a prime factor above the largest radix (127)
    with pytest.raises(L.CfgpuError):
        FlowField(9, 9, 8, 1, 1.0, 1.0)  # odd Nx
