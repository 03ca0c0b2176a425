"""field2vector / vector2field (channelflow/flowfield.cpp:4448-4760): the oracle's restatement pinned by its
defining properties, and the GPU kernels against the oracle.

The vector holds the independent reals of a divergence-free no-slip field; vector2field rebuilds the rest
from the wall conditions and continuity.  Properties: field -> vector -> field reproduces a div-free
no-slip field; vector -> field -> vector is the identity; every vector2field result is div-free and
vanishes at the walls; the size equals the reference's original closed form
4 (Kx + 2 Kx Kz + Kz)(Ny - 3) + 2 (Ny - 2) (flowfield.cpp:4453-4455).
GPU tolerances: field2vector is a gather (bit-exact); vector2field 1e-13 relative.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, to_cflags, to_cgrid

GRIDS = [(12, 13, 18, COUETTE_BOX), (18, 17, 12, POISEUILLE_BOX), (24, 9, 24, COUETTE_BOX)]


def _divergence(u, g):
    """max |i kx u + dv/dy + i kz w| over the modes (Chebyshev coefficients)."""
    L = g.b - g.a
    worst = 0.0
    for mx in range(g.Nx):
        kx = g.kx(mx)
        for kz in range(g.Mz):
            d = 1j * 2 * np.pi * kx / g.Lx * u[0, :, mx, kz] + 1j * 2 * np.pi * kz / g.Lz * u[2, :, mx, kz]
            d = d + (O.cdiff(u[1, :, mx, kz].real, L) + 1j * O.cdiff(u[1, :, mx, kz].imag, L))
            worst = max(worst, np.abs(d).max())
    return worst


@pytest.mark.parametrize("dims", GRIDS, ids=["12x13x18", "18x17x12", "24x9x24"])
def test_oracle_field_vector_properties(dims):
    g = O.Grid(dims[0], dims[1], dims[2], *dims[3])
    Kx, Kz = g.Nx // 3 - 1, g.Nz // 3 - 1
    assert O.field2vector_size(g) == 4 * (Kx + 2 * Kx * Kz + Kz) * (g.Ny - 3) + 2 * (g.Ny - 2)
    u = O.random_divfree_field(g, seed=sum(dims[:3]), norm=0.3)
    v = O.field2vector(u, g)
    assert v.shape == (O.field2vector_size(g),)
    assert np.abs(O.vector2field(v, g) - u).max() <= 1e-13 * np.abs(u).max()
    r = np.random.default_rng(7).standard_normal(v.shape[0])
    ur = O.vector2field(r, g)
    assert np.array_equal(O.field2vector(ur, g), r)
    assert _divergence(ur, g) <= 1e-12 * np.abs(ur).max() * g.Nx
    uy = np.moveaxis(ur, 1, 0)                     # Chebyshev index first
    walls = np.concatenate([O.eval_a(uy).ravel(), O.eval_b(uy).ravel()])
    assert np.abs(walls).max() <= 1e-12 * np.abs(ur).max()


@pytest.mark.gpu
@pytest.mark.parametrize("dims", GRIDS, ids=["12x13x18", "18x17x12", "24x9x24"])
def test_gpu_field_vector_matches_oracle(dims):
    from channelflow_gb300 import build
    from channelflow_gb300.dsi import field2vector, field2vector_size, vector2field
    build.build()
    g = O.Grid(dims[0], dims[1], dims[2], *dims[3])
    cg = to_cgrid(g)
    assert field2vector_size(cg) == O.field2vector_size(g)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=11, norm=0.3))
    assert np.array_equal(field2vector(u, cg), O.field2vector(u, g))
    r = np.random.default_rng(3).standard_normal(O.field2vector_size(g))
    got, ref = vector2field(r, cg), O.vector2field(r, g)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_field_vector_on_resident_slots():
    """The ensemble forms act on the GPU-resident field of a slot and agree with the standalone forms."""
    from channelflow_gb300 import Ensemble, build
    from channelflow_gb300.dsi import field2vector, vector2field
    build.build()
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    cg = to_cgrid(g)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    us = [np.ascontiguousarray(O.random_divfree_field(g, seed=20 + k, norm=0.2)) for k in range(3)]
    ens = Ensemble(cg, to_cflags(fl), 3)
    q = np.zeros((1,) + us[0].shape[1:], complex)
    for k in range(3):
        ens.set_field(k, us[k], q)
    for k in range(3):
        assert np.array_equal(ens.field2vector(k), field2vector(us[k], cg))
    r = np.random.default_rng(5).standard_normal(O.field2vector_size(g))
    ens.vector2field(r, 1)
    out, qo = np.zeros_like(us[0]), np.zeros_like(q)
    ens.get_field(1, out, qo)
    assert np.abs(out - vector2field(r, cg)).max() <= 1e-15 * np.abs(out).max()
    ens.get_field(2, out, qo)                      # other slots untouched
    m = np.abs(out) > 0
    assert np.array_equal(out[m], us[2][m])
    ens.close()
