"""FieldSymmetry on spectral fields and DNS::advance's symmetry projection.

sigma (u,v,w)(x,y,z) = s (sx u, sy v, sz w)(sx x + ax Lx, sy y, sz z + az Lz)
(channelflow/symmetry.h); FlowField::operator*= and project
(channelflow/flowfield.cpp:1095-1272); DNS::advance projects the velocity and
the scheme's stored fields when (int)t % symmetryprojectioninterval == 0
(channelflow/dns.cpp:151-155).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, oracle_run, rel_l2, to_cflags, to_cgrid

SHIFT_REFLECT = (1, 1, 1, -1, 0.5, 0.0)   # (s, sx, sy, sz, ax, az): the shift-reflect of plane Couette searches
SYMS = [SHIFT_REFLECT, (1, 1, 1, 1, 0.5, 0.25), (1, -1, 1, 1, 0.3, 0.0), (1, -1, -1, -1, 0.0, 0.0),
        (-1, 1, -1, 1, 0.25, 0.5), (1, -1, 1, -1, 0.5, 0.5)]


def test_oracle_symmetry_algebra():
    """Involutions square to the identity; projection is idempotent and its image is sigma-invariant."""
    g = O.Grid(12, 9, 12, *COUETTE_BOX)
    u = O.random_divfree_field(g, seed=3, norm=0.2)
    for sym in (SHIFT_REFLECT, (1, -1, -1, -1, 0.0, 0.0), (1, -1, 1, 1, 0.5, 0.0)):
        assert np.abs(O.apply_symmetry(O.apply_symmetry(u, g, sym), g, sym) - u).max() < 1e-14
        p = O.apply_symmetry(u, g, sym, project=True)
        assert np.abs(O.apply_symmetry(p, g, sym, project=True) - p).max() < 1e-14
        assert np.abs(O.apply_symmetry(p, g, sym) - p).max() < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("project", [False, True])
@pytest.mark.parametrize("dealias", [True, False])
def test_field_symmetry_matches_oracle(project, dealias):
    from channelflow_gb300 import build
    from channelflow_gb300.symmetry import FieldSymmetry, apply
    build.build()
    g = O.Grid(12, 9, 18, *COUETTE_BOX)
    rng = np.random.default_rng(2)
    for Nd in (3, 1):
        u = rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz)) + 1j * rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz))
        for sym in SYMS:
            s, sx, sy, sz, ax, az = sym
            got = apply(u, to_cgrid(g), FieldSymmetry(sx, sy, sz, ax, az, s), project=project, dealias=dealias)
            ref = O.apply_symmetry(u, g, sym, project=project, dealias=dealias)
            assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max(), sym


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [O.SBDF3, O.CNAB2])
def test_dns_symmetry_projection_matches_oracle(scheme):
    from channelflow_gb300 import DNS, build
    from channelflow_gb300.symmetry import FieldSymmetry, set_symmetries
    build.build()
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0,
                    timestepping=scheme)
    u0 = O.random_divfree_field(g, seed=12, norm=0.2)       # not symmetric: the first projection changes it
    chunks = [3, 4, 5, 6]
    q = np.zeros((1,) + u0.shape[1:], complex)
    ref = O.DNS(u0.copy(), q, g, fl)
    ref.symmetries = (SHIFT_REFLECT,)
    ref.symmetry_interval = 1
    ur, qr = u0.copy(), q.copy()
    for n in chunks:
        ur, qr = ref.advance(ur, qr, n)
    d = DNS(np.ascontiguousarray(u0), to_cgrid(g), to_cflags(fl))
    s, sx, sy, sz, ax, az = SHIFT_REFLECT
    set_symmetries(d, [FieldSymmetry(sx, sy, sz, ax, az, s)], interval=1)
    u, qq = np.ascontiguousarray(u0.copy()), q.copy()
    for n in chunks:
        d.advance(u, qq, n)
    assert rel_l2(u, ur, g) <= 1e-10


@pytest.mark.gpu
def test_symmetric_subspace_is_invariant():
    """Plane Couette commutes with the shift-reflect: a projected field stays symmetric without projection."""
    from channelflow_gb300 import DNS, build
    from channelflow_gb300.symmetry import FieldSymmetry, apply, apply_resident
    build.build()
    g = O.Grid(24, 33, 24, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    s, sx, sy, sz, ax, az = SHIFT_REFLECT
    sig = FieldSymmetry(sx, sy, sz, ax, az, s)
    u = apply(O.random_divfree_field(g, seed=31, norm=0.2), to_cgrid(g), sig, project=True)
    q = np.zeros((1,) + u.shape[1:], complex)
    d = DNS(u, to_cgrid(g), to_cflags(fl))
    d.advance(u, q, 40)
    su = apply(u, to_cgrid(g), sig)
    assert O.L2Dist(su, u, g) <= 1e-12 * O.L2Norm(u, g)
    # the resident-field form gives the same image
    d.set_fields(u, q)
    apply_resident(d, sig)
    out, qo = np.zeros_like(u), np.zeros_like(q)
    d.get_fields(out, qo)
    assert np.abs(out - su).max() <= 1e-14 * np.abs(su).max()
