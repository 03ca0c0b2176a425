"""Shared test helpers: oracle cases and field comparisons (test infrastructure)."""

import math

import numpy as np

from oracle import cf_oracle as O

COUETTE_BOX = (2 * math.pi / 1.14, 2 * math.pi / 2.5)
POISEUILLE_BOX = (4 * math.pi, 2 * math.pi)


def solved_mask(g, dealias=True):
    kxd = g.Nx // 3 - 1 if dealias else g.Nx // 2 - 1
    kzd = g.Nz // 3 - 1 if dealias else g.Nz // 2 - 1
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    kz = np.arange(g.Mz)
    return (np.abs(kx)[:, None] <= kxd) & (kz[None, :] <= kzd)


def rel_l2(a, b, g):
    """Relative L2 distance with the reference's Chebyshev-weighted norm (diffops.cpp:353-487)."""
    return O.L2Dist(a, b, g) / max(O.L2Norm(b, g), 1e-300)


def oracle_run(u0, g, fl, nsteps, base=None, chunks=None):
    q = np.zeros((1,) + u0.shape[1:], complex)
    dns = O.DNS(u0.copy(), q, g, fl, base=base)
    u = u0.copy()
    if chunks is None:
        chunks = [nsteps]
    for n in chunks:
        u, q = dns.advance(u, q, n)
    return u, q, dns


def to_cgrid(g):
    from channelflow_gb300 import Grid
    return Grid(g.Nx, g.Ny, g.Nz, g.Lx, g.Lz, g.a, g.b)


def to_cflags(fl):
    from channelflow_gb300 import DNSFlags
    d = DNSFlags()
    for k in d.__dataclass_fields__:
        setattr(d, k, getattr(fl, k))
    return d
