"""The reference's steady-state DNS tests on the GPU, through the C ABI.

* tests/dnsZeroTest.cpp:26-103 (registered in tests/CMakeLists.txt:68-81): 8x33x8, Lx = Lz = 2 pi, Re = 400,
  laminar base with walls at rest, Ubulk = 0, dPdx = 0, dt = 0.1; for t = 0, 1, ..., 9 the distance of u from
  the exact (zero) solution is summed before each advance of 10 steps; the sum must stay under the scheme's
  bound (1e-8 by default; cnfe1 2e-2, cnab2 4e-5, cnrk2 5e-6, smrk2 8e-6, sbdf2 2e-4, sbdf3 2e-6,
  sbdf4 1e-6). A Couette variant (walls at -1 and +1, a non-zero base flow) is checked the same way.
* tests/dnsParabolaTest.cpp:50-266 (tests/CMakeLists.txt:83-110): the same grid and stepping with
  dPdx = -2 nu, Ubulk = 2/3; either the base flow is the parabola 1 - y^2 and u = 0 ("--base"), or the base
  flow is zero and u carries the parabola ("--fluc"); under the bulk-velocity or the pressure-gradient
  constraint the flow must not move: the summed distance from the initial field stays below 1e-13.
"""

import math

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu

SCHEMES = {"cnfe1": (O.CNFE1, 2e-2), "cnab2": (O.CNAB2, 4e-5), "cnrk2": (O.CNRK2, 5e-6), "smrk2": (O.SMRK2, 8e-6),
           "sbdf2": (O.SBDF2, 2e-4), "sbdf3": (O.SBDF3, 2e-6), "sbdf4": (O.SBDF4, 1e-6)}
CONSTRAINTS = {"bulkv": O.BulkVelocity, "gradp": O.PressureGradient}
PARABOLA_MAXERR = 1e-13


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def summed_distance(g, fl, u_init, base=None):
    """Sum over t = 0..9 of L2Dist(u(t), u_init), 10 steps of dt = 0.1 between samples (the tests' loop)."""
    from channelflow_gb300 import DNS
    u = np.ascontiguousarray(u_init.copy())
    q = np.zeros((1,) + u.shape[1:], complex)
    dns = DNS(u, to_cgrid(g), to_cflags(fl), base=base)
    err = 0.0
    for _ in range(10):
        err += O.L2Dist(u, u_init, g)
        dns.advance(u, q, 10)
    return err


@pytest.mark.parametrize("constraint", list(CONSTRAINTS))
@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_dns_zero_gpu(scheme, constraint):
    ts, maxerr = SCHEMES[scheme]
    g = O.Grid(8, 33, 8, 2 * math.pi, 2 * math.pi)
    fl = O.DNSFlags(nu=1.0 / 400, dt=0.1, timestepping=ts, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    constraint=CONSTRAINTS[constraint], Ubulk=0.0, dPdx=0.0)
    u0 = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    assert summed_distance(g, fl, u0) < maxerr


@pytest.mark.parametrize("constraint", list(CONSTRAINTS))
@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_dns_zero_couette_gpu(scheme, constraint):
    """Zero fluctuation on the Couette base flow (walls -1, +1) stays zero."""
    ts, maxerr = SCHEMES[scheme]
    g = O.Grid(8, 33, 8, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1.0 / 400, dt=0.1, timestepping=ts, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    constraint=CONSTRAINTS[constraint], ulowerwall=-1.0, uupperwall=1.0, Ubulk=0.0, dPdx=0.0)
    u0 = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    assert summed_distance(g, fl, u0) < min(maxerr, 1e-8)


@pytest.mark.parametrize("constraint", list(CONSTRAINTS))
@pytest.mark.parametrize("where", ["fluc", "base"])
@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_dns_parabola_gpu(scheme, where, constraint):
    ts, _ = SCHEMES[scheme]
    g = O.Grid(8, 33, 8, 2 * math.pi, 2 * math.pi)
    nu = 1.0 / 400
    fl = O.DNSFlags(nu=nu, dt=0.1, timestepping=ts, initstepping=O.SMRK2, baseflow=O.ZeroBase,
                    constraint=CONSTRAINTS[constraint], dPdx=-2.0 * nu, Ubulk=2.0 / 3.0)
    zero = np.zeros(g.Ny)
    parabola = np.zeros(g.Ny)
    parabola[0], parabola[2] = 0.5, -0.5
    on_base = where == "base"
    u0 = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    if not on_base:
        u0[0, :, 0, 0] = parabola
    err = summed_distance(g, fl, u0, base=(parabola if on_base else zero, zero))
    assert err < PARABOLA_MAXERR
