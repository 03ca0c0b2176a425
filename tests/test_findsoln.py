"""Newton-Krylov-hookstep search on the GPU: the travelling wave of tests/findsolnTest.cpp.

The reference's test (tests/findsolnTest.cpp:30-220, registered as `findsolnTest -eqb -xrel -T 10 -sigma
data/sigmabest.asc`) starts from its equilibrium data/eq (24x33x24 plane Couette, Re = 400, box
2 pi/1.14 x 2 pi/2.5) multiplied by 1.001, with the symmetry sigmabest (an x shift of 0.2817 Lx) also
multiplied by 1.001, searches for the relative equilibrium sigma f^T(u) = u with the x shift as an unknown,
and requires the result to be within 1e-5 of data/eq.  Here f^T runs on the GPU (FP64, SBDF3, fixed
dt = 0.02, T = 10); eq.npz holds the reference's data/eq and sigmabest (extracted by make_golden.py).
"""

import math
import os

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import to_cflags, to_cgrid

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def eq_case():
    z = np.load(os.path.join(GOLD, "eq.npz"))
    g = O.Grid(int(z["eq_Nx"]), int(z["eq_Ny"]), int(z["eq_Nz"]), float(z["eq_Lx"]), float(z["eq_Lz"]))
    u = O.load_io_field(z["eq"], g.Nx, g.Nz)
    return g, u, z["sigmabest"]


def test_travelling_wave_search_converges():
    from channelflow_gb300.cfdsi import CFDSI, NewtonSearchFlags, hookstep_search
    from channelflow_gb300.dsi import TimeStep
    from channelflow_gb300.symmetry import FieldSymmetry
    g, ueq, sb = eq_case()
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    ts = TimeStep(dt=0.02, dtmin=0.02, dtmax=0.02, dT=10.0, CFLmin=0.0, CFLmax=1.0, variable=False)
    sigma = FieldSymmetry(int(sb[1]), int(sb[2]), int(sb[3]), float(sb[4]) * 1.001, float(sb[5]), int(sb[0]))
    dsi = CFDSI(to_cgrid(g), to_cflags(fl), ts, 10.0, sigma=sigma, xrelative=True)
    x0 = dsi.make_vector(np.ascontiguousarray(ueq * 1.001))
    flags = NewtonSearchFlags(epsSearch=1e-13, Nnewton=8, epsSolver=1e-9, Nsolver=120, delta=0.01, deltaMax=0.1)
    x, Gx, info = hookstep_search(dsi, x0, flags)
    assert info["converged"], info
    assert np.linalg.norm(Gx) < 1e-13
    u, sig = dsi._split(x)
    # the solution of the discrete map (dt = 0.02) lies within the fixture's own time-discretisation error
    assert O.L2Dist(u, ueq, g) <= 1e-4 * O.L2Norm(ueq, g)
    assert abs(sig.ax - float(sb[4])) < 1e-4
