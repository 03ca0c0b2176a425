"""Parity at the benchmark configurations, through the C ABI, against the oracle.

* 128x97x128 plane Poiseuille (CNAB2 with SMRK2 start-up, dt = 0.01, bulk velocity Ubulk = 2/3, Re_c = 4000,
  Lx = 4 pi, Lz = 2 pi), from the bench's own seeded field (L2 norm 0.3): 100 steps.
* 32x33x32 plane Couette (SBDF3 with SMRK2 start-up, dt = 0.02, Re = 400, Lx = 2 pi/1.14, Lz = 2 pi/2.5),
  seeded field of L2 norm 0.1: 500 steps (T = 10).

The plain FP64 path must agree with the oracle to relative L2 <= 1e-10; the mixed path (FP32 transforms and
nonlinear term, FP64 state and solves) to the tolerances stated below. After the run the GPU fields are
divergence-free and satisfy the wall conditions (u = v = w = 0 and dv/dy = 0 at y = +-1) to round-off, in
both precisions: the FP64 tau solves impose them whatever the accuracy of the nonlinear term.
"""

import math

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, oracle_run, rel_l2, solved_mask, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10           # relative L2 vs the oracle, plain FP64 path
MIXED_TOL_POIS_100 = 1e-6  # relative L2 vs the oracle, mixed path, 128x97x128 after 100 steps (t = 1)
MIXED_TOL_COUETTE = 1e-5   # relative L2 vs the oracle, mixed path, 32x33x32 after 500 steps (T = 10)
DIV_TOL = 1e-11            # ||div u|| / ||u||
BC_TOL = 1e-12             # wall values and wall slope of v, relative to ||u||


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def poiseuille_case():
    from channelflow_gb300.fields import random_divfree_field
    g = O.Grid(128, 97, 128, *POISEUILLE_BOX)
    fl = O.DNSFlags(nu=1 / 4000, dt=0.01, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    constraint=O.BulkVelocity, Ubulk=2.0 / 3.0)
    # the bench's initial field (seed 1, rank 0)
    u0 = random_divfree_field(g.Nx, g.Ny, g.Nz, g.Lx, g.Lz, seed=1, norm=0.3, zero_mean_u=True)
    return g, fl, u0, 100


def couette_case():
    from channelflow_gb300.fields import random_divfree_field
    g = O.Grid(32, 33, 32, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    ulowerwall=-1.0, uupperwall=1.0)
    u0 = random_divfree_field(g.Nx, g.Ny, g.Nz, g.Lx, g.Lz, seed=1, norm=0.1)
    return g, fl, u0, 500


_ORACLE = {}


def oracle_result(name):
    if name not in _ORACLE:
        g, fl, u0, n = {"poiseuille": poiseuille_case, "couette": couette_case}[name]()
        ou, oq, _ = oracle_run(u0, g, fl, n)
        ou[:, :, ~solved_mask(g)] = 0
        _ORACLE[name] = (g, fl, u0, n, ou)
    return _ORACLE[name]


def gpu_run(u0, g, fl, nsteps, precision, cheb=1):
    """cheb: Chebyshev transforms of the nonlinear term as matrix products on the CUDA cores (0), the library's
    timed choice (1), or through the FFT (2)."""
    from channelflow_gb300 import DNS
    from channelflow_gb300 import _lib as L
    lib = L.load()
    u = np.ascontiguousarray(u0.copy())
    q = np.zeros((1,) + u.shape[1:], complex)
    L.check(lib.cfgpu_set_cheb_fft(cheb))
    L.check(lib.cfgpu_set_cheb_tensor(1 if cheb == 1 else 0))
    try:
        dns = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
    finally:
        L.check(lib.cfgpu_set_cheb_fft(1))
        L.check(lib.cfgpu_set_cheb_tensor(1))
    dns.advance(u, q, nsteps)
    return u, dns


def check_constraints(u, g):
    n = O.L2Norm(u, g)
    assert O.divergence_norm(u, g) <= DIV_TOL * n
    assert O.bc_norm(u, g) <= BC_TOL * n
    assert O.wall_slope_norm(u, g) <= BC_TOL * n


CHEB = pytest.mark.parametrize("cheb", [0, 2], ids=["matrix", "fft"])


@CHEB
@pytest.mark.parametrize("name", ["poiseuille", "couette"])
def test_config_fp64_matches_oracle(name, cheb):
    g, fl, u0, n, ou = oracle_result(name)
    gu, dns = gpu_run(u0, g, fl, n, "fp64", cheb)
    assert rel_l2(gu, ou, g) <= FP64_TOL
    assert abs(dns.time() - n * fl.dt) < 1e-12
    check_constraints(gu, g)


@CHEB
@pytest.mark.parametrize("name,tol", [("poiseuille", MIXED_TOL_POIS_100), ("couette", MIXED_TOL_COUETTE)])
def test_config_mixed_matches_oracle(name, tol, cheb):
    g, fl, u0, n, ou = oracle_result(name)
    gu, _ = gpu_run(u0, g, fl, n, "mixed", cheb)
    assert rel_l2(gu, ou, g) <= tol
    check_constraints(gu, g)


def test_config_poiseuille_bulk_velocity_held():
    """The bulk-velocity constraint holds on the GPU result: Ubulk of U(y) + u_00 stays 2/3 to round-off."""
    g, fl, u0, n, _ = oracle_result("poiseuille")
    gu, dns = gpu_run(u0, g, fl, n, "fp64")
    nse = O.NSE(g, fl)
    ubulk = O.cmean(nse.Ubase + gu[0, :, 0, 0].real)
    assert abs(ubulk - 2.0 / 3.0) < 1e-13
    assert math.isfinite(dns.dPdx())
