"""The oracle against the reference's own golden data and self-checks (CPU only)."""

import math
import os

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, oracle_run

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_time_integration_golden():
    """tests/timeIntegrationTest.cpp: uinit -> 11 x 40 SBDF3 steps (SuctionBase) -> ufinal, L2Dist <= 1e-13."""
    z = np.load(os.path.join(GOLD, "timeintegration.npz"))
    g = O.Grid(int(z["uinit_Nx"]), int(z["uinit_Ny"]), int(z["uinit_Nz"]), float(z["uinit_Lx"]),
               float(z["uinit_Lz"]), float(z["uinit_a"]), float(z["uinit_b"]))
    u = O.load_io_field(z["uinit"], g.Nx, g.Nz)
    uf = O.load_io_field(z["ufinal"], g.Nx, g.Nz)
    fl = O.DNSFlags(baseflow=O.SuctionBase, timestepping=O.SBDF3, initstepping=O.SMRK2, nonlinearity=O.Rotational,
                    dealiasing=O.DealiasXZ, constraint=O.PressureGradient, dPdx=0.0, dt=1.0 / 40, nu=1.0 / 400,
                    Vsuck=1.0 / 400)
    u, q, _ = oracle_run(u, g, fl, 440, chunks=[40] * 11)
    assert O.L2Dist(u, uf, g) <= 1e-13


def _random_profile(N, kx, kz, Lx, Lz, a, b, rng):
    """Divergence-free (u,v,w) with u=v=w=v'=0 at both walls, and a random P (Chebyshev coefficients)."""
    y = O.chebypoints(N)  # on [-1,1]: coefficients do not depend on [a,b]
    w1 = 1 - y * y
    dec = 0.5 ** np.arange(N)
    gco = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) * dec
    gco[N - 4:] = 0
    hco = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) * dec
    hco[N - 2:] = 0
    v = O.chebyfft(w1 * w1 * O.ichebyfft(gco))
    eta = O.chebyfft(w1 * O.ichebyfft(hco))
    L = b - a
    vy = O.cdiff(v, L)
    al, ga = 2 * math.pi * kx / Lx, 2 * math.pi * kz / Lz
    k2 = al * al + ga * ga
    u = (al * (1j * vy) + ga * (-1j * eta)) / k2
    w = (ga * (1j * vy) - al * (-1j * eta)) / k2
    P = (rng.standard_normal(N) + 1j * rng.standard_normal(N)) * dec
    return u, v, w, P


def tau_case(rng, N=49):
    Lx = 2 * math.pi * (1 + rng.random())
    Lz = 2 * math.pi * (1 + rng.random())
    a = 1.0 + 0.1 * rng.random()
    b = a + (2 + rng.random())
    kx, kz = int(rng.integers(0, 32)), int(rng.integers(0, 32))
    if kx == 0 and kz == 0:
        kx = 1
    nu, dt = 1.0 / 1000.0, 0.02
    lam_t = 2.0 / dt
    lam = lam_t + 4 * math.pi ** 2 * nu * ((kx / Lx) ** 2 + (kz / Lz) ** 2)
    u, v, w, P = _random_profile(N, kx, kz, Lx, Lz, a, b, rng)
    L = b - a
    d2 = lambda f: O.cdiff2(f, L)
    Rx = lam * u - nu * d2(u) + 1j * (2 * math.pi * kx / Lx) * P
    Ry = lam * v - nu * d2(v) + O.cdiff(P, L)
    Rz = lam * w - nu * d2(w) + 1j * (2 * math.pi * kz / Lz) * P
    return dict(N=N, kx=kx, kz=kz, Lx=Lx, Lz=Lz, a=a, b=b, nu=nu, lam_t=lam_t, lam=lam, u=u, v=v, w=w, P=P,
                Rx=Rx, Ry=Ry, Rz=Rz)


def test_tausolver_random_cases():
    """tests/tausolverTest.cpp: 100 random modes/geometries, N=49; the solve reproduces the analytic
    divergence-free solution and its residual is below 1e-9."""
    rng = np.random.default_rng(2024)
    for _ in range(100):
        c = tau_case(rng)
        ts = O.TauSolver([c["kx"]], [c["kz"]], c["Lx"], c["Lz"], c["a"], c["b"], [c["lam"]], c["nu"], c["N"])
        col = lambda x: x[:, None]
        u, v, w, P = ts.solve(col(c["Rx"]), col(c["Ry"]), col(c["Rz"]))
        err = ts.verify(u, v, w, P, col(c["Rx"]), col(c["Ry"]), col(c["Rz"]))[0]
        assert err < 1e-9
        for got, ref in ((u, c["u"]), (v, c["v"]), (w, c["w"])):
            assert np.abs(got[:, 0] - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max())


def test_laminar_profiles():
    """tests/laminarTest.cpp: laminar profiles satisfy their BCs and constraint."""
    rng = np.random.default_rng(7)
    for _ in range(40):
        Ny = 65
        nu = 1.0 / (100 + 1000 * rng.random())
        ua, ub = rng.standard_normal(2)
        Vs = 0.0 if rng.random() < 0.5 else 0.01 * rng.random()
        Ubulk = rng.random()
        c = O.BulkVelocity if rng.random() < 0.5 else O.PressureGradient
        dPdx = -rng.random() * 1e-3
        U = O.laminarProfile(nu, c, dPdx, Ubulk, Vs, -1.0, 1.0, ua, ub, Ny)
        assert abs(O.eval_a(U) - ua) < 1e-10 and abs(O.eval_b(U) - ub) < 1e-10
        if c == O.BulkVelocity:
            assert abs(O.cmean(U) - Ubulk) < 1e-10
        else:
            # nu U'' + Vsuck U' = dPdx (suction enters as v = -Vsuck)
            res = nu * O.cdiff2(U, 2.0) + Vs * O.cdiff(U, 2.0)
            res[0] -= dPdx
            assert np.abs(res[: Ny - 2]).max() < 1e-8


@pytest.mark.parametrize("ts", [O.CNFE1, O.SBDF1, O.SBDF2, O.SBDF3, O.SBDF4, O.CNAB2, O.SMRK2, O.CNRK2])
@pytest.mark.parametrize("constraint", [O.PressureGradient, O.BulkVelocity])
def test_dns_zero(ts, constraint):
    """tests/dnsZeroTest.cpp: laminar base flow with zero fluctuation stays (numerically) zero."""
    g = O.Grid(8, 33, 8, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1.0 / 400, dt=0.1, timestepping=ts, initstepping=O.SMRK2, constraint=constraint,
                    baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, Ubulk=0.0, dPdx=0.0)
    u = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    u, q, _ = oracle_run(u, g, fl, 20)
    assert O.L2Norm(u, g) < 1e-8


@pytest.mark.parametrize("ts,where,constraint", [
    (O.CNFE1, "fluc", O.BulkVelocity), (O.CNAB2, "base", O.PressureGradient), (O.CNRK2, "fluc", O.PressureGradient),
    (O.SMRK2, "base", O.BulkVelocity), (O.SBDF2, "fluc", O.BulkVelocity), (O.SBDF3, "fluc", O.PressureGradient),
    (O.SBDF4, "base", O.BulkVelocity)])
def test_dns_parabola(ts, where, constraint):
    """tests/dnsParabolaTest.cpp:50-266: the parabola 1 - y^2, carried by the base flow ("base") or by u
    ("fluc"), is a steady state under dPdx = -2 nu or Ubulk = 2/3; the distance from it, summed over
    t = 0..9 (10 steps of dt = 0.1 between samples), stays below 1e-13. One case per scheme here; the GPU
    test runs all 28."""
    g = O.Grid(8, 33, 8, 2 * math.pi, 2 * math.pi)
    nu = 1.0 / 400
    fl = O.DNSFlags(nu=nu, dt=0.1, timestepping=ts, initstepping=O.SMRK2, constraint=constraint,
                    baseflow=O.ZeroBase, dPdx=-2.0 * nu, Ubulk=2.0 / 3.0)
    zero = np.zeros(g.Ny)
    parabola = np.zeros(g.Ny)
    parabola[0], parabola[2] = 0.5, -0.5
    u = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    if where == "fluc":
        u[0, :, 0, 0] = parabola
    ut = u.copy()
    q = np.zeros((1,) + u.shape[1:], complex)
    dns = O.DNS(u.copy(), q.copy(), g, fl, base=[parabola if where == "base" else zero, zero])
    err = 0.0
    for _ in range(10):
        err += O.L2Dist(u, ut, g)
        u, q = dns.advance(u, q, 10)
    assert err < 1e-13


def test_constraint_norms_of_seeded_field():
    """bc_norm / wall_slope_norm / divergence_norm vanish on the seeded initial fields and detect a violation."""
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    u = O.random_divfree_field(g, seed=3, norm=0.2)
    n = O.L2Norm(u, g)
    assert O.divergence_norm(u, g) < 1e-13 * n and O.bc_norm(u, g) < 1e-13 * n
    assert O.wall_slope_norm(u, g) < 1e-13 * n
    bad = u.copy()
    bad[1, 1, 1, 1] += 1e-3
    assert O.bc_norm(bad, g) > 1e-4 and O.wall_slope_norm(bad, g) > 1e-4


def test_io_grid_loader_matches_oracle():
    """The package's reader of I/O-grid physical data (the role of FlowField::readNetCDF and the padded-mode
    fill, flowfield.cpp:3605-3826) equals the oracle's on the reference's own files."""
    from channelflow_gb300.fields import io_to_spectral
    z = np.load(os.path.join(GOLD, "timeintegration.npz"))
    assert np.array_equal(io_to_spectral(z["uinit"], 48, 48), O.load_io_field(z["uinit"], 48, 48))
    e = np.load(os.path.join(GOLD, "eq.npz"))
    u = io_to_spectral(e["eq"], 24, 24)
    assert np.array_equal(u, O.load_io_field(e["eq"], 24, 24))
    g = O.Grid(24, 33, 24, float(e["eq_Lx"]), float(e["eq_Lz"]))
    assert O.divergence_norm(u, g) < 1e-13 and O.bc_norm(u, g) < 1e-13
