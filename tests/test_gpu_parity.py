"""GPU parity: libcfgpu.so (through its C ABI) against the oracle and the reference's golden data."""

import math
import os
import zlib

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, oracle_run, rel_l2, solved_mask, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
FP64_TOL = 1e-10     # relative L2 after the run, plain FP64 path (Chebyshev-weighted norm)
MIXED_TOL = 1e-5     # relative L2, FP32 transforms/nonlinear term + FP64 tau solves
Q_TOL = 1e-8         # pressure q, FP64 path: q solves a Neumann problem from the derivative of the RHS, one
                     # order less well conditioned than u (observed up to 1.04e-9 with rotation)


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def gpu_run(u0, g, fl, nsteps, precision="fp64", base=None, chunks=None):
    from channelflow_gb300 import DNS
    u = np.ascontiguousarray(u0.copy())
    q = np.zeros((1,) + u.shape[1:], complex)
    dns = DNS(u, to_cgrid(g), to_cflags(fl), base=base, precision=precision)
    for n in (chunks or [nsteps]):
        dns.advance(u, q, n)
    return u, q, dns


@pytest.mark.parametrize("N,cases", [(49, 10), (301, 2)])
def test_tau_batched_matches_oracle(N, cases):
    """N = 301 exceeds the shared-memory staging of the three-kernel solve and takes the one-kernel path."""
    from channelflow_gb300 import tau_solve_batched
    from tests.test_oracle_golden import tau_case
    rng = np.random.default_rng(11)
    for _ in range(cases):
        c = tau_case(rng, N=N)
        kxs = np.array([c["kx"], 0, 1, 3])
        kzs = np.array([c["kz"], 0, 0, 2])
        R = [np.stack([c[k]] * 4) for k in ("Rx", "Ry", "Rz")]
        u, v, w, P = tau_solve_batched(c["N"], kxs, kzs, c["Lx"], c["Lz"], c["a"], c["b"], c["lam_t"], c["nu"], *R)
        lam = c["lam_t"] + 4 * math.pi ** 2 * c["nu"] * ((kxs / c["Lx"]) ** 2 + (kzs / c["Lz"]) ** 2)
        ts = O.TauSolver(kxs, kzs, c["Lx"], c["Lz"], c["a"], c["b"], lam, c["nu"], c["N"])
        ou, ov, ow, oP = ts.solve(*[r.T.copy() for r in R])
        for got, ref in ((u, ou), (v, ov), (w, ow), (P, oP)):
            scale = np.abs(ref).max()
            assert np.abs(got - ref.T).max() <= 1e-12 * scale
        # the first mode reproduces the analytic solution
        assert np.abs(u[0] - c["u"]).max() < 1e-9 and np.abs(v[0] - c["v"]).max() < 1e-9


CASES = [
    # name, grid, flags kwargs, steps
    ("couette_sbdf3", (16, 17, 16, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0), 30),
    ("poiseuille_cnab2_bulk", (24, 33, 24, *POISEUILLE_BOX),
     dict(nu=1 / 4000, dt=0.01, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0), 30),
    ("couette_cnrk2_gradp", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.CNRK2, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0), 10),
    ("poiseuille_sbdf4_bulk", (12, 17, 12, *POISEUILLE_BOX),
     dict(nu=1 / 2000, dt=0.01, timestepping=O.SBDF4, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0), 12),
    ("couette_sbdf2", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0), 10),
    ("couette_cnfe1", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.CNFE1, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0), 10),
    ("couette_smrk2_nodealias", (8, 17, 8, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SMRK2, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0,
          dealiasing=O.NoDealiasing), 10),
    ("suction_sbdf1_gradp", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF1, baseflow=O.SuctionBase, Vsuck=1 / 400), 10),
    ("couette_sbdf3_convection", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Convection), 10),
    ("couette_cnab2_skew_bulk", (12, 17, 12, *POISEUILLE_BOX),
     dict(nu=1 / 2000, dt=0.01, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0, nonlinearity=O.SkewSymmetric), 10),
    ("couette_sbdf2_divergence", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Divergence), 10),
    ("couette_sbdf3_alternating", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Alternating), 11),
    ("suction_cnrk2_skew_nodealias", (8, 17, 8, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.CNRK2, baseflow=O.SuctionBase, Vsuck=1 / 400,
          nonlinearity=O.SkewSymmetric, dealiasing=O.NoDealiasing), 6),
    ("poiseuille_sbdf3_linearized_bulk", (12, 17, 12, *POISEUILLE_BOX),
     dict(nu=1 / 2000, dt=0.01, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0, nonlinearity=O.LinearAboutProfile), 10),
    ("couette_cnab2_linearized", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.LinearAboutProfile), 10),
    ("couette_sbdf3_rotation", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0, rotation=0.3), 10),
    ("poiseuille_cnrk2_rotation_skew_bulk", (12, 17, 12, *POISEUILLE_BOX),
     dict(nu=1 / 2000, dt=0.01, timestepping=O.CNRK2, baseflow=O.LaminarBase, constraint=O.BulkVelocity,
          Ubulk=2.0 / 3.0, rotation=-0.2, nonlinearity=O.SkewSymmetric), 8),
    ("suction_sbdf2_rotation", (12, 17, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF2, initstepping=O.SMRK2, baseflow=O.SuctionBase, Vsuck=1 / 400,
          rotation=0.5), 8),
    # x and z lengths with prime factors 7 and 13 (direct-DFT stages of the generic FFT)
    ("couette_sbdf3_radix7_13", (28, 17, 26, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0), 10),
    ("poiseuille_48_cnab2", (48, 49, 48, *POISEUILLE_BOX),
     dict(nu=1 / 4000, dt=0.01, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0), 5),
    # tall grids: the Chebyshev kernels' row tilings for Ny = 97 (the bench workload's Ny) and Ny = 129
    ("poiseuille_tall97_cnab2", (12, 97, 12, *POISEUILLE_BOX),
     dict(nu=1 / 4000, dt=0.01, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0), 6),
    ("couette_tall129_sbdf3", (12, 129, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.01, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0), 6),
    # taller than one block of the dense Chebyshev kernels: row blocks, curl then transform, tall CFL
    ("couette_tall161_sbdf3", (12, 161, 12, *COUETTE_BOX),
     dict(nu=1 / 400, dt=0.01, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          ulowerwall=-1.0, uupperwall=1.0), 6),
    ("poiseuille_tall257_cnab2", (12, 257, 12, *POISEUILLE_BOX),
     dict(nu=1 / 4000, dt=0.005, timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase,
          constraint=O.BulkVelocity, Ubulk=2.0 / 3.0), 6),
]


@pytest.mark.parametrize("name,grid,fk,nsteps", CASES, ids=[c[0] for c in CASES])
def test_dns_fp64_matches_oracle(name, grid, fk, nsteps):
    g = O.Grid(*grid)
    fl = O.DNSFlags(**fk)
    dealias = fl.dealiasing == O.DealiasXZ
    u0 = O.random_divfree_field(g, seed=zlib.crc32(name.encode()) % 1000, norm=0.1,
                                zero_mean_u=fl.constraint == O.BulkVelocity)
    if not dealias:
        u0[:, :, ~solved_mask(g, dealias)] = 0.0
    ou, oq, _ = oracle_run(u0, g, fl, nsteps, chunks=[nsteps // 2, nsteps - nsteps // 2])
    gu, gq, dns = gpu_run(u0, g, fl, nsteps, chunks=[nsteps // 2, nsteps - nsteps // 2])
    m = solved_mask(g, dealias)
    ou[:, :, ~m] = 0
    oq[:, :, ~m] = 0
    assert rel_l2(gu, ou, g) <= FP64_TOL
    assert rel_l2(gq, oq, g) <= Q_TOL
    assert abs(dns.time() - (fl.t0 + nsteps * fl.dt)) < 1e-12


def test_time_integration_golden_gpu():
    """The reference's golden regression on the GPU: uinit -> 440 SBDF3 steps -> ufinal."""
    z = np.load(os.path.join(GOLD, "timeintegration.npz"))
    g = O.Grid(int(z["uinit_Nx"]), int(z["uinit_Ny"]), int(z["uinit_Nz"]), float(z["uinit_Lx"]),
               float(z["uinit_Lz"]), float(z["uinit_a"]), float(z["uinit_b"]))
    u0 = O.load_io_field(z["uinit"], g.Nx, g.Nz)
    uf = O.load_io_field(z["ufinal"], g.Nx, g.Nz)
    fl = O.DNSFlags(baseflow=O.SuctionBase, timestepping=O.SBDF3, initstepping=O.SMRK2, dt=1.0 / 40,
                    nu=1.0 / 400, Vsuck=1.0 / 400)
    gu, _, _ = gpu_run(u0, g, fl, 440, chunks=[40] * 11)
    m = solved_mask(g)
    uf[:, :, ~m] = 0
    gu[:, :, ~m] = 0
    assert O.L2Dist(gu, uf, g) <= 1e-13


def test_dns_mixed_matches_oracle():
    g = O.Grid(32, 33, 32, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    ulowerwall=-1.0, uupperwall=1.0)
    u0 = O.random_divfree_field(g, seed=5, norm=0.1)
    ou, _, _ = oracle_run(u0, g, fl, 50)
    gu, _, _ = gpu_run(u0, g, fl, 50, precision="mixed")
    ou[:, :, ~solved_mask(g)] = 0
    assert rel_l2(gu, ou, g) <= MIXED_TOL


@pytest.mark.parametrize("ny", [97, 129, 161, 257])
def test_dns_mixed_tall_grids(ny):
    """Mixed path with the compensated forward Chebyshev sums at Ny = 97 and 129 (7 and 9 rows per warp)."""
    g = O.Grid(12, ny, 12, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.01, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    ulowerwall=-1.0, uupperwall=1.0)
    u0 = O.random_divfree_field(g, seed=ny, norm=0.1)
    ou, _, _ = oracle_run(u0, g, fl, 20)
    gu, _, _ = gpu_run(u0, g, fl, 20, precision="mixed")
    ou[:, :, ~solved_mask(g)] = 0
    assert rel_l2(gu, ou, g) <= MIXED_TOL


@pytest.mark.parametrize("nl", [O.Convection, O.SkewSymmetric, O.Divergence])
def test_dns_mixed_gradient_forms(nl):
    g = O.Grid(24, 25, 24, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase,
                    ulowerwall=-1.0, uupperwall=1.0, nonlinearity=nl)
    u0 = O.random_divfree_field(g, seed=7, norm=0.1)
    ou, _, _ = oracle_run(u0, g, fl, 20)
    gu, _, _ = gpu_run(u0, g, fl, 20, precision="mixed")
    ou[:, :, ~solved_mask(g)] = 0
    assert rel_l2(gu, ou, g) <= MIXED_TOL


def test_resident_path_equals_host_path():
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u0 = O.random_divfree_field(g, seed=3, norm=0.1)
    a, _, _ = gpu_run(u0, g, fl, 12)
    from channelflow_gb300 import DNS
    u = u0.copy()
    q = np.zeros((1,) + u.shape[1:], complex)
    dns = DNS(u, to_cgrid(g), to_cflags(fl))
    dns.set_fields(u, q)
    dns.advance_resident(12)
    dns.get_fields(u, q)
    assert np.array_equal(u, a)


@pytest.mark.parametrize("ny", [33, 161])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_cfl_and_l2norm_match_oracle(precision, tol, ny):
    g = O.Grid(24, ny, 24, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u0 = O.random_divfree_field(g, seed=21, norm=0.2)
    gu, gq, dns = gpu_run(u0, g, fl, 3, precision=precision)
    nse = O.NSE(g, fl)
    ref = O.cfl_factor(gu, g, nse.Ubase, nse.Wbase) * (2 * math.pi / 3 * fl.dt)
    assert abs(dns.CFL() - ref) <= tol * ref
    assert abs(dns.l2norm(0) - O.L2Norm(gu, g)) <= 1e-12 * O.L2Norm(gu, g)
    assert abs(dns.l2norm(1) - O.L2Norm(gq, g)) <= 1e-12 * max(O.L2Norm(gq, g), 1e-300)
