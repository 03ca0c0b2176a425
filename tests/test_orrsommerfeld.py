"""Orr-Sommerfeld eigenfunction growth (the reference's tests/dnsOrrsommTest.cpp).

Plane Poiseuille flow at Re = 7500 on a 4 x 65 x 4 grid (Lx = 2 pi, Lz = pi)
carries the least stable Orr-Sommerfeld mode (kx = 1) at amplitude 1e-4 of
the base flow.  The DNS (rotational form, no dealiasing, bulk-velocity
constraint, SBDF3 started with CNRK2, dt = 0.02) must follow the analytic
solution exp(-i omega t) times the eigenfunction: the sum over t = 0, 1, ..., 13
of L2Dist(u, u_lin) + L2Dist(p, p_lin) stays below the reference's bound for
the scheme (dnsOrrsommTest.cpp:90-113, 269-337).  The reference registers no
run of this program (its variants are commented out in tests/CMakeLists.txt),
and its no-argument bound of 1e-7 (dnsOrrsommTest.cpp:40) is not met by this
restatement: the sum is 1.084e-7, independent of dt (1.0844e-7 at dt = 0.01
as well), i.e. it is the nonlinear self-interaction of the 1e-4 mode, not
time-stepping error.  The per-scheme bounds given with an explicit scheme
flag (2e-6 for --sbdf3) are used here.

The initial q comes from the physically consistent form of DNS::up2q: the
reference's up2q adds U's Chebyshev coefficients instead of U(y), for w as
well (dns.cpp:421-434), which corrupts q, its (0,0) mode at O(1).  The SBDF schemes
never read q and pass either way; CNRK2 and CNAB2 (started with CNRK2) read
q in their linear term and, from the reference's q, miss their bounds by six
orders of magnitude (sum 5.65), from the consistent q pass them.  The eigenfunctions and omega are the
reference's fixtures (tests/data/os_ueig10_65.asc, os_peig10_65.asc,
os_omega10_65.cmplx) copied into tests/golden/orrsommerfeld.npz.

The oracle run pins the oracle to that physics check; the GPU run goes
through the C ABI (FP64 path) and is compared with both the analytic solution
and the oracle's final fields.
"""

import math
import os

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import to_cflags, to_cgrid

GOLD = os.path.join(os.path.dirname(__file__), "golden", "orrsommerfeld.npz")
# per-scheme bounds of dnsOrrsommTest.cpp:90-113
MAXERR = {O.CNFE1: 2e-2, O.CNAB2: 4e-5, O.CNRK2: 5e-6, O.SMRK2: 8e-6, O.SBDF2: 2e-4, O.SBDF3: 2e-6,
          O.SBDF4: 2e-6}
ORACLE_ERR_SBDF3 = 1.0844443029260426e-07   # the oracle's sum for the SBDF3 / parabola-base case
NOUT, DT, T1 = 50, 0.02, 13.0


MAXERR_LINU = 1e-9   # dnsOrrsommTest.cpp:144-145: LinearAboutProfile follows the linear solution


def os_case(baseflow=True, timestepping=O.SBDF3, constraint=O.BulkVelocity, nonlinearity=O.Rotational):
    d = np.load(GOLD)
    g = O.Grid(4, 65, 4, 2 * math.pi, math.pi, -1.0, 1.0)
    nu = 1.0 / 7500.0
    fl = O.DNSFlags(nu=nu, dt=DT, baseflow=O.ZeroBase, dealiasing=O.NoDealiasing, nonlinearity=nonlinearity,
                    constraint=constraint, timestepping=timestepping, initstepping=O.CNRK2,
                    ulowerwall=0.0, uupperwall=0.0, dPdx=-2.0 * nu, Ubulk=2.0 / 3.0)
    y = O.chebypoints(g.Ny, g.a, g.b)
    parabola = O.chebyfft(1.0 - y ** 2)
    # amplitude: perturbation / parabola = 1e-4 in L2 (dnsOrrsommTest.cpp:186-206)
    utmp = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
    utmp[0, :, 0, 0] = parabola
    ueig0 = O.basisfunc_field(d["ueig"], 1, 0, g)
    c = 1e-4 * O.L2Norm(utmp, g) / O.L2Norm(ueig0, g)
    lam = -1j * complex(d["omega"])
    ueig_prof, peig_prof = c * d["ueig"], c * d["peig"]
    if baseflow:
        fl.baseflow = O.ArbitraryBase
        base = (parabola, np.zeros(g.Ny))
    else:
        base = (np.zeros(g.Ny), np.zeros(g.Ny))

    def lin(t):
        ul = O.basisfunc_field(ueig_prof * np.exp(lam * t), 1, 0, g)
        pl = O.basisfunc_field(peig_prof * np.exp(lam * t), 1, 0, g)
        if not baseflow:
            ul[0, :, 0, 0] += parabola
        return ul, pl

    return g, fl, base, lin


def run_os(g, fl, base, lin, make_dns):
    """The reference test's loop: check at t = 0, 1, ..., 13, then advance 50 steps."""
    un, pn = lin(0.0)
    Ub, Wb = base
    qn = O.up2q(un, pn, g, Ub, Wb, fl.nonlinearity, as_reference=False)
    advance = make_dns(un, qn)
    err = 0.0
    t, k = 0.0, 0
    while t <= T1:
        ul, pl = lin(k * NOUT * DT)
        err += O.L2Dist(un, ul, g) + O.L2Dist(pn, pl, g)
        assert O.L2Norm(un, g) <= 1
        un, qn = advance(un, qn, NOUT)
        pn = O.uq2p(un, qn, g, Ub, Wb, fl.nonlinearity)
        t += NOUT * DT
        k += 1
    return err, un, qn


def oracle_dns(g, fl, base):
    b = base if fl.baseflow == O.ArbitraryBase else None

    def make(u0, q0):
        dns = O.DNS(u0.copy(), q0.copy(), g, fl, base=b)
        return lambda u, q, n: dns.advance(u, q, n)

    return make


def test_oracle_orrsommerfeld_growth():
    g, fl, base, lin = os_case()
    err, _, _ = run_os(g, fl, base, lin, oracle_dns(g, fl, base))
    assert err < MAXERR[O.SBDF3], err
    assert abs(err - ORACLE_ERR_SBDF3) <= 1e-6 * ORACLE_ERR_SBDF3


def test_reference_up2q_offsets_mean_mode():
    """The reference's up2q moves q's (0,0) mode by O(1) (|U|^2 profile) and the kx = 1 mode by O(u U)."""
    g, fl, base, lin = os_case()
    un, pn = lin(0.0)
    qa = O.up2q(un, pn, g, *base, fl.nonlinearity, as_reference=True)
    qb = O.up2q(un, pn, g, *base, fl.nonlinearity, as_reference=False)
    d = np.abs(qa - qb)
    assert d[0, :, 0, 0].max() > 1e-2
    assert 1e-7 < d[0, :, 1, 0].max() < 1e-3


def test_oracle_orrsommerfeld_linearized():
    """LinearAboutProfile about the parabola (the reference's --linU case): the DNS is the linear problem."""
    g, fl, base, lin = os_case(nonlinearity=O.LinearAboutProfile)
    err, _, _ = run_os(g, fl, base, lin, oracle_dns(g, fl, base))
    assert err < MAXERR_LINU, err


GPU_CASES = [(O.SBDF3, True, True), (O.SBDF3, False, True), (O.SBDF2, True, False), (O.SBDF4, True, False),
             (O.CNAB2, True, False), (O.SMRK2, True, False), (O.CNRK2, True, False), (O.CNFE1, True, False),
             ("linU", True, True)]


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,baseflow,vs_oracle", GPU_CASES,
                         ids=["sbdf3_parabola_base", "sbdf3_zero_base", "sbdf2", "sbdf4", "cnab2", "smrk2", "cnrk2",
                              "cnfe1", "sbdf3_linearized"])
def test_gpu_orrsommerfeld_growth(scheme, baseflow, vs_oracle):
    from channelflow_gb300 import DNS, build
    build.build()
    if scheme == "linU":
        g, fl, base, lin = os_case(baseflow=baseflow, nonlinearity=O.LinearAboutProfile)
        maxerr = MAXERR_LINU
    else:
        g, fl, base, lin = os_case(baseflow=baseflow, timestepping=scheme)
        maxerr = MAXERR[scheme]
    handles = []

    def make_gpu(u0, q0):
        b = base if fl.baseflow == O.ArbitraryBase else None
        dns = DNS(np.ascontiguousarray(u0), to_cgrid(g), to_cflags(fl), base=b, precision="fp64")
        handles.append(dns)

        def adv(u, q, n):
            u, q = np.ascontiguousarray(u.copy()), np.ascontiguousarray(q.copy())
            dns.advance(u, q, n)
            return u, q
        return adv

    err, un, qn = run_os(g, fl, base, lin, make_gpu)
    assert err < maxerr, err
    if not vs_oracle:
        return
    err_r, ur, qr = run_os(g, fl, base, lin, oracle_dns(g, fl, base))
    assert abs(err - err_r) <= 1e-6 * err_r
    # u is the 1e-4 perturbation of an O(1) flow: the round-off scale is set by the total flow
    scale = max(O.L2Norm(ur, g), 1.0)
    assert O.L2Dist(un, ur, g) <= 1e-12 * scale
    assert O.L2Dist(qn, qr, g) <= 1e-12 * max(O.L2Norm(qr, g), 1.0)
