"""Field ensembles: many fields of one grid advanced by shared kernel launches.

Each field of an ensemble must give the same result as a single-field DNS of
that field (the per-mode and per-plane arithmetic is the same; only the
launch covers more modes and planes).  Tolerance: 1e-13 relative L2 (FP64
path) and 1e-12 (mixed path; both sides run the same FP32 kernels).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, rel_l2, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _fields(g, n, seed0, zero_mean_u=False):
    norms = np.linspace(0.05, 0.3, n)
    return [np.ascontiguousarray(O.random_divfree_field(g, seed=seed0 + k, norm=float(norms[k]),
                                                        zero_mean_u=zero_mean_u)) for k in range(n)]


CASES = [
    # grid, box, flags, fields, steps
    ("couette_sbdf3", (16, 17, 16), COUETTE_BOX,
     dict(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, timestepping=O.SBDF3,
          initstepping=O.SMRK2), 5, 12),
    ("poiseuille_cnab2_bulk", (24, 33, 24), POISEUILLE_BOX,
     dict(nu=1 / 2000, dt=0.01, baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3,
          timestepping=O.CNAB2, initstepping=O.SMRK2), 3, 8),
    ("couette_cnrk2_skew", (16, 17, 16), COUETTE_BOX,
     dict(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, timestepping=O.CNRK2,
          nonlinearity=O.SkewSymmetric), 4, 5),
]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-12)])
@pytest.mark.parametrize("name,dims,box,fkw,nf,steps", CASES, ids=[c[0] for c in CASES])
def test_ensemble_equals_single_runs(name, dims, box, fkw, nf, steps, precision, tol):
    from channelflow_gb300 import DNS, Ensemble
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(**fkw)
    us = _fields(g, nf, 40, zero_mean_u=fl.constraint == O.BulkVelocity)
    ens = Ensemble(to_cgrid(g), to_cflags(fl), nf, precision=precision)
    U = np.ascontiguousarray(np.stack(us))
    Q = np.zeros((nf, 1) + us[0].shape[1:], complex)
    ens.advance(U, Q, steps)
    cfl_e, l2_e, dp_e = ens.CFL(), ens.l2norm(0), ens.dPdx()
    for k in range(nf):
        u = us[k].copy()
        q = np.zeros((1,) + u.shape[1:], complex)
        d = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
        d.advance(u, q, steps)
        assert rel_l2(U[k], u, g) <= tol, (k, rel_l2(U[k], u, g))
        assert rel_l2(Q[k], q, g) <= tol * 10
        assert abs(cfl_e[k] - d.CFL()) <= 1e-12 * d.CFL()
        assert abs(l2_e[k] - d.l2norm(0)) <= 1e-12 * d.l2norm(0)
        assert abs(dp_e[k] - d.dPdx()) <= 1e-9 * max(abs(d.dPdx()), 1e-12)
        d.close()
    ens.close()


def test_ensemble_slots_roundtrip_and_restart():
    """set_field/get_field address one slot; a slot rewritten mid-run continues from the new field."""
    from channelflow_gb300 import DNS, Ensemble
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0,
                    timestepping=O.SMRK2)  # self-starting: no history to restart
    us = _fields(g, 4, 70)
    ens = Ensemble(to_cgrid(g), to_cflags(fl), 4)
    q0 = np.zeros((1,) + us[0].shape[1:], complex)
    for k in range(4):
        ens.set_field(k, us[k], q0)
    out = np.zeros_like(us[0])
    qo = np.zeros_like(q0)
    for k in range(4):
        ens.get_field(k, out, qo)
        m = np.abs(out) > 0
        assert np.array_equal(out[m], us[k][m])
    ens.advance_resident(6)
    new = _fields(g, 1, 99)[0]
    ens.set_field(2, new, q0)
    ens.advance_resident(6)
    ens.get_field(2, out, qo)
    u = new.copy()
    q = q0.copy()
    d = DNS(u, to_cgrid(g), to_cflags(fl))
    d.advance(u, q, 6)
    assert rel_l2(out, u, g) <= 1e-13
    ens.get_field(1, out, qo)
    u = us[1].copy()
    q = q0.copy()
    d2 = DNS(u, to_cgrid(g), to_cflags(fl))
    d2.advance(u, q, 12)
    assert rel_l2(out, u, g) <= 1e-13


def _mixed_params(g):
    """Couette and Poiseuille fields at different Reynolds numbers in one box."""
    out = []
    for k, re in enumerate([400.0, 900.0, 1500.0, 2000.0]):
        if k % 2 == 0:
            out.append(dict(nu=1 / re, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0))
        else:
            out.append(dict(nu=1 / re, baseflow=O.LaminarBase, ulowerwall=0.0, uupperwall=0.0,
                            constraint=O.BulkVelocity, Ubulk=2 / 3))
    return out


@pytest.mark.parametrize("scheme", [O.SBDF3, O.CNAB2])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-12)])
def test_heterogeneous_ensemble_equals_single_runs(scheme, precision, tol):
    from channelflow_gb300 import DNS, Ensemble
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    common = dict(dt=0.02, timestepping=scheme, initstepping=O.SMRK2)
    params = _mixed_params(g)
    ens = Ensemble(to_cgrid(g), to_cflags(O.DNSFlags(**common, **params[0])), len(params), precision=precision)
    us = []
    for k, p in enumerate(params):
        ens.set_params(k, to_cflags(O.DNSFlags(**common, **p)))
        us.append(np.ascontiguousarray(O.random_divfree_field(g, seed=200 + k, norm=0.15,
                                                              zero_mean_u=p.get("constraint") == O.BulkVelocity)))
    U = np.ascontiguousarray(np.stack(us))
    Q = np.zeros((len(params), 1) + us[0].shape[1:], complex)
    ens.advance(U, Q, 10)
    dps = ens.dPdx()
    for k, p in enumerate(params):
        fl = O.DNSFlags(**common, **p)
        u, q = us[k].copy(), np.zeros((1,) + us[k].shape[1:], complex)
        d = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
        d.advance(u, q, 10)
        assert rel_l2(U[k], u, g) <= tol, (k, rel_l2(U[k], u, g))
        assert abs(dps[k] - d.dPdx()) <= 1e-9 * max(abs(d.dPdx()), 1e-12)
        d.close()


@pytest.mark.parametrize("scheme", [O.SBDF3, O.CNAB2, O.CNRK2])
def test_load_slot_continues_a_started_request(scheme):
    """A request started alone (through its start-up steps) and moved into a running batch takes the
    same steps it would have taken alone."""
    from channelflow_gb300 import DNS, Ensemble
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    common = dict(dt=0.02, timestepping=scheme, initstepping=O.SMRK2)
    params = _mixed_params(g)[:3]
    ens = Ensemble(to_cgrid(g), to_cflags(O.DNSFlags(**common, **params[0])), 3)
    us = [np.ascontiguousarray(O.random_divfree_field(g, seed=300 + k, norm=0.1,
                                                      zero_mean_u=p.get("constraint") == O.BulkVelocity))
          for k, p in enumerate(params)]
    for k, p in enumerate(params):
        ens.set_params(k, to_cflags(O.DNSFlags(**common, **p)))
    U = np.ascontiguousarray(np.stack(us))
    Q = np.zeros((3, 1) + us[0].shape[1:], complex)
    ens.set_fields(U, Q)
    ens.advance_resident(5)
    # a new request with its own parameters: 3 steps alone, then into slot 1
    newp = dict(nu=1 / 1200, baseflow=O.LaminarBase, ulowerwall=0.0, uupperwall=0.0,
                constraint=O.BulkVelocity, Ubulk=2 / 3)
    fl = O.DNSFlags(**common, **newp)
    un = np.ascontiguousarray(O.random_divfree_field(g, seed=377, norm=0.12, zero_mean_u=True))
    qn = np.zeros((1,) + un.shape[1:], complex)
    alone = DNS(un.copy(), to_cgrid(g), to_cflags(fl))
    alone.set_fields(un, qn)
    alone.advance_resident(3)
    ens.set_params(1, to_cflags(fl))
    ens.load_slot(1, alone)
    ens.advance_resident(6)
    out, qo = np.zeros_like(un), np.zeros_like(qn)
    ens.get_field(1, out, qo)
    ref = DNS(un.copy(), to_cgrid(g), to_cflags(fl))
    u, q = un.copy(), qn.copy()
    ref.advance(u, q, 9)
    assert rel_l2(out, u, g) <= 1e-13
    # the other fields are untouched by the swap
    ens.get_field(2, out, qo)
    fl2 = O.DNSFlags(**common, **params[2])
    u, q = us[2].copy(), np.zeros_like(qn)
    d2 = DNS(u, to_cgrid(g), to_cflags(fl2))
    d2.advance(u, q, 11)
    assert rel_l2(out, u, g) <= 1e-13


@pytest.mark.parametrize("scheme", [O.SBDF3, O.CNAB2, O.CNRK2])
def test_per_field_dt_equals_single_runs(scheme):
    """Fields with their own dt (and nu) in one ensemble: each equals its single-field DNS bit for bit
    up to round-off (scheme coefficients and tables are computed as the single DNS computes them)."""
    from channelflow_gb300 import DNS, Ensemble
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    params = _mixed_params(g)
    dts = [0.02, 0.013, 0.0075, 0.016]
    ens = Ensemble(to_cgrid(g), to_cflags(O.DNSFlags(dt=0.02, timestepping=scheme, **params[0])), 4)
    us = []
    for k, p in enumerate(params):
        ens.set_params(k, to_cflags(O.DNSFlags(dt=dts[k], timestepping=scheme, **p)))
        us.append(np.ascontiguousarray(O.random_divfree_field(g, seed=500 + k, norm=0.15,
                                                              zero_mean_u=p.get("constraint") == O.BulkVelocity)))
    U = np.ascontiguousarray(np.stack(us))
    Q = np.zeros((4, 1) + us[0].shape[1:], complex)
    ens.advance(U, Q, 9)
    cfl = ens.CFL()
    for k, p in enumerate(params):
        fl = O.DNSFlags(dt=dts[k], timestepping=scheme, **p)
        u, q = us[k].copy(), np.zeros((1,) + us[k].shape[1:], complex)
        d = DNS(u, to_cgrid(g), to_cflags(fl))
        d.advance(u, q, 9)
        assert rel_l2(U[k], u, g) <= 1e-13, (k, rel_l2(U[k], u, g))
        assert abs(cfl[k] - d.CFL()) <= 1e-12 * d.CFL()
        d.close()
