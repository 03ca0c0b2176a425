"""Order-1 multistep schemes (SBDF1, CNFE1) as the start-up scheme of a multistep or CNAB2 run, against the oracle.

DNS::advance (dns.cpp:135-163) pushes the current field into the main scheme and advances the start-up scheme
one step until the main scheme is full; a multistep start-up scheme is MultistepDNS::advance with order 1
(dnsalgo.cpp:202-251).  Higher-order multistep start-up schemes would need start-up themselves (DNS::DNS warns,
dns.cpp:34-37) and are refused.  Tolerances: FP64 1e-10, mixed 1e-5 relative L2 after the steps.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, oracle_run, rel_l2, solved_mask, to_cflags, to_cgrid

CASES = [
    ("sbdf3_from_sbdf1", (16, 33, 16), COUETTE_BOX,
     dict(timestepping=O.SBDF3, initstepping=O.SBDF1, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0), 8),
    ("sbdf4_from_cnfe1_bulk", (12, 25, 12), POISEUILLE_BOX,
     dict(timestepping=O.SBDF4, initstepping=O.CNFE1, baseflow=O.LaminarBase, constraint=O.BulkVelocity,
          Ubulk=2 / 3), 10),
    ("cnab2_from_sbdf1", (16, 33, 16), POISEUILLE_BOX,
     dict(timestepping=O.CNAB2, initstepping=O.SBDF1, baseflow=O.LaminarBase, constraint=O.PressureGradient,
          dPdx=-2 / 1000), 6),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
@pytest.mark.parametrize("name,dims,box,fkw,nsteps", CASES, ids=[c[0] for c in CASES])
def test_multistep_startup_matches_oracle(name, dims, box, fkw, nsteps, precision, tol):
    from channelflow_gb300 import DNS, build
    build.build()
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(nu=1 / 1000, dt=0.01, **fkw)
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=dims[1] + 5, norm=0.2,
                                                     zero_mean_u=fl.constraint == O.BulkVelocity))
    ou, _, _ = oracle_run(u0, g, fl, nsteps, chunks=[1, 2, nsteps - 3])
    ou[:, :, ~solved_mask(g)] = 0
    u = u0.copy()
    q = np.zeros((1,) + u.shape[1:], complex)
    d = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
    for n in (1, 2, nsteps - 3):  # through the start-up steps in pieces, as the oracle
        d.advance(u, q, n)
    d.close()
    assert rel_l2(u, ou, g) <= tol, rel_l2(u, ou, g)


@pytest.mark.gpu
def test_higher_order_multistep_startup_refused():
    from channelflow_gb300 import DNS, build
    from channelflow_gb300._lib import CfgpuError
    build.build()
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, timestepping=O.SBDF4, initstepping=O.SBDF2, baseflow=O.LaminarBase,
                    ulowerwall=-1.0, uupperwall=1.0)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=3, norm=0.1))
    with pytest.raises(CfgpuError, match="order 1"):
        DNS(u, to_cgrid(g), to_cflags(fl), precision="fp64")
