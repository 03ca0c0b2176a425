"""DNS::reset_gradp / reset_bulkv / reset_time mid-run (channelflow/dns.cpp:199-232, nse.cpp:724-745)
against the oracle: switching the constraint keeps the base flow and changes the step from the next call
on.  Tolerance 1e-10 relative L2 (FP64 path)."""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import POISEUILLE_BOX, rel_l2, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scheme", [O.SBDF3, O.CNAB2])
def test_constraint_switch_matches_oracle(scheme):
    from channelflow_gb300 import DNS, build
    build.build()
    g = O.Grid(16, 33, 16, *POISEUILLE_BOX)
    fl = O.DNSFlags(nu=1 / 2000, dt=0.01, baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3,
                    timestepping=scheme, initstepping=O.SMRK2)
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=41, norm=0.1, zero_mean_u=True))
    q0 = np.zeros((1,) + u0.shape[1:], complex)
    ref = O.DNS(u0.copy(), q0.copy(), g, fl)
    ur, qr = u0.copy(), q0.copy()
    d = DNS(u0.copy(), to_cgrid(g), to_cflags(fl))
    u, q = u0.copy(), q0.copy()
    c = d.constraint()
    assert abs(c["UbulkRef"] - 2 / 3) < 1e-15 and abs(c["Ubulk"] - 2 / 3) < 1e-12   # laminar 2/3 + zero-mean field
    for action, n in ((None, 6), (("gradp", -2.2e-3, 1e-4), 6), (("bulkv", 0.6, 0.01), 5)):
        if action and action[0] == "gradp":
            ref.reset_gradp(action[1], action[2])
            d.reset_gradp(action[1], action[2])
        elif action:
            ref.reset_bulkv(action[1], action[2])
            d.reset_bulkv(action[1], action[2])
        ur, qr = ref.advance(ur, qr, n)
        d.advance(u, q, n)
        assert rel_l2(u, ur, g) <= 1e-10, (action, rel_l2(u, ur, g))
    c = d.constraint()
    assert c["UbulkRef"] == 0.6 and c["WbulkRef"] == 0.01 and c["dPdxRef"] == 0.0
    d.reset_time(5.0)
    ref.reset_time(5.0)
    ur, qr = ref.advance(ur, qr, 2)
    d.advance(u, q, 2)
    assert rel_l2(u, ur, g) <= 1e-10
    assert abs(d.time() - 5.02) < 1e-12
    d.close()
