"""The step solve with segmented parity sweeps against the one-lane sweeps and the oracle.

TauSolver::solve (tausolver.cpp:193-402) per mode: the default path splits every parity sweep of the
pressure / v and u / w passes (Helmholtz solves and derivative recurrences) over four lanes (first-order
linear recurrences joined across segments); cfgpu_set_tau_segmented(0) runs one lane per sweep.  Both are the same arithmetic up to
the order of the sums, so FP64 runs agree to 1e-12 relative L2 after 20 steps in the velocity and 1e-8 in
the pressure (whose solve amplifies round-off more); both agree with the oracle.
Cases cover the schemes (CNAB2 with SMRK2 start-up, SBDF3, CNRK2, SMRK2), both constraints (the bulk-velocity
solve is the mean-constrained Helmholtz solve of the (0,0) mode) and Ny from 9 (two rows per segment lane)
to 129 (17, the largest the segmented kernels take).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, oracle_run, rel_l2, solved_mask, to_cflags, to_cgrid

CASES = [
    ("couette_cnab2_33", (16, 33, 16), COUETTE_BOX,
     dict(timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)),
    ("poiseuille_sbdf3_bulk_35", (16, 35, 12), POISEUILLE_BOX,
     dict(timestepping=O.SBDF3, initstepping=O.SMRK2, baseflow=O.LaminarBase, constraint=O.BulkVelocity,
          Ubulk=2 / 3)),
    ("poiseuille_cnrk2_17", (12, 17, 8), POISEUILLE_BOX,
     dict(timestepping=O.CNRK2, baseflow=O.LaminarBase, constraint=O.PressureGradient, dPdx=-2 / 2000)),
    ("poiseuille_cnab2_bulk_97", (32, 97, 32), POISEUILLE_BOX,
     dict(timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase, constraint=O.BulkVelocity,
          Ubulk=2 / 3)),
    ("couette_smrk2_129", (16, 129, 8), COUETTE_BOX,
     dict(timestepping=O.SMRK2, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)),
    ("couette_cnab2_9", (16, 9, 8), COUETTE_BOX,
     dict(timestepping=O.CNAB2, initstepping=O.SMRK2, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)),
]
NSTEPS = 20


def run(u0, g, fl, precision, seg):
    from channelflow_gb300 import DNS
    from channelflow_gb300 import _lib as L
    lib = L.load()
    u = np.ascontiguousarray(u0.copy())
    q = np.zeros((1,) + u.shape[1:], complex)
    L.check(lib.cfgpu_set_tau_segmented(seg))
    try:
        d = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
        d.advance(u, q, NSTEPS)
        d.close()
    finally:
        L.check(lib.cfgpu_set_tau_segmented(1))
    return u, q


@pytest.mark.gpu
@pytest.mark.parametrize("name,dims,box,fkw", CASES, ids=[c[0] for c in CASES])
def test_segmented_solve_matches_serial_and_oracle(name, dims, box, fkw):
    from channelflow_gb300 import build
    build.build()
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(nu=1 / 1000, dt=0.01, **fkw)
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=dims[1] + 3, norm=0.2))
    useg, qseg = run(u0, g, fl, "fp64", 1)
    user, qser = run(u0, g, fl, "fp64", 0)
    assert rel_l2(useg, user, g) <= 1e-12, rel_l2(useg, user, g)
    ou, oq, _ = oracle_run(u0, g, fl, NSTEPS)
    ou[:, :, ~solved_mask(g)] = 0
    oq[:, :, ~solved_mask(g)] = 0
    assert rel_l2(useg, ou, g) <= 1e-10, rel_l2(useg, ou, g)
    # the pressure amplifies round-off (its Helmholtz solve has lambda = kappa^2, and the influence and tau
    # corrections subtract nearly equal terms): both paths agree with each other and with the oracle to 1e-8
    assert rel_l2(qseg, qser, g) <= 1e-8, rel_l2(qseg, qser, g)
    assert rel_l2(qseg, oq, g) <= 1e-8, rel_l2(qseg, oq, g)
    assert rel_l2(qser, oq, g) <= 1e-8, rel_l2(qser, oq, g)
    # the mixed path takes the same solve
    umx, _ = run(u0, g, fl, "mixed", 1)
    assert rel_l2(umx, ou, g) <= 1e-5
