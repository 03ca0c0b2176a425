"""The mixed path's forward Chebyshev transform on the tensor cores against the FP32 matrix products and the oracle.

chebyfft (chebyshev.cpp:262-284) of every real line of the nonlinear product as one GEMM on tcgen05
(BF16 splits: four of the constant matrix, three of the FP32 data, nine partial products accumulated in
FP32 in tensor memory).  The result is an FP32 transform of FP32 data: it agrees with the compensated FP32
matrix products to 2e-6 relative L2 and with the oracle's FP64 nonlinear term to the mixed path's 1e-5;
over 100 steps of the 128x97x128 benchmark the mixed run stays within the mixed tolerance of the oracle.
"""

import ctypes

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, rel_l2, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu

CASES = [
    ("couette_rot_33", (16, 33, 16), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Rotational)),
    ("poiseuille_rot_97", (32, 97, 32), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3, nonlinearity=O.Rotational)),
    ("couette_conv_49", (24, 49, 18), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Convection)),
    ("poiseuille_rot_111", (16, 111, 12), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3, nonlinearity=O.Rotational)),
]


def nonlinear(u, g, fl, mode):
    from channelflow_gb300 import DNS
    from channelflow_gb300 import _lib as L
    lib = L.load()
    L.check(lib.cfgpu_set_cheb_tensor(mode))
    try:
        d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision="mixed")
    finally:
        L.check(lib.cfgpu_set_cheb_tensor(1))
    on = ctypes.c_int(-1)
    L.check(lib.cfgpu_dns_cheb_tensor(d._h, on))
    f = d.nonlinear(u)
    d.close()
    return f, on.value


@pytest.mark.parametrize("name,dims,box,fkw", CASES, ids=[c[0] for c in CASES])
def test_tensor_forward_matches_matrix_and_oracle(name, dims, box, fkw):
    from channelflow_gb300 import build
    build.build()
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(nu=1 / 1000, dt=0.01, **fkw)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=dims[1] + 11, norm=0.3))
    ref, _ = O.NSE(g, fl, None, u).nonlinear(u)
    ftc, on = nonlinear(u, g, fl, 2)
    assert on == 1
    fmx, off = nonlinear(u, g, fl, 0)
    assert off == 0
    assert rel_l2(ftc, fmx, g) <= 2e-6, rel_l2(ftc, fmx, g)
    assert rel_l2(ftc, ref, g) <= 1e-5, rel_l2(ftc, ref, g)


def test_tensor_forward_benchmark_config_100_steps():
    from channelflow_gb300 import DNS, build
    from channelflow_gb300 import _lib as L
    from tests.test_config_parity import MIXED_TOL_POIS_100, check_constraints, oracle_result
    build.build()
    lib = L.load()
    g, fl, u0, n, ou = oracle_result("poiseuille")
    u = np.ascontiguousarray(u0.copy())
    q = np.zeros((1,) + u.shape[1:], complex)
    L.check(lib.cfgpu_set_cheb_tensor(2))
    try:
        d = DNS(u, to_cgrid(g), to_cflags(fl), precision="mixed")
    finally:
        L.check(lib.cfgpu_set_cheb_tensor(1))
    d.advance(u, q, n)
    d.close()
    assert rel_l2(u, ou, g) <= MIXED_TOL_POIS_100, rel_l2(u, ou, g)
    check_constraints(u, g)
