"""cfDSI residual/Jacobian over the GPU library and the FP64 Arnoldi step.

* cfgpu_orthogonalize (the Gram-Schmidt step of nsolver/gmres.cpp:47-83) against NumPy: 1e-13.
* CFDSI.eval = field2vector((f^T(u) - u)/T) (cfdsi.cpp:52-61, 691-703) against the oracle's f^T: 1e-10.
* DSI::Jacobian (nsolver/dsi.cpp:66-88) along several directions evaluated together through the request
  server equals the one-at-a-time evaluation (the served f^T results equal the lone ones).
* Newton-GMRES on these pieces converges to the laminar fixed point (u = 0) to |G| < 1e-12.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def test_orthogonalize_matches_numpy():
    from channelflow_gb300.cfdsi import orthogonalize
    rng = np.random.default_rng(0)
    n, k = 20011, 12
    V = np.linalg.qr(rng.standard_normal((n, k)))[0].T.copy()
    w0 = rng.standard_normal(n)
    w, h = orthogonalize(V, w0)
    p = V @ w0
    r = w0 - V.T @ p
    assert np.abs(h[:k] - p).max() <= 1e-13 * np.abs(p).max()
    assert abs(h[k] - np.linalg.norm(r)) <= 1e-13 * np.linalg.norm(r)
    assert np.abs(w - r / np.linalg.norm(r)).max() <= 1e-13
    assert np.abs(V @ w).max() <= 1e-14
    w1, h1 = orthogonalize(np.zeros((0, n)), w0)     # k = 0: normalisation only
    assert abs(h1[0] - np.linalg.norm(w0)) <= 1e-13 * np.linalg.norm(w0)


def _setup(T=1.0, dims=(16, 17, 16)):
    from channelflow_gb300.cfdsi import CFDSI
    from channelflow_gb300.dsi import TimeStep
    g = O.Grid(dims[0], dims[1], dims[2], *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    ts = TimeStep(dt=0.02, dtmin=0.02, dtmax=0.02, dT=T, CFLmin=0.0, CFLmax=1.0, variable=False)
    return g, fl, ts, CFDSI(to_cgrid(g), to_cflags(fl), ts, T)


def test_cfdsi_eval_matches_oracle():
    g, fl, ts, dsi = _setup()
    u = O.random_divfree_field(g, seed=8, norm=0.05)
    x = O.field2vector(u, g)
    Gx = dsi.eval(x)
    uo = O.vector2field(x, g)
    fu, _ = O.ft(uo, g, fl, O.TimeStep(ts.dt, ts.dtmin, ts.dtmax, ts.dT, ts.CFLmin, ts.CFLmax, ts.variable), 1.0)
    ref = O.field2vector((fu - uo) / 1.0, g)
    assert np.linalg.norm(Gx - ref) <= 1e-10 * np.linalg.norm(ref)


def test_jacobian_batched_through_server_equals_sequential():
    from channelflow_gb300.server import Server
    g, fl, ts, dsi = _setup()
    x = O.field2vector(O.random_divfree_field(g, seed=9, norm=0.05), g)
    Gx = dsi.eval(x)
    rng = np.random.default_rng(4)
    dxs = [rng.standard_normal(x.shape[0]) for _ in range(5)]
    seq = [dsi.jacobian(x, dx, Gx) for dx in dxs]
    srv = Server(slots=4)
    dsi.server = srv
    many = dsi.jacobian_many(x, dxs, Gx)
    srv.close()
    for a, b in zip(seq, many):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)


def test_newton_gmres_converges_to_laminar():
    """8x9x8: 110 unknowns, so GMRES (kmax 120) solves each Newton system to round-off; started inside the
    quadratic region (a perturbation of L2 norm 1e-4)."""
    from channelflow_gb300.cfdsi import newton_gmres
    g, fl, ts, dsi = _setup(dims=(8, 9, 8))
    x0 = O.field2vector(O.random_divfree_field(g, seed=10, norm=1e-4), g)
    assert x0.shape[0] == 110
    x, Gx, hist = newton_gmres(dsi, x0, tol=1e-12, maxit=4, kmax=120, gmres_rtol=1e-10)
    assert hist[-1] < 1e-12, hist
    assert np.linalg.norm(x) <= 1e-6 * np.linalg.norm(x0)   # |G| < 1e-12 and the slowest mode decays at ~0.006
