"""Newton-Krylov-hookstep search (nsolver/newtonalgorithm.cpp:334-789, 895-1346) on the host.

The search logic (GMRES, the SVD of the Hessenberg matrix, the trust-region radius and the classification of
the residual's improvement) runs on a small nonlinear system with the finite-difference Jacobian of
DSI::Jacobian (nsolver/dsi.cpp:66-88); the Gram-Schmidt step is the host form of the GPU step.  CPU only.
"""

import numpy as np

from channelflow_gb300.cfdsi import GMRES, NewtonSearchFlags, _numpy_ortho, hookstep_search


class Quadratic:
    """G(x) = A x + 0.4 (x * x) - g with a well-conditioned random A; root x*."""

    def __init__(self, n, seed):
        rng = np.random.default_rng(seed)
        self.A = np.eye(n) * 2.0 + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
        self.xs = rng.standard_normal(n) * 0.5
        self.g = self.A @ self.xs + 0.4 * self.xs * self.xs
        self.xrelative = False
        self.count = 0

    def eval(self, x):
        self.count += 1
        return self.A @ x + 0.4 * x * x - self.g

    def jacobian(self, x, dx, Gx, epsDx=1e-7, centdiff=False):
        m = float(np.linalg.norm(dx))
        eps = 1.0 if m < epsDx else epsDx / m
        if centdiff:
            return (self.eval(x + 0.5 * eps * dx) - self.eval(x - 0.5 * eps * dx)) / eps
        return (self.eval(x + eps * dx) - Gx) / eps


def test_gmres_solves_linear_system():
    rng = np.random.default_rng(1)
    n = 30
    A = np.eye(n) + 0.2 * rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    gm = GMRES(b, n, 1e-14, ortho=_numpy_ortho)
    for _ in range(n):
        gm.iterate(A @ gm.test_vector())
        if gm.residual < 1e-12:
            break
    assert np.linalg.norm(A @ gm.x - b) <= 1e-10 * np.linalg.norm(b)
    assert gm.n <= n


def test_hookstep_search_converges_from_far():
    """Started far from the root (|x0 - x*| ~ 3): the trust region limits the early steps, the search then
    converges quadratically to L2Norm(G) < 1e-13."""
    p = Quadratic(40, 3)
    x0 = p.xs + 3.0 * np.random.default_rng(5).standard_normal(40) / np.sqrt(40)
    fl = NewtonSearchFlags(epsSearch=1e-13, Nnewton=40, epsSolver=1e-10, delta=0.5, deltaMax=2.0)
    x, Gx, info = hookstep_search(p, x0, fl, ortho=_numpy_ortho)
    assert info["converged"], info
    assert np.linalg.norm(Gx) < 1e-13
    assert np.linalg.norm(x - p.xs) < 1e-10
    assert min(info["delta"]) < 2.0 or len(info["gx"]) > 2
    # the residual decreases monotonically
    assert all(b < a for a, b in zip(info["gx"], info["gx"][1:]))


def test_hookstep_trust_region_grows_from_small_radius():
    """Started with a trust radius far below the Newton step (0.02 against |dxN| ~ 4): hooksteps of radius
    delta are taken, accurate quadratic predictions grow the radius to deltaMax within the first Newton step,
    and the search converges."""
    p = Quadratic(25, 8)
    x0 = p.xs + 4.0 * np.random.default_rng(2).standard_normal(25) / 5
    fl = NewtonSearchFlags(epsSearch=1e-12, Nnewton=60, epsSolver=1e-10, delta=0.02, deltaMax=1.0)
    x, Gx, info = hookstep_search(p, x0, fl, ortho=_numpy_ortho)
    assert info["converged"], info
    assert info["delta"][0] == 0.02 and info["delta"][1] == 1.0
    assert np.linalg.norm(x - p.xs) < 1e-12
