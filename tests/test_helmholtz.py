"""Batched HelmholtzSolver (cfgpu_helmholtz_solve_batched / _mean_batched) against the oracle.

HelmholtzSolver(N, a, b, lambda, nu).solve(u, f, ua, ub) (channelflow/helmholtz.cpp:18-95) and the
mean-constrained solve(u, mu, f, umean, ua, ub) (:158-213); the residual check follows the reference's
helmholtzTest (tau equations nu u'' - lambda u = f on the first N-2 coefficients, boundary values).
Tolerance: 1e-12 relative to the oracle (FP64 on both sides).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O


def _case(N, nsys, seed):
    rng = np.random.default_rng(seed)
    lam = 10.0 ** rng.uniform(-2, 4, nsys)
    f = rng.standard_normal((nsys, N)) * 0.8 ** np.arange(N)
    ua, ub = rng.standard_normal(nsys), rng.standard_normal(nsys)
    return lam, f, ua, ub


@pytest.mark.gpu
@pytest.mark.parametrize("N,a,b,nu", [(33, -1.0, 1.0, 1.0), (65, -1.0, 1.0, 1 / 400), (97, 0.0, 2.0, 1 / 4000)])
def test_helmholtz_batched_matches_oracle(N, a, b, nu):
    from channelflow_gb300 import build
    from channelflow_gb300.dns import helmholtz_solve_batched
    build.build()
    lam, f, ua, ub = _case(N, 64, N)
    u = helmholtz_solve_batched(a, b, lam, nu, f, ua, ub)
    ref = O.HelmholtzSolver(N, a, b, lam, nu).solve(f.T.copy(), ua, ub).T
    assert np.linalg.norm(u - ref) <= 1e-12 * np.linalg.norm(ref)
    # helmholtzTest-style residual: tau rows and boundary values
    s = 2.0 / (b - a)
    for k in range(0, 64, 7):
        d2 = np.polynomial.chebyshev.chebder(u[k], 2) * s * s
        r = nu * d2[: N - 2] - lam[k] * u[k][: N - 2] - f[k][: N - 2]
        assert np.abs(r).max() <= 1e-9 * max(1.0, lam[k]) * np.abs(u[k]).max()
        assert abs(np.polynomial.chebyshev.chebval(-1.0, u[k]) - ua[k]) <= 1e-11
        assert abs(np.polynomial.chebyshev.chebval(1.0, u[k]) - ub[k]) <= 1e-11


@pytest.mark.gpu
def test_helmholtz_mean_batched_matches_oracle():
    from channelflow_gb300 import build
    from channelflow_gb300.dns import helmholtz_solve_batched
    build.build()
    N, a, b, nu = 49, -1.0, 1.0, 1 / 2000
    lam, f, ua, ub = _case(N, 40, 3)
    umean = np.linspace(-0.5, 0.7, 40)
    u, mu = helmholtz_solve_batched(a, b, lam, nu, f, ua, ub, umean=umean)
    solver = O.HelmholtzSolver(N, a, b, lam, nu)
    ref, mref = solver.solve_mean(f.T.copy(), umean, ua, ub)
    assert np.linalg.norm(u - ref.T) <= 1e-12 * np.linalg.norm(ref)
    assert np.abs(mu - mref).max() <= 1e-11 * np.abs(mref).max()
    means = np.array([O.cmean(u[k]) for k in range(40)])
    assert np.abs(means - umean).max() <= 1e-12


def test_helmholtz_argument_errors():
    """Host-side checks (no GPU needed)."""
    from channelflow_gb300 import build
    from channelflow_gb300._lib import CfgpuError
    from channelflow_gb300.dns import helmholtz_solve_batched
    build.build()
    with pytest.raises(CfgpuError, match="odd"):
        helmholtz_solve_batched(-1.0, 1.0, 1.0, 1.0, np.zeros((2, 32)))
    with pytest.raises(CfgpuError):
        helmholtz_solve_batched(1.0, -1.0, 1.0, 1.0, np.zeros((2, 33)))
