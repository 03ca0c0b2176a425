"""Arnoldi eigenvalues of a linearised map (nsolver/arnoldi.cpp:24-133, Eigenvals::solve in
nsolver/eigenvals.cpp:118-279, the iteration behind findeigenvals) on the host.

The operator is a matrix with known eigenvalues (a complex pair among them), reached either directly or, as in
findeigenvals, through DSI::Jacobian (nsolver/dsi.cpp:66-88) of a map f^T with a fixed point, and the DNS map
of the reference's Orr-Sommerfeld test (the oracle's DNS) whose least stable eigenvalue is the reference's
fixture; the Gram-Schmidt step is the host form of the GPU step.  CPU only.
"""

import numpy as np
import pytest

from channelflow_gb300.cfdsi import Arnoldi, EigenvalsFlags, _numpy_ortho, eigenvals

LEAD = np.array([1.5, 0.9 + 0.3j, 0.9 - 0.3j, 0.7, -0.6])


def known_matrix(n, seed):
    """A = S D S^-1: the eigenvalues LEAD (a complex pair as a 2 x 2 rotation block) and n - 5 more of
    modulus below 0.25."""
    rng = np.random.default_rng(seed)
    D = np.zeros((n, n))
    D[0, 0] = 1.5
    D[1:3, 1:3] = [[0.9, 0.3], [-0.3, 0.9]]
    D[3, 3] = 0.7
    D[4, 4] = -0.6
    D[5:, 5:] = np.diag(rng.uniform(-0.25, 0.25, n - 5))
    S = np.eye(n) + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
    return S @ D @ np.linalg.inv(S)


def sorted_by_abs(v):
    # descending modulus, ties by imaginary part (conjugate pairs come out in either order)
    return v[np.lexsort((-v.imag, -np.abs(v)))]


def test_arnoldi_finds_the_leading_eigenvalues():
    n = 80
    A = known_matrix(n, 1)
    b = np.random.default_rng(2).standard_normal(n)
    arn = Arnoldi(b, 40, 1e-13, ortho=_numpy_ortho)
    for _ in range(40):
        arn.iterate(A @ arn.test_vector())
    lam, V, rd = arn.ew(), arn.ev(), arn.rd()
    assert np.all(np.diff(np.abs(lam)) <= 1e-12)          # sorted by decreasing modulus
    assert np.allclose(sorted_by_abs(lam[:5]), sorted_by_abs(LEAD), atol=1e-9)
    for j in range(5):                                    # Ritz pairs of the leading eigenvalues
        v = V[:, j]
        assert np.linalg.norm(A @ v - lam[j] * v) <= 1e-7 * np.linalg.norm(v)
        assert rd[j] < 1e-6
    # the Krylov basis stays orthonormal
    Q = np.array(arn.Q)
    assert np.abs(Q @ Q.T - np.eye(Q.shape[0])).max() < 1e-12


def test_arnoldi_breakdown_and_iteration_limit():
    n = 20
    A = np.diag(np.arange(1.0, n + 1.0))
    e = np.zeros(n)
    e[3] = 1.0                                            # an eigenvector: the Krylov space closes at once
    arn = Arnoldi(e, 5, 1e-13, ortho=_numpy_ortho)
    with pytest.raises(RuntimeError):
        arn.iterate(A @ arn.test_vector())
    arn = Arnoldi(np.ones(n), 2, 1e-13, ortho=_numpy_ortho)
    for _ in range(2):
        arn.iterate(A @ arn.test_vector())
    with pytest.raises(ValueError):
        arn.iterate(A @ arn.test_vector())


class LinearMap:
    """A forward map with a fixed point: f^T(x) = x* + A (x - x*) + 0.05 |x - x*|^2 c, G(x) = f^T(x) - x,
    with DSI::Jacobian's finite differences (eps = epsDx / |dx|)."""

    def __init__(self, A, seed):
        rng = np.random.default_rng(seed)
        self.A = A
        self.xs = rng.standard_normal(A.shape[0])
        self.c = rng.standard_normal(A.shape[0])
        self.fcount = 0

    def ft(self, x):
        d = x - self.xs
        return self.xs + self.A @ d + 0.05 * float(d @ d) * self.c

    def eval(self, x):
        self.fcount += 1
        return self.ft(x) - x

    def jacobian(self, x, dx, Gx, epsDx=1e-7, centdiff=False):
        m = float(np.linalg.norm(dx))
        eps = 1.0 if m < epsDx else epsDx / m
        if centdiff:
            return (self.eval(x + 0.5 * eps * dx) - self.eval(x - 0.5 * eps * dx)) / eps
        return (self.eval(x + eps * dx) - Gx) / eps


@pytest.mark.parametrize("centdiff", [False, True])
def test_eigenvals_of_a_map_at_its_fixed_point(centdiff):
    n, T = 60, 10.0
    A = known_matrix(n, 4)
    dsi = LinearMap(A, 5)
    dx = np.random.default_rng(6).standard_normal(n)
    fl = EigenvalsFlags(Narnoldi=30, Nstable=2, centdiff=centdiff)
    res = eigenvals(dsi, dsi.xs, dx, T, eps=1e-7, flags=fl, ortho=_numpy_ortho)
    lam = res["Lambda"]
    tol = 1e-6 if centdiff else 2e-5                      # forward differences carry the quadratic term
    assert np.allclose(sorted_by_abs(lam[:5]), sorted_by_abs(LEAD), atol=tol)
    assert np.allclose(res["lambda"], np.log(lam.astype(complex)) / T)
    # |Lambda| > 1 only for 1.5: one unstable growth rate (the pair 0.9 +- 0.3i has modulus 0.949)
    assert res["Nnonstable"] == 1
    assert res["Nsave"] == 3
    assert res["fcount"] == (2 if centdiff else 1) * fl.Narnoldi
    assert len(res["history"]) == fl.Narnoldi
    # saved eigenfunctions: the real eigenvector of 1.5, then the pair as real and imaginary parts
    idx = [j for j, _ in res["eigvecs"]]
    assert idx == [0, 1, 2]
    v0 = res["eigvecs"][0][1]
    assert np.linalg.norm(A @ v0 - 1.5 * v0) <= 1e-4 * np.linalg.norm(v0)
    vr, vi = res["eigvecs"][1][1], res["eigvecs"][2][1]
    l1 = lam[1]
    w = vr + 1j * vi
    assert np.linalg.norm(A @ w - l1 * w) <= 1e-4 * np.linalg.norm(w)


def test_eigenvals_find_the_orr_sommerfeld_mode():
    """findeigenvals' use on a physical map: f^T of the plane-Poiseuille DNS of the reference's Orr-Sommerfeld
    test (Re = 7500, 4 x 65 x 4, SBDF3, dt = 0.02; the oracle's DNS) on the kx = 1 coefficients, T = 2,
    linearised about the laminar state by DSI::Jacobian's finite differences.  Started from the reference's
    eigenfunction (tests/data/os_ueig10_65.asc) plus noise, six Arnoldi iterations give the least stable
    mode's growth rate and frequency -i omega (os_omega10_65.cmplx) to 5e-5 (2e-5 measured; nine iterations:
    1e-5)."""
    from oracle import cf_oracle as O
    from tests.test_orrsommerfeld import GOLD, os_case

    d = np.load(GOLD)
    omega = complex(d["omega"])
    g, fl, base, _ = os_case()
    T = 2.0
    nsteps = int(round(T / fl.dt))
    n = 3 * g.Ny

    def field(x):
        c = (x[:n] + 1j * x[n:]).reshape(3, g.Ny)
        u = np.zeros((3, g.Ny, g.Nx, g.Mz), complex)
        u[:, :, 1, 0] = c
        u[:, :, g.Nx - 1, 0] = np.conj(c)          # kx = -1: the conjugate (real field, kz = 0)
        return u

    def vec(u):
        c = u[:, :, 1, 0].reshape(-1)
        return np.concatenate([c.real, c.imag])

    class OSMap:
        fcount = 0

        def eval(self, x):
            self.fcount += 1
            u = field(x)
            q = np.zeros((1, g.Ny, g.Nx, g.Mz), complex)
            u, _ = O.DNS(u.copy(), q.copy(), g, fl, base=base).advance(u, q, nsteps)
            return vec(u) - x

        def jacobian(self, x, dx, Gx, epsDx=1e-7, centdiff=False):
            m = float(np.linalg.norm(dx))
            eps = 1.0 if m < epsDx else epsDx / m
            return (self.eval(x + eps * dx) - Gx) / eps

    dx = vec(O.basisfunc_field(d["ueig"], 1, 0, g))
    dx = dx / np.linalg.norm(dx) + 1e-3 * np.random.default_rng(1).standard_normal(2 * n) / np.sqrt(2 * n)
    res = eigenvals(OSMap(), np.zeros(2 * n), dx, T, eps=1e-7, flags=EigenvalsFlags(Narnoldi=6, Nstable=1),
                    ortho=_numpy_ortho)
    lead = res["lambda"][:2]                         # the conjugate pair of the least stable mode
    exact = -1j * omega
    best = lead[np.argmin(np.abs(lead - exact))]
    assert abs(best.real - exact.real) < 5e-5 and abs(best.imag - exact.imag) < 5e-5, (best, exact)
    assert res["Nnonstable"] == 2                    # the growing pair (Im omega > 0)
    assert res["residual"][0] < 1e-3


def test_lanczos_for_a_self_adjoint_operator():
    """Lanczos (nsolver/lanczos.cpp): the extreme eigenvalues of a symmetric matrix, through eigenvals with
    isnormal as findeigenvals selects it."""
    from channelflow_gb300.cfdsi import Lanczos
    n = 70
    rng = np.random.default_rng(7)
    Qm, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.concatenate([[1.8, -1.5, 1.2], rng.uniform(-0.3, 0.3, n - 3)])
    A = (Qm * ev) @ Qm.T
    lz = Lanczos(rng.standard_normal(n), 30, 1e-13)
    for _ in range(30):
        lz.iterate(A @ lz.test_vector())
    lam = lz.ew()
    assert np.allclose(lam[:3].real, [1.8, -1.5, 1.2], atol=1e-10) and np.all(lam.imag == 0)
    v = lz.ev()[:, 0].real
    assert np.linalg.norm(A @ v - 1.8 * v) < 1e-8 * np.linalg.norm(v)
    # the tridiagonal matrix is symmetric
    T = lz.H[:30, :30]
    assert np.allclose(T, T.T)
    dsi = LinearMap(A, 8)
    res = eigenvals(dsi, dsi.xs, rng.standard_normal(n), 1.0, eps=1e-7,
                    flags=EigenvalsFlags(isnormal=True, Narnoldi=30, Nstable=1, centdiff=True))
    assert np.allclose(res["Lambda"][:3].real, [1.8, -1.5, 1.2], atol=1e-6)
