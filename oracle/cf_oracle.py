"""CPU oracle for the channelflow DNS time step (test infrastructure only).

This module is the correctness oracle of the GPU implementation.  It is a
NumPy/SciPy restatement of channelflow's FP64 DNS step, written from the
reference sources function by function (citations are to files inside the
channelflow project).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` may import it; the product path in
``channelflow_gb300`` never does.

Parity pins: the oracle reproduces the reference's golden regression
``tests/timeIntegrationTest.cpp`` (``data/uinit`` -> 440 SBDF3 steps ->
``data/ufinal``) and the reference's self-checking tests (tau solver
residuals, laminar profiles, zero/parabola steady states, Orr-Sommerfeld
growth).  See ``tests/test_oracle_golden.py``.

Layout conventions (identical to the reference's serial FlowField):
  spectral field  u[i, my, mx, mz]  complex128, Mz = Nz//2 + 1
  physical field  u[i, ny, nx, nz]  float64
Per-mode 1-D work (Chebyshev profiles) uses arrays shaped (N, B): the
Chebyshev index first, a batch of (kx, kz) modes last, exactly like the GPU
layout [n][mode].

The transforms use numpy's pocketfft for the xz FFTs and scipy's DCT-I for
the Chebyshev transform.  They are not bit-identical to FFTW but agree to
round-off; everything else follows the reference's operation order.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import scipy.fft as sfft

PI = math.pi
# Threads for the FFT/DCT calls (scipy.fft workers). The transforms are the oracle's cost at large grids;
# the thread count does not change any result.
WORKERS = int(os.environ.get("CF_ORACLE_WORKERS", "0")) or (os.cpu_count() or 1)

# Enumerations mirroring channelflow/dnsflags.h:24-38 (same names, same order).
ZeroBase, LinearBase, ParabolicBase, LaminarBase, SuctionBase, ArbitraryBase = range(6)
PressureGradient, BulkVelocity = range(2)
CNFE1, CNAB2, CNRK2, SMRK2, SBDF1, SBDF2, SBDF3, SBDF4 = range(8)
Rotational, Convection, Divergence, SkewSymmetric, Alternating, Alternating_, LinearAboutProfile = range(7)
NoDealiasing, DealiasXZ, DealiasY, DealiasXYZ = range(4)


# ---------------------------------------------------------------------------
# Chebyshev primitives (channelflow/chebyshev.cpp)
# ---------------------------------------------------------------------------

def chebypoints(N: int, a: float = -1.0, b: float = 1.0) -> np.ndarray:
    """Gauss-Lobatto points, y_j = c + r cos(j pi/(N-1)) (chebyshev.cpp:720-728)."""
    piN = PI / (N - 1)
    radius = (b - a) / 2
    center = (b + a) / 2
    return np.array([center + radius * math.cos(j * piN) for j in range(N)])


def chebyfft(x: np.ndarray, axis: int = 0) -> np.ndarray:
    """Physical values -> Chebyshev coefficients (ChebyCoeff::chebyfft, chebyshev.cpp:262-284).

    FFTW REDFT00 is the unnormalised DCT-I; scipy's type-1 DCT is the same sum.
    """
    N = x.shape[axis]
    y = sfft.dct(x, type=1, axis=axis, workers=WORKERS)
    nrm = 1.0 / (N - 1)
    y = y * nrm
    sl0 = [slice(None)] * y.ndim
    sl0[axis] = 0
    y[tuple(sl0)] *= 0.5
    sl0[axis] = N - 1
    y[tuple(sl0)] *= 0.5
    return y


def ichebyfft(c: np.ndarray, axis: int = 0) -> np.ndarray:
    """Chebyshev coefficients -> physical values (ChebyCoeff::ichebyfft, chebyshev.cpp:286-303)."""
    N = c.shape[axis]
    x = np.array(c, copy=True)
    sl = [slice(None)] * x.ndim
    sl[axis] = slice(1, N - 1)
    x[tuple(sl)] *= 0.5
    return sfft.dct(x, type=1, axis=axis, workers=WORKERS)


def cdiff(u: np.ndarray, L: float) -> np.ndarray:
    """Spectral y-derivative along axis 0 (diff, chebyshev.cpp:672-697)."""
    N = u.shape[0]
    Nb = N - 1
    d = np.zeros_like(u)
    if Nb <= 0:
        return d
    scale = 4.0 / L
    d[Nb - 1] = (scale * Nb) * u[Nb]
    for n in range(Nb - 2, -1, -1):
        d[n] = d[n + 2] + (scale * (n + 1)) * u[n + 1]
    d[0] = d[0] * 0.5
    return d


def cdiff2(u: np.ndarray, L: float) -> np.ndarray:
    """Second derivative by two first derivatives (diff2, chebyshev.cpp:699-708)."""
    return cdiff(cdiff(u, L), L)


def eval_b(u: np.ndarray):
    """Value at y=b: sum of coefficients, high index first (chebyshev.cpp:405-416)."""
    s = np.zeros_like(u[0])
    for n in range(u.shape[0] - 1, -1, -1):
        s = s + u[n]
    return s


def eval_a(u: np.ndarray):
    """Value at y=a: alternating sum, high index first (chebyshev.cpp:418-430)."""
    s = np.zeros_like(u[0])
    for n in range(u.shape[0] - 1, -1, -1):
        s = s + (u[n] if n % 2 == 0 else -u[n])
    return s


def cmean(u: np.ndarray):
    """Mean over [a,b] from coefficients (ChebyCoeff::mean, chebyshev.cpp:505-513)."""
    s = np.array(u[0], copy=True)
    for n in range(2, u.shape[0], 2):
        s = s - u[n] / (n * n - 1)
    return s


def l2_weight_matrix(N: int) -> np.ndarray:
    """Quadratic-form weights of the Chebyshev L2 norm (L2Norm2, chebyshev.cpp:758-773)."""
    W = np.zeros((N, N))
    e = 1
    for m in range(N):
        for n in range(m % 2, N, 2):
            W[m, n] = (e - m * m - n * n) / ((e + m - n) * (e - m + n) * (e + m + n) * (e - m - n))
    return W


def cheb_l2norm2(u: np.ndarray, a: float = -1.0, b: float = 1.0, normalize: bool = True):
    """Chebyshev L2 norm squared along axis 0 (chebyshev.cpp:758-773); complex = re + im parts."""
    if np.iscomplexobj(u):
        return cheb_l2norm2(u.real, a, b, normalize) + cheb_l2norm2(u.imag, a, b, normalize)
    N = u.shape[0]
    W = l2_weight_matrix(N)
    s = np.zeros_like(u[0])
    for m in range(N - 1, -1, -1):
        s = s + u[m] * np.tensordot(W[m], u, axes=(0, 0))
    if not normalize:
        s = s * (b - a)
    return s


# ---------------------------------------------------------------------------
# Banded tridiagonal UL solver (channelflow/bandedtridiag.cpp), batched
# ---------------------------------------------------------------------------

class BandedTridiag:
    """Row 0 full, rows 1.. tridiagonal; batch of matrices along the last axis.

    Storage follows the reference's aliasing (bandedtridiag.h:79-117): the
    first row is ``band``; element (0,0) is band[0] and (0,1) is band[1].
    """

    def __init__(self, M: int, batch: int = 1):
        self.M = M
        self.band = np.zeros((M, batch))
        self.diag = np.zeros((M, batch))
        self.up = np.zeros((M, batch))
        self.lo = np.zeros((M, batch))
        self.invdiag = np.zeros((M, batch))

    def d0(self):
        return self.band[0]

    def ULdecomp(self):
        """No-pivot UL factorisation (bandedtridiag.cpp:212-229)."""
        M = self.M
        Mb = M - 1
        for k in range(Mb, 1, -1):
            Akk = self.diag[k]
            w = self.lo[k]
            self.up[k - 1] = self.up[k - 1] / Akk
            self.diag[k - 1] = self.diag[k - 1] - w * self.up[k - 1]
            self.band[k] = self.band[k] / Akk
            self.band[k - 1] = self.band[k - 1] - w * self.band[k]
        self.band[1] = self.band[1] / self.diag[1]
        self.band[0] = self.band[0] - self.lo[1] * self.band[1]
        self.diag[0] = self.band[0]
        self.invdiag = 1.0 / np.where(np.arange(M)[:, None] == 0, self.band[0][None, :], self.diag)

    def ULsolve(self, b: np.ndarray) -> np.ndarray:
        """Solve A x = b given UL = A (ULsolveStrided, bandedtridiag.cpp:232-277)."""
        M = self.M
        Mb = M - 1
        b = np.array(b, copy=True)
        for i in range(Mb - 1, 0, -1):
            b[i] = b[i] - self.up[i] * b[i + 1]
        for j in range(1, M):
            b[0] = b[0] - self.band[j] * b[j]
        b[0] = b[0] / self.band[0]
        for i in range(1, M):
            b[i] = (b[i] - self.lo[i] * b[i - 1]) * self.invdiag[i]
        return b

    def multiply(self, x: np.ndarray) -> np.ndarray:
        """b = A x (multiplyStrided, bandedtridiag.cpp:315-333)."""
        M = self.M
        Mbar = M - 1
        out = np.empty_like(x)
        s = np.zeros_like(x[0])
        for j in range(M):
            s = s + self.band[j] * x[j]
        out[0] = s
        for i in range(1, Mbar):
            out[i] = self.lo[i] * x[i - 1] + self.diag[i] * x[i] + self.up[i] * x[i + 1]
        out[Mbar] = self.lo[Mbar] * x[Mbar - 1] + self.diag[Mbar] * x[Mbar]
        return out


# ---------------------------------------------------------------------------
# Helmholtz solver (channelflow/helmholtz.cpp), batched over lambda
# ---------------------------------------------------------------------------

class HelmholtzSolver:
    """nu u'' - lambda u = f, u(a)=ua, u(b)=ub, Chebyshev tau (helmholtz.cpp:18-77)."""

    def __init__(self, nModes: int, a: float, b: float, lam, nu: float = 1.0):
        lam = np.atleast_1d(np.asarray(lam, dtype=float))
        B = lam.shape[0]
        self.nModes = nModes
        self.N_ = N_ = nModes - 1
        self.a, self.b, self.lam, self.nu = a, b, lam, nu
        nE = N_ // 2 + 1
        nO = N_ // 2
        assert nModes % 2 == 1 and nModes > 2
        nuscaled = nu / (((b - a) / 2) ** 2)

        def beta(n):
            return 0 if n > N_ - 2 else 1

        def c(n):
            return 2 if (n == 0 or n == N_) else 1

        self.Ae, self.Ao = BandedTridiag(nE, B), BandedTridiag(nO, B)
        self.Be, self.Bo = BandedTridiag(nE, 1), BandedTridiag(nO, 1)
        for A, Bm, M, first in ((self.Ae, self.Be, nE, 0), (self.Ao, self.Bo, nO, 1)):
            Bm.band[0] = 1.0
            A.band[:] = 1.0
            A.up[0] = A.band[1] if M > 1 else 0.0
            for i in range(1, M):
                n = 2 * i + first
                nn = n * n
                A.lo[i] = -(c(n - 2) * lam) / (4 * n * (n - 1))
                A.diag[i] = nuscaled + (beta(n) * lam) / (2 * (nn - 1))
                if beta(n + 2):
                    A.up[i] = -lam / (4 * n * (n + 1))
                Bm.lo[i] = float(c(n - 2)) / (4 * n * (n - 1))
                Bm.diag[i] = -float(beta(n)) / (2 * (nn - 1))
                if beta(n + 2):
                    Bm.up[i] = 1.0 / (4 * n * (n + 1))
            A.diag[0] = A.band[0]
            Bm.diag[0] = Bm.band[0]
        self.Ae.ULdecomp()
        self.Ao.ULdecomp()

    def solve(self, f: np.ndarray, ua=0.0, ub=0.0) -> np.ndarray:
        """HelmholtzSolver::solve (helmholtz.cpp:79-95); f shaped (N, B) real."""
        u = np.empty_like(f)
        u[0::2] = self.Be.multiply(f[0::2])
        u[1::2] = self.Bo.multiply(f[1::2])
        u[0] = (ub + ua) / 2
        u[1] = (ub - ua) / 2
        u[0::2] = self.Ae.ULsolve(u[0::2])
        u[1::2] = self.Ao.ULsolve(u[1::2])
        return u

    def solve_mean(self, f: np.ndarray, umean, ua=0.0, ub=0.0):
        """Mean-constrained solve for (u, mu) (helmholtz.cpp:158-213)."""
        utmp = self.solve(f, ua, ub)
        uamean = cmean(utmp)
        rtmp = np.zeros_like(f)
        rtmp[0] = self.nu
        utmp = self.solve(rtmp, 0.0, 0.0)
        ucmean = cmean(utmp)
        mu = self.nu * (umean - uamean) / ucmean
        rtmp = np.array(f, copy=True)
        rtmp[0] = rtmp[0] + mu
        return self.solve(rtmp, ua, ub), mu


# ---------------------------------------------------------------------------
# Tau solver (channelflow/tausolver.cpp), batched over (kx, kz) modes
# ---------------------------------------------------------------------------

def n_func(k: int, Nb: int) -> int:
    """tausolver.cpp:17-26."""
    if k == 0:
        return Nb - 1
    elif k == Nb:
        return 0
    elif k % 2 == 0:
        return 2 * (Nb - 1)
    return 2 * Nb


class TauSolver:
    """Per-mode Stokes/tau solver with influence matrix and tau correction.

    Batched restatement of TauSolver (tausolver.cpp:81-176 ctor,
    178-191 influenceCorrection, 193-251 solve_P_and_v, 347-450 solve).
    ``kx``, ``kz``, ``lam`` are arrays of length B.
    """

    def __init__(self, kx, kz, Lx, Lz, a, b, lam, nu, N, tauCorrection=True):
        kx = np.atleast_1d(np.asarray(kx))
        kz = np.atleast_1d(np.asarray(kz))
        lam = np.atleast_1d(np.asarray(lam, dtype=float))
        self.N, self.Nb = N, N - 1
        self.kx, self.kz = kx, kz
        self.a, self.b, self.nu, self.lam = a, b, nu, lam
        self.L = b - a
        self.tauCorrection = tauCorrection
        self.two_pi_kxLx = 2 * PI * kx / Lx
        self.two_pi_kzLz = 2 * PI * kz / Lz
        self.kappa2 = 4 * PI ** 2 * ((kx / Lx) ** 2 + (kz / Lz) ** 2)
        self.zero = (kx == 0) & (kz == 0)
        self.pH = HelmholtzSolver(N, a, b, self.kappa2, 1.0)
        self.vH = HelmholtzSolver(N, a, b, lam, nu)
        B = kx.shape[0]
        L = self.L
        zero = np.zeros((N, B))
        with np.errstate(divide="ignore", invalid="ignore"):
            self.P_plus = self.pH.solve(zero, 0.0, 1.0)
            self.v_plus = self.vH.solve(cdiff(self.P_plus, L), 0.0, 0.0)
            self.P_minus = self.pH.solve(zero, 1.0, 0.0)
            self.v_minus = self.vH.solve(cdiff(self.P_minus, L), 0.0, 0.0)
            dvp = cdiff(self.v_plus, L)
            dvm = cdiff(self.v_minus, L)
            A = eval_b(dvp)
            Bq = eval_b(dvm)
            C = eval_a(dvp)
            D = eval_a(dvm)
            disc = A * D - Bq * C
            self.i00 = D / disc
            self.i01 = -Bq / disc
            self.i10 = -C / disc
            self.i11 = A / disc
            c = 2 / (b - a)
            p0_rhs = np.array([c * n_func(i, self.Nb) for i in range(N)])[:, None] * np.ones((1, B))
            self.P_0 = self.pH.solve(p0_rhs, 0.0, 0.0)
            dP0dy = cdiff(self.P_0, L)
            self.v_0 = self.vH.solve(dP0dy, 0.0, 0.0)
            self.P_0, self.v_0 = self.influenceCorrection(self.P_0, self.v_0)
            v0yy = cdiff2(self.v_0, L)
            Nb = self.Nb
            self.sigma0_Nb1 = lam * self.v_0[Nb - 1] + dP0dy[Nb - 1] - nu * v0yy[Nb - 1]
            self.sigma0_Nb = lam * self.v_0[Nb] + dP0dy[Nb] - nu * v0yy[Nb]

    def influenceCorrection(self, P, v):
        tmp = cdiff(v, self.L)
        plus = eval_b(tmp)
        minus = eval_a(tmp)
        dp = -self.i00 * plus - self.i01 * minus
        dm = -self.i10 * plus - self.i11 * minus
        P = P + (dp * self.P_plus + dm * self.P_minus)
        v = v + (dp * self.v_plus + dm * self.v_minus)
        return P, v

    def solve_P_and_v(self, r, Ry):
        """tausolver.cpp:193-251 (real part or imaginary part)."""
        L, Nb, nu, lam = self.L, self.Nb, self.nu, self.lam
        P = self.pH.solve(r, 0.0, 0.0)
        tmp = cdiff(P, L) - Ry
        v = self.vH.solve(tmp, 0.0, 0.0)
        with np.errstate(divide="ignore", invalid="ignore"):
            P2, v2 = self.influenceCorrection(P, v)
            if self.tauCorrection:
                tmp = cdiff2(v2, L)
                s1_Nb = lam * v2[Nb] - nu * tmp[Nb] - Ry[Nb]
                s1_Nb1 = lam * v2[Nb - 1] - nu * tmp[Nb - 1] - Ry[Nb - 1]
                tmp = cdiff(P2, L)
                s1_Nb = s1_Nb + tmp[Nb]
                s1_Nb1 = s1_Nb1 + tmp[Nb - 1]
                sNb = s1_Nb / (1.0 - self.sigma0_Nb)
                sNb1 = s1_Nb1 / (1.0 - self.sigma0_Nb1)
                ev = (np.arange(self.N) % 2 == 0)[:, None]
                P2 = P2 + np.where(ev, sNb1, sNb) * self.P_0
                v2 = v2 + np.where(ev, sNb, sNb1) * self.v_0
        z = self.zero[None, :]
        P = np.where(z, P, P2)
        v = np.where(z, 0.0, v2)
        return P, v

    def _pv(self, Rx, Ry, Rz):
        L = self.L
        kxL = self.two_pi_kxLx
        kzL = self.two_pi_kzLz
        rr = cdiff(Ry.real, L)
        rr = rr - (kxL * Rx.imag + kzL * Rz.imag)
        Pre, vre = self.solve_P_and_v(rr, Ry.real)
        rr = cdiff(Ry.imag, L)
        rr = rr + (kxL * Rx.real + kzL * Rz.real)
        Pim, vim = self.solve_P_and_v(rr, Ry.imag)
        return Pre, Pim, vre, vim

    def solve(self, Rx, Ry, Rz):
        """General-mode solve (tausolver.cpp:347-402); returns complex (u, v, w, P)."""
        kxL, kzL = self.two_pi_kxLx, self.two_pi_kzLz
        Pre, Pim, vre, vim = self._pv(Rx, Ry, Rz)
        # r = i kx P - Rx : re = -kx*Pim - Rx.re, im = kx*Pre - Rx.im
        ure = self.vH.solve(-(kxL * Pim) - Rx.real, 0.0, 0.0)
        uim = self.vH.solve(kxL * Pre - Rx.imag, 0.0, 0.0)
        wre = self.vH.solve(-(kzL * Pim) - Rz.real, 0.0, 0.0)
        wim = self.vH.solve(kzL * Pre - Rz.imag, 0.0, 0.0)
        return ure + 1j * uim, vre + 1j * vim, wre + 1j * wim, Pre + 1j * Pim

    def solve_bulk(self, Rx, Ry, Rz, umean, wmean):
        """(0,0) solve with bulk-flux constraint (tausolver.cpp:404-450); returns (u,v,w,P,dPdx,dPdz)."""
        kxL, kzL = self.two_pi_kxLx, self.two_pi_kzLz
        Pre, Pim, vre, vim = self._pv(Rx, Ry, Rz)
        ure, dPdx = self.vH.solve_mean(-(kxL * Pim) - Rx.real, umean, 0.0, 0.0)
        uim = self.vH.solve(kxL * Pre - Rx.imag, 0.0, 0.0)
        wre, dPdz = self.vH.solve_mean(-(kzL * Pim) - Rz.real, wmean, 0.0, 0.0)
        wim = self.vH.solve(kzL * Pre - Rz.imag, 0.0, 0.0)
        return ure + 1j * uim, vre + 1j * vim, wre + 1j * wim, Pre + 1j * Pim, dPdx, dPdz

    def verify(self, u, v, w, P, Rx, Ry, Rz):
        """Residual of the discrete Stokes problem (after TauSolver::verify, tausolver.cpp:452-629).

        Returns, per mode, the sum of: L2 residual of nu u'' - lambda u -
        grad P + R (lambda includes nu kappa^2) over the first N-2 Chebyshev
        equations of each momentum component, the divergence, and the
        boundary values of u, v, w and v'.
        """
        L, nu, lam = self.L, self.nu, self.lam
        k2 = self.kappa2
        Dx = 1j * self.two_pi_kxLx
        Dz = 1j * self.two_pi_kzLz
        err = np.zeros(u.shape[1])
        for f, Rf, grad in ((u, Rx, Dx * P), (w, Rz, Dz * P)):
            res = nu * (cdiff2(f.real, L) + 1j * cdiff2(f.imag, L)) - lam * f - grad + Rf
            err += np.sqrt(cheb_l2norm2(res[: self.N - 2]))
        Py = cdiff(P.real, L) + 1j * cdiff(P.imag, L)
        res = nu * (cdiff2(v.real, L) + 1j * cdiff2(v.imag, L)) - lam * v - Py + Ry
        err += np.sqrt(cheb_l2norm2(res[: self.N - 2]))
        vy = cdiff(v.real, L) + 1j * cdiff(v.imag, L)
        div = Dx * u + vy + Dz * w
        err += np.sqrt(cheb_l2norm2(div))
        for f in (u, v, w):
            err += np.abs(eval_a(f)) + np.abs(eval_b(f))
        err += np.abs(eval_a(vy)) + np.abs(eval_b(vy))
        return err


# ---------------------------------------------------------------------------
# Laminar profiles (channelflow/nse.cpp:823-943)
# ---------------------------------------------------------------------------

def laminarProfile(nu, constraint, dPdx, Ubulk, Vsuck, a, b, ua, ub, Ny) -> np.ndarray:
    u = np.zeros(Ny)
    H = b - a
    mu = Vsuck * H / nu
    if abs(mu) == 0.0:
        if constraint == BulkVelocity:
            u[0] = 0.125 * (ub + ua) + 0.75 * Ubulk
            u[1] = 0.5 * (ub - ua)
            u[2] = 0.375 * (ub + ua) - 0.75 * Ubulk
        else:
            dPdx = dPdx * ((b - a) / 2) ** 2
            u[0] = 0.5 * (ub + ua) - 0.25 * dPdx / nu
            u[1] = 0.5 * (ub - ua)
            u[2] = 0.25 * dPdx / nu
        return u
    mu = H * Vsuck / nu
    ub_ua = ub - ua
    expm1_mu = math.expm1(-mu)
    dPdx_HH_nu = dPdx * H * H / nu
    y = chebypoints(Ny, a, b)
    phys = np.zeros(Ny)
    if abs(mu) > 1e-01:
        if constraint == BulkVelocity:
            k = -1.0 / expm1_mu - 1 / mu
            dPdx_HH_nu = mu * (Ubulk - ua - ub_ua * k) / (0.5 - k)
        for i in range(Ny):
            yhat = (y[i] - a) / H
            e = math.expm1(-mu * yhat)
            phys[i] = ua + ub_ua * e / expm1_mu + dPdx_HH_nu * (yhat - e / expm1_mu) / mu
    else:
        if constraint == BulkVelocity:
            mu2 = mu * mu
            A = ub - ua
            Bc = ua + ub - 2 * Ubulk
            dPdx_HH_nu = 6 * Bc + mu * (A + mu * (Bc / 10 + mu2 * (-Bc / 1400 + mu2 * Bc / 126000)))
        one_2, one_12, one_24 = 1.0 / 2, 1.0 / 12, 1.0 / 24
        one_720, one_1440, one_30240, one_120960 = 1.0 / 720, 1.0 / 1440, 1.0 / 30240, 1.0 / 120960
        for i in range(Ny):
            yh = (y[i] - a) / H
            yh2 = yh * yh
            yh3 = yh2 * yh
            yh4 = yh3 * yh
            yh_1 = yh - 1
            t1 = yh + mu * (-one_2 * yh * yh_1 + mu * (one_12 * yh * yh_1 * (2 * yh - 1) + mu * (
                -one_24 * (yh * yh_1) ** 2 + mu * (one_720 * yh * yh_1 * (2 * yh - 1) * (3 * yh2 - 3 * yh - 1) + mu * (
                    -one_1440 * (yh * yh_1) ** 2 * (2 * yh2 - 2 * yh - 1) + mu * (
                        one_30240 * yh * yh_1 * (2 * yh - 1) * (3 * yh4 - 6 * yh3 + 3 * yh + 1)))))))
            t2 = one_2 * yh * yh_1 + mu * (-one_12 * yh * yh_1 * (2 * yh - 1) + mu * (one_24 * (yh * yh_1) ** 2 + mu * (
                -one_720 * yh * yh_1 * (2 * yh - 1) * (3 * yh2 - 3 * yh - 1) + mu * (
                    one_1440 * (yh * yh_1) ** 2 * (2 * yh2 - 2 * yh - 1) + mu * (
                        -one_30240 * yh * yh_1 * (2 * yh - 1) * (3 * yh4 - 6 * yh3 + 3 * yh + 1) + mu * (
                            one_120960 * (yh * yh_1) ** 2 * (3 * yh4 - 6 * yh3 + 4 * yh + 2)))))))
            phys[i] = ua + ub_ua * t1 + dPdx_HH_nu * t2
    return chebyfft(phys)


# ---------------------------------------------------------------------------
# Flags and grid
# ---------------------------------------------------------------------------

@dataclass
class DNSFlags:
    """Subset of channelflow DNSFlags used by the DNS step (dnsflags.h:84-92 defaults)."""
    nu: float = 0.0025
    dPdx: float = 0.0
    dPdz: float = 0.0
    Ubulk: float = 0.0
    Wbulk: float = 0.0
    ulowerwall: float = 0.0
    uupperwall: float = 0.0
    wlowerwall: float = 0.0
    wupperwall: float = 0.0
    Vsuck: float = 0.0
    t0: float = 0.0
    dt: float = 0.03125
    baseflow: int = LaminarBase
    constraint: int = PressureGradient
    timestepping: int = SBDF3
    initstepping: int = SMRK2
    nonlinearity: int = Rotational
    dealiasing: int = DealiasXZ
    taucorrection: bool = True
    rotation: float = 0.0

    def dealias_xz(self) -> bool:
        return self.dealiasing in (DealiasXZ, DealiasXYZ)

    def dealias_y(self) -> bool:
        return self.dealiasing in (DealiasY, DealiasXYZ)


@dataclass
class Grid:
    Nx: int
    Ny: int
    Nz: int
    Lx: float
    Lz: float
    a: float = -1.0
    b: float = 1.0

    @property
    def Mz(self):
        return self.Nz // 2 + 1

    def kx(self, mx):
        return mx if mx <= self.Nx // 2 else mx - self.Nx

    def mx(self, kx):
        return kx if kx >= 0 else kx + self.Nx


# ---------------------------------------------------------------------------
# Field transforms (channelflow/flowfield.cpp:1850-1987, 2235-2255)
# ---------------------------------------------------------------------------

def make_physical(u: np.ndarray, g: Grid) -> np.ndarray:
    """Spectral [i,my,mx,mz] -> physical [i,ny,nx,nz] (makePhysical_y then makePhysical_xz)."""
    uy = ichebyfft(u, axis=1)
    return sfft.irfft2(uy, s=(g.Nx, g.Nz), axes=(2, 3), workers=WORKERS) * (g.Nx * g.Nz)


def make_spectral(p: np.ndarray, g: Grid) -> np.ndarray:
    """Physical -> spectral (makeSpectral_xz with 1/(Nx Nz) scaling, then makeSpectral_y)."""
    s = sfft.rfft2(p, axes=(2, 3), workers=WORKERS) * (1.0 / (g.Nx * g.Nz))
    return chebyfft(s, axis=1)


def aliased_mask(g: Grid, kxmax_d: int, kzmax_d: int) -> np.ndarray:
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    kz = np.arange(g.Mz)
    return (np.abs(kx)[:, None] > kxmax_d) | (kz[None, :] > kzmax_d)


def zero_padded_modes(u: np.ndarray, g: Grid) -> np.ndarray:
    """FlowField::zeroPaddedModes (flowfield.cpp:2235-2255)."""
    u = np.array(u, copy=True)
    u[:, :, aliased_mask(g, g.Nx // 3 - 1, g.Nz // 3 - 1)] = 0.0
    return u


def L2Norm2(u: np.ndarray, g: Grid, normalize: bool = True) -> float:
    """FlowField L2Norm2 over all modes, factor 2 for kz>0 (diffops.cpp:417-487)."""
    s = 0.0
    cz = np.where(np.arange(g.Mz) == 0, 1.0, 2.0)
    for i in range(u.shape[0]):
        n2 = cheb_l2norm2(u[i].reshape(g.Ny, -1)).reshape(g.Nx, g.Mz)
        s += float(np.sum(n2 * cz[None, :]))
    if not normalize:
        s *= g.Lx * g.Lz
    return s


def L2Norm(u, g, normalize=True):
    return math.sqrt(L2Norm2(u, g, normalize))


def L2Dist(u, v, g, normalize=True):
    return math.sqrt(L2Norm2(u - v, g, normalize))


def curl(u: np.ndarray, g: Grid) -> np.ndarray:
    """Spectral curl with y-derivatives by recurrence (diffops.cpp:2229-2334)."""
    Ny = g.Ny
    Myb = Ny - 1
    scale = 4.0 / (g.b - g.a)
    om = np.zeros_like(u)
    # om0 = d(u2)/dy ; om2 = -d(u0)/dy
    om[0, Myb] = 0.0
    om[0, Myb - 1] = (Myb * scale) * u[2, Myb]
    for my in range(Myb - 2, -1, -1):
        om[0, my] = om[0, my + 2] + ((my + 1) * scale) * u[2, my + 1]
    om[0, 0] *= 0.5
    om[2, Myb] = 0.0
    om[2, Myb - 1] = -(Myb * scale) * u[0, Myb]
    for my in range(Myb - 2, -1, -1):
        om[2, my] = om[2, my + 2] - ((my + 1) * scale) * u[0, my + 1]
    om[2, 0] *= 0.5
    kxmax, kzmax = g.Nx // 2, g.Nz // 2
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    kz = np.arange(g.Mz)
    ddx = 1j * (2.0 * PI * kx / g.Lx * (kx != kxmax))
    ddz = 1j * (2.0 * PI * kz / g.Lz * (kz != kzmax))
    Dx = ddx[None, :, None]
    Dz = ddz[None, None, :]
    f0, f1, f2 = u[0], u[1], u[2]
    om[0] = om[0] - Dz * f1
    om[1] = Dz * f0 - Dx * f2
    om[2] = om[2] + Dx * f1
    return om


def cross(f: np.ndarray, gph: np.ndarray) -> np.ndarray:
    """(f x g)_i = f_j g_k - f_k g_j in physical space (diffops.cpp:2560-2611)."""
    out = np.empty_like(f)
    for i in range(3):
        j, k = (i + 1) % 3, (i + 2) % 3
        out[i] = f[j] * gph[k] - f[k] * gph[j]
    return out


def grad_vec(u: np.ndarray, g: Grid) -> np.ndarray:
    """Spectral gradient tensor G[i*3+j] = d u_i / d x_j (after grad, diffops.cpp:1784-1941)."""
    kxmax, kzmax = g.Nx // 2, g.Nz // 2
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    kz = np.arange(g.Mz)
    Dx = (1j * (2.0 * PI * kx / g.Lx * (kx != kxmax)))[None, :, None]
    Dz = (1j * (2.0 * PI * kz / g.Lz * (kz != kzmax)))[None, None, :]
    L = g.b - g.a
    G = np.zeros((9,) + u.shape[1:], dtype=complex)
    for i in range(3):
        G[3 * i + 0] = Dx * u[i]
        G[3 * i + 1] = cdiff(u[i], L)
        G[3 * i + 2] = Dz * u[i]
    return G


# ---------------------------------------------------------------------------
# NSE (channelflow/nse.cpp)
# ---------------------------------------------------------------------------

class NSE:
    def __init__(self, g: Grid, flags: DNSFlags, base: Optional[Sequence[np.ndarray]] = None,
                 u0: Optional[np.ndarray] = None):
        self.g, self.flags = g, flags
        Ny = g.Ny
        self.Nyd = 2 * (Ny - 1) // 3 + 1 if flags.dealias_y() else Ny
        self.kxd_max = g.Nx // 3 - 1 if flags.dealias_xz() else g.Nx // 2
        self.kzd_max = g.Nz // 3 - 1 if flags.dealias_xz() else g.Nz // 2
        self.kxmax, self.kzmax = g.Nx // 2, g.Nz // 2
        if base is not None:
            self.Ubase, self.Wbase = np.array(base[0], float), np.array(base[1], float)
        else:
            self._create_base_flow()
        self._init_constraint(u0)
        # Solved modes in the reference's loop order with its `break` rule (nse.cpp:489-500).
        modes = []
        for mx in range(g.Nx):
            kx = g.kx(mx)
            for mz in range(g.Mz):
                kz = mz
                if (kx == self.kxmax or kz == self.kzmax) or (flags.dealias_xz() and self.is_aliased(kx, kz)):
                    break
                modes.append((mx, mz))
        self.modes = modes
        self.mx_idx = np.array([m[0] for m in modes])
        self.mz_idx = np.array([m[1] for m in modes])
        kxs = np.array([g.kx(m) for m in self.mx_idx])
        kzs = self.mz_idx.copy()
        self.kxs, self.kzs = kxs, kzs
        self.is00 = (kxs == 0) & (kzs == 0)
        self.tau = []

    def is_aliased(self, kx, kz):
        return abs(kx) > self.kxd_max or abs(kz) > self.kzd_max

    def _create_base_flow(self):
        f, g = self.flags, self.g
        Ny = g.Ny
        if f.baseflow == ZeroBase:
            self.Ubase, self.Wbase = np.zeros(Ny), np.zeros(Ny)
        elif f.baseflow == LinearBase:
            self.Ubase, self.Wbase = np.zeros(Ny), np.zeros(Ny)
            self.Ubase[1] = 1
        elif f.baseflow == ParabolicBase:
            self.Ubase, self.Wbase = np.zeros(Ny), np.zeros(Ny)
            self.Ubase[0], self.Ubase[2] = 0.5, -0.5
        elif f.baseflow == SuctionBase:
            self.Ubase = laminarProfile(f.nu, PressureGradient, 0, f.Ubulk, f.Vsuck, g.a, g.b, -0.5, 0.5, Ny)
            self.Wbase = np.zeros(Ny)
        elif f.baseflow == LaminarBase:
            self.Ubase = laminarProfile(f.nu, f.constraint, f.dPdx, f.Ubulk, f.Vsuck, g.a, g.b,
                                        f.ulowerwall, f.uupperwall, Ny)
            self.Wbase = laminarProfile(f.nu, f.constraint, f.dPdz, f.Wbulk, f.Vsuck, g.a, g.b,
                                        f.wlowerwall, f.wupperwall, Ny)
        else:
            raise ValueError("ArbitraryBase needs explicit base profiles")

    def _init_constraint(self, u0):
        """NSE::initCFConstraint (nse.cpp:634-671)."""
        f, g = self.flags, self.g
        L = g.b - g.a
        self.UbulkBase = float(cmean(self.Ubase))
        self.Ubaseyy = cdiff(cdiff(self.Ubase, L), L)
        self.WbulkBase = float(cmean(self.Wbase))
        self.Wbaseyy = cdiff(cdiff(self.Wbase, L), L)
        self.dPdxRef = self.dPdzRef = 0.0
        self.UbulkRef = self.WbulkRef = 0.0
        self.dPdxAct = self.dPdzAct = 0.0
        if f.constraint == BulkVelocity:
            self.UbulkRef = f.Ubulk
            self.WbulkRef = f.Wbulk
        else:
            self.dPdxAct = self.dPdxRef = f.dPdx
            self.dPdzAct = self.dPdzRef = f.dPdz

    def reset_lambda(self, lambda_t: Sequence[float]):
        """NSE::reset_lambda (nse.cpp:673-705): one batched TauSolver table per substep."""
        g, f = self.g, self.flags
        c = 4.0 * PI ** 2 * f.nu
        self.tau = []
        for lt in lambda_t:
            lam = lt + c * ((self.kxs / g.Lx) ** 2 + (self.kzs / g.Lz) ** 2)
            self.tau.append(TauSolver(self.kxs, self.kzs, g.Lx, g.Lz, g.a, g.b, lam, f.nu, self.Nyd,
                                      f.taucorrection))

    def nonlinear(self, u: np.ndarray):
        """navierstokesNL + zeroPaddedModes (nse.cpp:12-91, 383-391).

        Returns (f, u_after): the reference transforms u to physical space and
        back inside rotationalNL (diffops.cpp:2878), so u changes at round-off
        level; the returned u_after is that round-tripped field.
        """
        g, fl = self.g, self.flags
        if fl.nonlinearity == LinearAboutProfile:
            f = self._linearized(u)
            if fl.dealias_xz():
                f = zero_padded_modes(f, g)
            return f, np.array(u, copy=True)
        u = np.array(u, copy=True)
        u[0, :, 0, 0] += self.Ubase
        u[2, :, 0, 0] += self.Wbase
        u[1, 0, 0, 0] -= fl.Vsuck
        nl = fl.nonlinearity
        if nl == Alternating:  # nse.cpp:50-57: the flag flips on every call
            nl = Divergence
            fl.nonlinearity = Alternating_
        elif nl == Alternating_:
            nl = Convection
            fl.nonlinearity = Alternating
        if nl == Rotational:
            om = curl(u, g)
            up = make_physical(u, g)
            omp = make_physical(om, g)
            f = make_spectral(cross(omp, up), g)
            u = make_spectral(up, g)
        elif nl in (Convection, SkewSymmetric, Divergence):
            f, u = self._nl_grad_forms(u, nl)
        else:
            raise NotImplementedError("nonlinearity %d" % nl)
        if fl.rotation != 0.0:
            # -(Omega x u) with Omega = rotation e_z, on u + U (nse.cpp:62-78), linear in u
            f = f.copy()
            f[0] -= fl.rotation * u[1]
            f[1] += fl.rotation * u[0]
        u[0, :, 0, 0] -= self.Ubase
        u[2, :, 0, 0] -= self.Wbase
        u[1, 0, 0, 0] += fl.Vsuck
        if fl.dealias_xz():
            f = zero_padded_modes(f, g)
        return f, u

    def _linearized(self, u):
        """linearizedNL (diffops.cpp:3288-3361): f = (U d/dx + W d/dz) u + v (U', 0, W'), per mode in
        y-physical space (Nyquist derivatives zeroed)."""
        g = self.g
        L = g.b - g.a
        U = ichebyfft(self.Ubase)
        W = ichebyfft(self.Wbase)
        Uy = ichebyfft(cdiff(self.Ubase, L))
        Wy = ichebyfft(cdiff(self.Wbase, L))
        uy = ichebyfft(u, axis=1)  # [i, ny, mx, mz] spectral in x,z, physical in y
        kx = np.array([g.kx(m) for m in range(g.Nx)])
        kz = np.arange(g.Mz)
        ddx = 1j * 2 * PI * kx / g.Lx * (np.abs(kx) != g.Nx // 2)
        ddz = 1j * 2 * PI * kz / g.Lz * (kz != g.Nz // 2)
        D = U[:, None, None] * ddx[None, :, None] + W[:, None, None] * ddz[None, None, :]
        f = np.zeros_like(uy)
        f[0] = D * uy[0] + uy[1] * Uy[:, None, None]
        f[1] = D * uy[1]
        f[2] = D * uy[2] + uy[1] * Wy[:, None, None]
        return chebyfft(f, axis=1)

    def _nl_grad_forms(self, u, nl):
        """u.grad u (dotgrad), div(uu) (divergence) and their average (skew-symmetric).

        Follows convectionNL/dotgrad (diffops.cpp:2883-2885, 3586-3643),
        divergenceNL (3110-3134) and skewsymmetricNL (3142-3286).
        """
        g = self.g
        up = make_physical(u, g)
        out = []
        if nl in (Convection, SkewSymmetric):
            Gp = make_physical(grad_vec(u, g), g)
            conv = np.zeros_like(up)
            for i in range(3):
                for j in range(3):
                    conv[i] += up[j] * Gp[3 * i + j]
            out.append(make_spectral(conv, g))
        if nl in (Divergence, SkewSymmetric):
            uu = np.zeros((9,) + up.shape[1:])
            for i in range(3):
                for j in range(3):
                    uu[3 * i + j] = up[i] * up[j]
            uus = make_spectral(uu, g)
            kxmax, kzmax = g.Nx // 2, g.Nz // 2
            kx = np.array([g.kx(m) for m in range(g.Nx)])
            kz = np.arange(g.Mz)
            Dx = (1j * (2.0 * PI * kx / g.Lx * (kx != kxmax)))[None, :, None]
            Dz = (1j * (2.0 * PI * kz / g.Lz * (kz != kzmax)))[None, None, :]
            L = g.b - g.a
            div = np.zeros_like(u)
            for i in range(3):
                div[i] = Dx[0] * uus[3 * i + 0] + cdiff(uus[3 * i + 1], L) + Dz[0] * uus[3 * i + 2]
            out.append(div)
        f = out[0] if len(out) == 1 else 0.5 * (out[0] + out[1])
        return f, make_spectral(up, g)

    def _profiles(self, u, comp):
        return u[comp][:, self.mx_idx, self.mz_idx]

    def linear(self, u: np.ndarray, q: np.ndarray) -> np.ndarray:
        """NSE::linear (nse.cpp:393-477); unsolved modes are left zero."""
        g, fl = self.g, self.flags
        L = g.b - g.a
        Nyd = self.Nyd
        out = np.zeros_like(u)
        uk = fl.nu * self._profiles(u, 0)[:Nyd]
        vk = fl.nu * self._profiles(u, 1)[:Nyd]
        wk = fl.nu * self._profiles(u, 2)[:Nyd]
        Pk = self._profiles(q, 0)[:Nyd]
        d2 = lambda x: cdiff2(x.real, L) + 1j * cdiff2(x.imag, L)
        d1 = lambda x: cdiff(x.real, L) + 1j * cdiff(x.imag, L)
        Ruk, Rvk, Rwk = d2(uk), d2(vk), d2(wk)
        Pyk = d1(Pk)
        kappa2 = 4 * PI * PI * ((self.kxs / g.Lx) ** 2 + (self.kzs / g.Lz) ** 2)
        Dx = 1j * (2 * PI * self.kxs / g.Lx * (self.kxs != self.kxmax))
        Dz = 1j * (2 * PI * self.kzs / g.Lz * (self.kzs != self.kzmax))
        o0 = Ruk - kappa2 * uk - Dx * Pk
        o1 = Rvk - kappa2 * vk - Pyk
        o2 = Rwk - kappa2 * wk - Dz * Pk
        j00 = np.nonzero(self.is00)[0]
        if j00.size:
            j = j00[0]
            o0[:, j] += fl.nu * self.Ubaseyy[:Nyd]
            o2[:, j] += fl.nu * self.Wbaseyy[:Nyd]
            if fl.constraint == PressureGradient:
                o0[0, j] -= self.dPdxRef
                o2[0, j] -= self.dPdzRef
            else:
                Ly = g.b - g.a
                ru = cdiff(uk[:, j].real, L)
                rw = cdiff(wk[:, j].real, L)
                dPdxAct = (eval_b(ru) - eval_a(ru)) / Ly
                dPdzAct = (eval_b(rw) - eval_a(rw)) / Ly
                Uy = cdiff(self.Ubase, L)
                Wy = cdiff(self.Wbase, L)
                dPdxAct += fl.nu * (eval_b(Uy) - eval_a(Uy)) / Ly
                dPdzAct += fl.nu * (eval_b(Wy) - eval_a(Wy)) / Ly
                o0[0, j] -= dPdxAct
                o2[0, j] -= dPdzAct
        for comp, o in ((0, o0), (1, o1), (2, o2)):
            out[comp][:Nyd, self.mx_idx, self.mz_idx] = o
        return out

    def solve(self, u_out: np.ndarray, q_out: np.ndarray, rhs: np.ndarray, s: int = 0):
        """NSE::solve (nse.cpp:479-575): per-mode tau solves, written into u_out/q_out in place."""
        fl = self.flags
        Nyd = self.Nyd
        ts = self.tau[s]
        Rx = self._profiles(rhs, 0)[:Nyd].copy()
        Ry = self._profiles(rhs, 1)[:Nyd].copy()
        Rz = self._profiles(rhs, 2)[:Nyd].copy()
        uk, vk, wk, Pk = ts.solve(Rx, Ry, Rz)
        j00 = np.nonzero(self.is00)[0]
        if j00.size:
            j = j00[0]
            sub = TauSolver(np.array([0]), np.array([0]), self.g.Lx, self.g.Lz, self.g.a, self.g.b,
                            ts.lam[j:j + 1], fl.nu, Nyd, fl.taucorrection) if not hasattr(ts, "_sub00") else ts._sub00
            ts._sub00 = sub
            rx = Rx[:, j:j + 1].copy()
            ry = Ry[:, j:j + 1].copy()
            rz = Rz[:, j:j + 1].copy()
            rx.real[:, 0] += fl.nu * self.Ubaseyy[:Nyd]
            rz.real[:, 0] += fl.nu * self.Wbaseyy[:Nyd]
            if fl.constraint == PressureGradient:
                rx.real[0, 0] -= self.dPdxRef
                rz.real[0, 0] -= self.dPdzRef
                a_, b_, c_, d_ = sub.solve(rx, ry, rz)
            else:
                a_, b_, c_, d_, dPdx, dPdz = sub.solve_bulk(rx, ry, rz, self.UbulkRef - self.UbulkBase,
                                                            self.WbulkRef - self.WbulkBase)
                self.dPdxAct = float(dPdx[0])
                self.dPdzAct = float(dPdz[0])
            uk[:, j] = a_[:, 0].real
            vk[:, j] = b_[:, 0].real
            wk[:, j] = c_[:, 0].real
            Pk[:, j] = d_[:, 0].real
        for comp, x in ((0, uk), (1, vk), (2, wk)):
            u_out[comp][:Nyd, self.mx_idx, self.mz_idx] = x
        q_out[0][:Nyd, self.mx_idx, self.mz_idx] = Pk


# ---------------------------------------------------------------------------
# Time-stepping schemes (channelflow/dnsalgo.cpp) and DNS facade (dns.cpp)
# ---------------------------------------------------------------------------

class MultistepDNS:
    """SBDF1-4 / CNFE1 (dnsalgo.cpp:102-179, 202-253, 287-315)."""

    COEF = {
        CNFE1: (1.0, [-1.0], [1.0]),
        SBDF1: (1.0, [-1.0], [1.0]),
        SBDF2: (1.5, [-2.0, 0.5], [2.0, -1.0]),
        SBDF3: (11.0 / 6.0, [-3.0, 1.5, -1.0 / 3.0], [3.0, -3.0, 1.0]),
        SBDF4: (25.0 / 12.0, [-4.0, 3.0, -4.0 / 3.0, 0.25], [4.0, -6.0, 4.0, -1.0]),
    }

    def __init__(self, u, q, nse: NSE, flags: DNSFlags):
        self.nse, self.flags = nse, flags
        self.eta, self.alpha, self.beta = self.COEF[flags.timestepping]
        self.order = len(self.alpha)
        nse.reset_lambda([self.eta / flags.dt])
        self.fields = [[np.zeros_like(u), np.zeros_like(q)] for _ in range(self.order)]
        self.nonlf = [np.zeros_like(u) for _ in range(self.order)]
        self.Ninitsteps = self.order - 1
        self.countdown = self.Ninitsteps
        self.t = flags.t0

    def full(self):
        return self.countdown == 0

    def reset_dt(self, dt):
        """MultistepDNS::reset_dt (dnsalgo.cpp:191-200): new lambda, initialisation starts over."""
        self.flags.dt = dt
        self.nse.reset_lambda([self.eta / dt])
        self.countdown = self.Ninitsteps

    def _shift(self):
        for j in range(self.order - 1, 0, -1):
            self.nonlf[j], self.nonlf[j - 1] = self.nonlf[j - 1], self.nonlf[j]
            self.fields[j], self.fields[j - 1] = self.fields[j - 1], self.fields[j]

    def push(self, u, q):
        self._shift()
        if self.order > 1:
            self.fields[1] = [u.copy(), q.copy()]
            f, unew = self.nse.nonlinear(self.fields[1][0])
            self.fields[1][0] = unew
            self.nonlf[1] = f
        self.t += self.flags.dt
        self.countdown -= 1
        return u

    def advance(self, u, q, nsteps):
        J = self.order - 1
        dt = self.flags.dt
        self.fields[0] = [u.copy(), q.copy()]
        for _ in range(nsteps):
            f, unew = self.nse.nonlinear(self.fields[0][0])
            self.fields[0][0] = unew
            self.nonlf[0] = f
            rhs = np.zeros_like(u)
            for j in range(self.order):
                a = -self.alpha[j] / dt
                b = -self.beta[j]
                rhs = rhs + (a * self.fields[j][0] + b * self.nonlf[j])
            self.nse.solve(self.fields[J][0], self.fields[J][1], rhs)
            self._shift()
            self.t += dt
        return self.fields[0][0].copy(), self.fields[0][1].copy()


class CNABstyleDNS:
    """CNAB2 and SMRK2 (dnsalgo.cpp:510-576, 608-617, 641-697)."""

    def __init__(self, u, q, nse: NSE, flags: DNSFlags):
        self.nse, self.flags = nse, flags
        if flags.timestepping == CNAB2:
            self.nsub, self.Ninitsteps, self._full = 1, 1, False
            self.alpha, self.beta, self.gamma, self.zeta = [0.5], [0.5], [1.5], [-0.5]
        elif flags.timestepping == SMRK2:
            self.nsub, self.Ninitsteps, self._full = 3, 0, True
            self.alpha = [29.0 / 96.0, -3.0 / 40.0, 1.0 / 6.0]
            self.beta = [37.0 / 160.0, 5.0 / 24.0, 1.0 / 6.0]
            self.gamma = [8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0]
            self.zeta = [0.0, -17.0 / 60.0, -5.0 / 12.0]
        else:
            raise ValueError("not a CNAB-style scheme")
        self.lambda_t = [1.0 / (b * flags.dt) for b in self.beta]
        nse.reset_lambda(self.lambda_t)
        self.fj = np.zeros_like(u)
        self.fj1 = np.zeros_like(u)
        self.t = flags.t0

    def full(self):
        return self._full

    def reset_dt(self, dt):
        """CNABstyleDNS::reset_dt (dnsalgo.cpp:588-606): CNAB2 re-takes its forward-Euler start."""
        self.flags.dt = dt
        self.lambda_t = [1.0 / (b * dt) for b in self.beta]
        self.nse.reset_lambda(self.lambda_t)
        if self.flags.timestepping == CNAB2:
            self._full = False

    def push(self, u, q):
        """Returns the caller's u after the in-place transform round trip of nonlinear()."""
        self.fj, self.fj1 = self.fj1, self.fj
        self.fj, u = self.nse.nonlinear(u)
        self.t += self.flags.dt
        self._full = True
        return u

    def advance(self, u, q, nsteps):
        u, q = u.copy(), q.copy()
        for _ in range(nsteps):
            for j in range(self.nsub):
                self.fj, self.fj1 = self.fj1, self.fj
                self.fj, u = self.nse.nonlinear(u)
                a_b = self.alpha[j] / self.beta[j]
                g_b = self.gamma[j] / self.beta[j]
                z_b = self.zeta[j] / self.beta[j]
                lt = self.nse.linear(u, q)
                rhs = u * self.lambda_t[j]
                rhs = rhs + a_b * lt
                rhs = rhs + ((-g_b) * self.fj + (-z_b) * self.fj1)
                self.nse.solve(u, q, rhs, j)
            self.t += self.flags.dt
        return u, q


class RungeKuttaDNS:
    """CNRK2 (Peyret RK3/CN, dnsalgo.cpp:354-395, 419-470)."""

    def __init__(self, u, q, nse: NSE, flags: DNSFlags):
        self.nse, self.flags = nse, flags
        self.nsub = 3
        self.A = [0.0, -5.0 / 9.0, -153.0 / 128.0]
        self.B = [1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0]
        self.C = [1.0 / 6.0, 5.0 / 24.0, 1.0 / 8.0]
        self.Ninitsteps = 0
        self.lambda_t = [1.0 / (c * flags.dt) for c in self.C]
        nse.reset_lambda(self.lambda_t)
        self.Qj = np.zeros_like(u)
        self.t = flags.t0

    def full(self):
        return True

    def reset_dt(self, dt):
        """RungeKuttaDNS::reset_dt (dnsalgo.cpp:407-417)."""
        self.flags.dt = dt
        self.lambda_t = [1.0 / (c * dt) for c in self.C]
        self.nse.reset_lambda(self.lambda_t)

    def push(self, u, q):
        return u

    def advance(self, u, q, nsteps):
        u, q = u.copy(), q.copy()
        for _ in range(nsteps):
            for j in range(self.nsub):
                self.Qj = self.Qj * self.A[j]
                Qj1, u = self.nse.nonlinear(u)
                self.Qj = self.Qj - Qj1
                lt = self.nse.linear(u, q)
                B_C = self.B[j] / self.C[j]
                rhs = lt + (self.lambda_t[j] * u + B_C * self.Qj)
                self.nse.solve(u, q, rhs, j)
            self.t += self.flags.dt
        return u, q


def _new_algorithm(u, q, nse, flags):
    if flags.timestepping in (CNFE1, SBDF1, SBDF2, SBDF3, SBDF4):
        return MultistepDNS(u, q, nse, flags)
    if flags.timestepping in (CNAB2, SMRK2):
        return CNABstyleDNS(u, q, nse, flags)
    if flags.timestepping == CNRK2:
        return RungeKuttaDNS(u, q, nse, flags)
    raise ValueError("unknown time stepping %r" % flags.timestepping)


class DNS:
    """DNS facade: main scheme plus init scheme for multistep start-up (dns.cpp:22-62, 135-163)."""

    def __init__(self, u, q, g: Grid, flags: DNSFlags, base=None):
        import copy
        self.g = g
        self.flags = copy.copy(flags)
        if base is not None:
            self.flags.baseflow = ArbitraryBase
        self.main_nse = NSE(g, self.flags, base, u)
        self.main = _new_algorithm(u, q, self.main_nse, self.flags)
        self.init = None
        if not self.main.full() and flags.initstepping != flags.timestepping:
            iflags = copy.copy(self.flags)
            iflags.timestepping = flags.initstepping
            self.init_nse = NSE(g, iflags, base, u)
            self.init = _new_algorithm(u, q, self.init_nse, iflags)

    symmetries = ()
    symmetry_interval = 100

    def _project(self, u):
        """DNS::advance's projection (dns.cpp:151-155, dnsalgo.cpp:255-262, 628-632)."""
        dxz = self.flags.dealias_xz()
        for sym in self.symmetries:
            u = apply_symmetry(u, self.g, sym, True, dxz)
            m = self.main
            if isinstance(m, MultistepDNS):
                for j in range(m.order):
                    m.fields[j][0] = apply_symmetry(m.fields[j][0], self.g, sym, True, dxz)
                    m.nonlf[j] = apply_symmetry(m.nonlf[j], self.g, sym, True, dxz)
            elif isinstance(m, CNABstyleDNS):
                m.fj = apply_symmetry(m.fj, self.g, sym, True, dxz)
        return u

    def advance(self, u, q, nsteps):
        if self.symmetries and int(self.main.t) % int(self.symmetry_interval) == 0:
            u = self._project(u)
        n = 0
        while not self.main.full() and n < nsteps:
            u = self.main.push(u, q)
            u, q = self.init.advance(u, q, 1)
            n += 1
        return self.main.advance(u, q, nsteps - n)

    def reset_dt(self, dt):
        """DNS::reset_dt (dns.cpp:191-196)."""
        self.main.reset_dt(dt)
        if self.init is not None:
            self.init.reset_dt(dt)

    def reset_time(self, t):
        """DNS::reset_time (dns.cpp:199-205): both schemes' clocks."""
        self.main.t = t
        if self.init is not None:
            self.init.t = t

    def _nses(self):
        return [n for n in (getattr(self, "init_nse", None) if self.init is not None else None, self.main_nse) if n]

    def reset_gradp(self, dPdx, dPdz):
        """DNS::reset_gradp (dns.cpp:221-226) -> NSE::reset_gradp (nse.cpp:724-734): the pressure-gradient
        constraint from now on; the base flow is kept."""
        for n in self._nses():
            f = n.flags
            f.constraint, f.dPdx, f.dPdz, f.Ubulk, f.Wbulk = PressureGradient, dPdx, dPdz, 0.0, 0.0
            n.dPdxRef, n.dPdzRef, n.UbulkRef, n.WbulkRef = dPdx, dPdz, 0.0, 0.0

    def reset_bulkv(self, Ubulk, Wbulk):
        """DNS::reset_bulkv (dns.cpp:227-232) -> NSE::reset_bulkv (nse.cpp:735-745)."""
        for n in self._nses():
            f = n.flags
            f.constraint, f.Ubulk, f.Wbulk, f.dPdx, f.dPdz = BulkVelocity, Ubulk, Wbulk, 0.0, 0.0
            n.UbulkRef, n.WbulkRef, n.dPdxRef, n.dPdzRef = Ubulk, Wbulk, 0.0, 0.0

    def CFL(self, u):
        """DNSAlgorithm::CFL (dnsalgo.cpp:62-66)."""
        c = cfl_factor(u, self.g, self.main_nse.Ubase, self.main_nse.Wbase)
        f = self.main.flags
        return c * (2.0 * PI / 3.0 * f.dt if f.dealiasing in (DealiasXZ, DealiasXYZ) else PI * f.dt)


# ---------------------------------------------------------------------------
# Pressure conversions of the rotational form and single-mode fields
# ---------------------------------------------------------------------------

def up2q(u, p, g: Grid, Ubase, Wbase, nonlinearity, as_reference: bool = True):
    """DNS::up2q (dns.cpp:408-440): q = p + 1/2 |u + U|^2 for the rotational form, else q = p.

    With as_reference=True it is restated as the reference computes it: U is
    read without leaving its spectral state and the w shift uses U as well
    (dns.cpp:421-434), so the added profile is U's Chebyshev coefficients, for
    both u and w.  That corrupts q (its (0,0) mode at O(1)); schemes whose linear term
    reads q (CNRK2, and CNAB2 through its CNRK2 start) carry the error on.
    as_reference=False uses the physical U and W (the inverse of uq2p).
    """
    if nonlinearity != Rotational:
        return p.copy()
    up = make_physical(u, g)
    pp = make_physical(p, g)
    if as_reference:
        U = W = np.asarray(Ubase, float)[:, None, None]
    else:
        U = ichebyfft(np.asarray(Ubase, float))[:, None, None]
        W = ichebyfft(np.asarray(Wbase, float))[:, None, None]
    pp[0] += 0.5 * ((up[0] + U) ** 2 + up[1] ** 2 + (up[2] + W) ** 2)
    return make_spectral(pp, g)


def uq2p(u, q, g: Grid, Ubase, Wbase, nonlinearity):
    """DNS::uq2p (dns.cpp:372-406): p = q - 1/2 |u + U|^2 for the rotational form, else p = q."""
    if nonlinearity != Rotational:
        return q.copy()
    up = make_physical(u, g)
    qp = make_physical(q, g)
    U = ichebyfft(np.asarray(Ubase, float))[:, None, None]
    W = ichebyfft(np.asarray(Wbase, float))[:, None, None]
    qp[0] -= 0.5 * ((up[0] + U) ** 2 + up[1] ** 2 + (up[2] + W) ** 2)
    return make_spectral(qp, g)


def basisfunc_field(profiles, kx: int, kz: int, g: Grid) -> np.ndarray:
    """FlowField += BasisFunc and += conjugate(BasisFunc) (basisfunc.cpp:43-73, flowfield.cpp operator+=).

    ``profiles`` are the BasisFunc's complex y-profiles [ny, i] at the
    Chebyshev points (state P); the field gets their Chebyshev coefficients at
    (kx, kz) and the conjugates at (-kx, -kz), i.e. 2 Re(f(y) e^{i(alpha x + beta z)}).
    """
    prof = np.asarray(profiles, complex)
    Nd = prof.shape[1]
    c = chebyfft(prof.T, axis=1)  # [i, ny]
    out = np.zeros((Nd, g.Ny, g.Nx, g.Mz), complex)
    mx = kx % g.Nx
    out[:, :, mx, kz] += c
    out[:, :, (-kx) % g.Nx, kz] += np.conj(c)
    return out


# ---------------------------------------------------------------------------
# TimeStep (dnsflags.cpp:736-972) and f^T(u) (cfdsi.cpp:705-775)
# ---------------------------------------------------------------------------

def iround(x: float) -> int:
    """iround (cfbasics/mathdefs.h): round half away from zero."""
    return int(x + 0.5) if x > 0 else int(x - 0.5)


class TimeStep:
    """TimeStep(dt, dtmin, dtmax, dT, CFLmin, CFLmax, variable) (dnsflags.cpp:752-801, 811-972)."""

    def __init__(self, dt, dtmin, dtmax, dT, CFLmin, CFLmax, variable):
        if dtmin < 0 or dt < dtmin or dtmax < dt:
            raise ValueError("condition 0 <= dtmin <= dt <= dtmax does not hold")
        if CFLmin < 0 or CFLmax < CFLmin:
            raise ValueError("condition 0 <= CFLmin <= CFLmax does not hold")
        if dT < dtmin:
            raise ValueError("dT < dtmin")
        self.dtmin, self.dtmax, self.dT, self.T = dtmin, dtmax, dT, 0.0
        self.CFLmin, self.CFLmax, self.CFL = CFLmin, CFLmax, (CFLmax + CFLmin) / 2
        self.variable = bool(variable)
        self.N = 0
        self.n = max(iround(dT / dt), 1)
        self.dt = dT / self.n
        while self.dt < dtmin and self.n >= 2 and dT != 0:
            self.n -= 1
            self.dt = dT / self.n
        while self.dt > dtmax and dT != 0:
            self.n += 1
            self.dt = dT / self.n

    def value(self):
        """TimeStep::operator Real: dT / n."""
        return self.dT / self.n

    def adjust(self, CFL):
        self.CFL = CFL
        if self.variable and (CFL <= self.CFLmin or CFL >= self.CFLmax):
            return self.adjust_to_middle(CFL)
        return False

    def adjust_to_middle(self, CFL):
        if self.dtmin == self.dtmax or self.dT == 0.0:
            return False
        n = max(iround(2 * self.n * CFL / (self.CFLmax + self.CFLmin)), 1)
        dt = self.dT / n
        while dt < self.dtmin and dt < self.dT:
            n -= 1
            dt = self.dT / n
        while dt > self.dtmax:
            n += 1
            dt = self.dT / n
        CFL *= dt / self.dt
        adj = n != self.n
        if adj:
            self.n, self.dt, self.CFL = n, dt, CFL
        return adj

    def adjust_for_T(self, T):
        self.T = T
        if T < 0:
            raise ValueError("can't integrate backwards in time")
        if T == 0:
            adj = self.dt != 0
            self.dt, self.n, self.dT, self.T = 0.0, 0, 0.0, 0.0
            return adj
        N = max(iround(T / self.dT), 1)
        dT = T / N
        n = max(iround(dT / self.dt), 1)
        dt = dT / n
        while dt < self.dtmin and n > 2 and dT != 0:
            n -= 1
            dt = dT / n
        while dt > self.dtmax and dT != 0:
            n += 1
            dt = dT / n
        CFL = dt * self.CFL / self.dt
        adj = dt != self.dt
        self.n, self.N, self.dt, self.dT, self.CFL = n, N, dt, dT, CFL
        return adj


def ft(u, g: Grid, flags: DNSFlags, timestep: TimeStep, T: float):
    """f(u, T, h=0, ...) of cfdsi.cpp:705-775: returns (f^T(u), last CFL number)."""
    import copy
    if not np.all(np.isfinite(u)):
        raise FloatingPointError("f: u is not finite")
    if T < 0:
        return u * (1 + abs(T)), 0.0
    if T == 0:
        return u.copy(), 0.0
    dt = copy.copy(timestep)
    dt.adjust_for_T(T)
    fl = copy.copy(flags)
    fl.dt = dt.value()
    q = np.zeros((1,) + u.shape[1:], dtype=complex)
    dns = DNS(u, q, g, fl)
    f = u.copy()
    cfl = 0.0
    if dt.variable:
        f, q = dns.advance(f, q, 1)
        dt.adjust(dns.CFL(f))
        dns.reset_dt(dt.value())
        f = u.copy()
    for _ in range(1, dt.N + 1):
        cfl = dns.CFL(f)
        f, q = dns.advance(f, q, dt.n)
        if dt.variable and dt.adjust(cfl):
            dns.reset_dt(dt.value())
    if not np.all(np.isfinite(f)):
        raise FloatingPointError("f: f^T(u) is not finite")
    return f, cfl


# ---------------------------------------------------------------------------
# Seeded synthetic fields (the workloads' initial conditions)
# ---------------------------------------------------------------------------

def solved_modes(g: Grid, dealias_xz: bool = True):
    """(kx, kz) pairs of the solved set, in the reference's loop order."""
    kxd = g.Nx // 3 - 1 if dealias_xz else g.Nx // 2
    kzd = g.Nz // 3 - 1 if dealias_xz else g.Nz // 2
    out = []
    for mx in range(g.Nx):
        kx = g.kx(mx)
        for mz in range(g.Mz):
            if kx == g.Nx // 2 or mz == g.Nz // 2 or abs(kx) > kxd or mz > kzd:
                break
            out.append((kx, mz))
    return out


# ---------------------------------------------------------------------------
# Vector of the independent real coefficients of a divergence-free, no-slip
# velocity field (field2vector / vector2field, flowfield.cpp:4448-4760; the
# table of Gibson, Halcrow & Cvitanovic cited there).  The vector is what
# cfDSI's Newton-Krylov search works on (cfdsi.cpp:52-61, 140).
# ---------------------------------------------------------------------------

def fix_diri(f: np.ndarray) -> np.ndarray:
    """fixDiri (utilfuncs.cpp:712-719, complex form :757-760): f(a) = f(b) = 0 via f[0], f[1]."""
    fa, fb = eval_a(f), eval_b(f)
    f = np.array(f, copy=True)
    f[0] = f[0] - 0.5 * (fb + fa)
    f[1] = f[1] - 0.5 * (fb - fa)
    return f


def fix_diri_mean(f: np.ndarray) -> np.ndarray:
    """fixDiriMean (utilfuncs.cpp:721-728): f(a) = f(b) = 0 and mean 0 via f[0], f[1], f[2]."""
    fa, fb, fm = eval_a(f), eval_b(f), cmean(f)
    f = np.array(f, copy=True)
    f[0] = f[0] - (0.125 * (fa + fb) + 0.75 * fm)
    f[1] = f[1] - 0.5 * (fb - fa)
    f[2] = f[2] - (0.375 * (fa + fb) - 0.75 * fm)
    return f


def cintegrate(du: np.ndarray, a: float, b: float) -> np.ndarray:
    """integrate (chebyshev.cpp:637-664, complex form :1243-1246), N >= 3: zero-mean antiderivative."""
    N = du.shape[0]
    h2 = (b - a) / 2
    u = np.zeros_like(du)
    u[1] = h2 * (du[0] - du[2] / 2)
    for n in range(2, N - 1):
        u[n] = h2 * (du[n - 1] - du[n + 1]) / (2 * n)
    u[N - 1] = h2 * du[N - 2] / (2 * (N - 1))
    u[0] = u[0] - cmean(u)
    return u


def field2vector_size(g: Grid) -> int:
    """field2vector_size (flowfield.cpp:4448-4478)."""
    Kx, Kz, Ny = g.Nx // 3 - 1, g.Nz // 3 - 1, g.Ny
    return 2 * (Ny - 2) + (Kx + Kz + 2 * Kx * Kz) * (2 * (Ny - 2) + 2 * (Ny - 4))


def _ri(c: np.ndarray) -> np.ndarray:
    return np.column_stack([c.real, c.imag]).ravel()


def field2vector(u: np.ndarray, g: Grid) -> np.ndarray:
    """field2vector (flowfield.cpp:4480-4557): the independent real coefficients, in the reference's order."""
    Kx, Kz, Ny = g.Nx // 3 - 1, g.Nz // 3 - 1, g.Ny
    out = [u[0, 2:Ny, 0, 0].real, u[2, 2:Ny, 0, 0].real]
    for kx in range(1, Kx + 1):
        mx = g.mx(kx)
        out += [_ri(u[2, 2:Ny, mx, 0]), _ri(u[0, 3:Ny - 1, mx, 0])]
    for kz in range(1, Kz + 1):
        out += [_ri(u[0, 2:Ny, 0, kz]), _ri(u[2, 3:Ny - 1, 0, kz])]
    for kx in range(-Kx, Kx + 1):
        if kx == 0:
            continue
        mx = g.mx(kx)
        for kz in range(1, Kz + 1):
            out += [_ri(u[0, 2:Ny, mx, kz]), _ri(u[2, 3:Ny - 1, mx, kz])]
    return np.concatenate(out)


def vector2field(a: np.ndarray, g: Grid) -> np.ndarray:
    """vector2field (flowfield.cpp:4559-4760): the field whose independent coefficients are a, the others from
    the no-slip BCs and continuity; (kz=0, kx<0) modes are the conjugates of kx>0."""
    Kx, Kz, Ny = g.Nx // 3 - 1, g.Nz // 3 - 1, g.Ny
    Lx, Lz, ya, yb = g.Lx, g.Lz, g.a, g.b
    u = np.zeros((3, Ny, g.Nx, g.Mz), dtype=complex)
    pos = [0]

    def real(k):
        v = a[pos[0]:pos[0] + k]
        pos[0] += k
        return v

    def cplx(k):
        v = a[pos[0]:pos[0] + 2 * k:2] + 1j * a[pos[0] + 1:pos[0] + 2 * k:2]
        pos[0] += 2 * k
        return v

    f0 = np.zeros(Ny)
    f0[2:] = real(Ny - 2)
    u[0, :, 0, 0] = fix_diri(f0)
    f2 = np.zeros(Ny)
    f2[2:] = real(Ny - 2)
    u[2, :, 0, 0] = fix_diri(f2)
    for kx in range(1, Kx + 1):
        mx = g.mx(kx)
        f2 = np.zeros(Ny, complex)
        f2[2:] = cplx(Ny - 2)
        f2 = fix_diri(f2)
        f0 = np.zeros(Ny, complex)
        f0[3:Ny - 1] = cplx(Ny - 4)
        f0 = fix_diri_mean(f0)
        f1 = cintegrate(f0, ya, yb)
        f1[0] = f1[0] - 0.5 * (eval_a(f1) + eval_b(f1))
        f1 = f1 * complex(0.0, -(2 * PI * kx) / Lx)
        u[0, :, mx, 0], u[1, :, mx, 0], u[2, :, mx, 0] = f0, f1, f2
        mxm = g.mx(-kx)
        u[:, :, mxm, 0] = np.conj(u[:, :, mx, 0])
    for kz in range(1, Kz + 1):
        f0 = np.zeros(Ny, complex)
        f0[2:] = cplx(Ny - 2)
        f0 = fix_diri(f0)
        f2 = np.zeros(Ny, complex)
        f2[3:Ny - 1] = cplx(Ny - 4)
        f2 = fix_diri_mean(f2)
        f1 = cintegrate(f2, ya, yb)
        f1[0] = f1[0] - 0.5 * (eval_a(f1) + eval_b(f1))
        f1 = f1 * complex(0.0, -(2 * PI * kz) / Lz)
        u[0, :, 0, kz], u[1, :, 0, kz], u[2, :, 0, kz] = f0, f1, f2
    for kx in range(-Kx, Kx + 1):
        if kx == 0:
            continue
        mx = g.mx(kx)
        for kz in range(1, Kz + 1):
            f0 = np.zeros(Ny, complex)
            f0[2:] = cplx(Ny - 2)
            f0 = fix_diri(f0)
            u[0, :, mx, kz] = f0
            r = (kx * Lz) / (kz * Lx)
            f2 = np.zeros(Ny, complex)
            f2[3:Ny - 1] = cplx(Ny - 4)
            f2[Ny - 1] = -f0[Ny - 1] * r
            f2a, f2b = eval_a(f2), eval_b(f2)
            f2m = cmean(f2) + r * cmean(f0)
            f2[0] = f2[0] - (0.125 * (f2a + f2b) + 0.75 * f2m)
            f2[1] = f2[1] - 0.5 * (f2b - f2a)
            f2[2] = f2[2] - (0.375 * (f2a + f2b) - 0.75 * f2m)
            u[2, :, mx, kz] = f2
            g0 = f0 * complex(0, -2 * PI * kx / Lx) + f2 * complex(0, -2 * PI * kz / Lz)
            f1 = cintegrate(g0, ya, yb)
            f1[0] = f1[0] - 0.5 * (eval_a(f1) + eval_b(f1))
            u[1, :, mx, kz] = f1
    assert pos[0] == a.shape[0]
    return u


def random_divfree_field(g: Grid, seed: int, norm: float, decay_k: float = 0.5, decay_n: float = 0.7,
                         zero_mean_u: bool = False) -> np.ndarray:
    """Seeded divergence-free, no-slip perturbation with the workloads' spectral decay.

    Random Chebyshev coefficients N(0,1) * decay_k^(|kx|+|kz|) * decay_n^n
    define, per mode, v = (1-y^2)^2 g(y) and the wall-normal vorticity
    eta = (1-y^2) h(y); u and w follow from continuity, so the field is
    exactly divergence-free with u = v = w = v' = 0 at the walls.  The (0,0)
    mode carries (1-y^2) h(y) in u and w (u's mean removed when
    ``zero_mean_u``).  The kz=0 plane is Hermitian and the field is scaled
    to the requested L2Norm (diffops.cpp:415-487, normalize=true).
    Only [-1,1] walls are supported.
    """
    assert g.a == -1.0 and g.b == 1.0
    rng = np.random.default_rng(seed)
    Ny = g.Ny
    y = chebypoints(Ny)
    w1 = 1.0 - y * y
    u = np.zeros((3, Ny, g.Nx, g.Mz), dtype=complex)
    nn = np.arange(Ny)

    def rand_coeffs(kx, kz, nmax):
        amp = (decay_k ** (abs(kx) + abs(kz))) * (decay_n ** nn)
        c = (rng.standard_normal(Ny) + 1j * rng.standard_normal(Ny)) * amp
        c[nmax:] = 0.0
        return c

    L = g.b - g.a
    for kx, kz in solved_modes(g):
        if kz == 0 and kx < 0:
            continue
        mx = g.mx(kx)
        if kx == 0 and kz == 0:
            hu = ichebyfft(rand_coeffs(0, 0, Ny - 2).real)
            hw = ichebyfft(rand_coeffs(0, 0, Ny - 2).real)
            uc = chebyfft(w1 * hu)
            wc = chebyfft(w1 * hw)
            if zero_mean_u:
                # subtract (1-y^2) scaled to remove the mean: mean(1-y^2) = 2/3
                uc = uc - cmean(uc) / (2.0 / 3.0) * chebyfft(w1)
            u[0, :, 0, 0] = uc
            u[2, :, 0, 0] = wc
            continue
        gphys = ichebyfft(rand_coeffs(kx, kz, Ny - 4))
        hphys = ichebyfft(rand_coeffs(kx, kz, Ny - 2))
        vc = chebyfft(w1 * w1 * gphys)
        eta = chebyfft(w1 * hphys)
        vy = cdiff(vc.real, L) + 1j * cdiff(vc.imag, L)
        alpha = 2 * PI * kx / g.Lx
        gamma = 2 * PI * kz / g.Lz
        k2 = alpha * alpha + gamma * gamma
        uc = (alpha * (1j * vy) + gamma * (-1j * eta)) / k2
        wc = (gamma * (1j * vy) - alpha * (-1j * eta)) / k2
        u[0, :, mx, kz] = uc
        u[1, :, mx, kz] = vc
        u[2, :, mx, kz] = wc
        if kz == 0:
            mxn = g.mx(-kx)
            u[:, :, mxn, 0] = np.conj(u[:, :, mx, 0])
    nrm = L2Norm(u, g)
    return u * (norm / nrm)


def divergence_norm(u: np.ndarray, g: Grid) -> float:
    """L2 norm of div(u) for a spectral field (divNorm, diffops.cpp:89-115: the divergence's normalised L2 norm)."""
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    kz = np.arange(g.Mz)
    Dx = (1j * 2 * PI * kx / g.Lx)[None, :, None]
    Dz = (1j * 2 * PI * kz / g.Lz)[None, None, :]
    L = g.b - g.a
    d = Dx * u[0] + Dz * u[2] + cdiff(u[1].real, L) + 1j * cdiff(u[1].imag, L)
    return L2Norm(d[None], g)


def bc_norm(u: np.ndarray, g: Grid) -> float:
    """bcNorm (diffops.cpp:18-48, 85): sqrt of the sum over components and (kx, kz) modes of |u(a)|^2 + |u(b)|^2."""
    ua = eval_a(u.reshape(u.shape[0], g.Ny, -1).transpose(1, 0, 2).reshape(g.Ny, -1))
    ub = eval_b(u.reshape(u.shape[0], g.Ny, -1).transpose(1, 0, 2).reshape(g.Ny, -1))
    return math.sqrt(float(np.sum(np.abs(ua) ** 2) + np.sum(np.abs(ub) ** 2)))


def wall_slope_norm(u: np.ndarray, g: Grid) -> float:
    """Like bc_norm for dv/dy: the no-slip and continuity conditions give v' = 0 at both walls."""
    L = g.b - g.a
    v = u[1].reshape(g.Ny, -1)
    dv = cdiff(v.real, L) + 1j * cdiff(v.imag, L)
    return math.sqrt(float(np.sum(np.abs(eval_a(dv)) ** 2) + np.sum(np.abs(eval_b(dv)) ** 2)))


def load_io_field(phys_io: np.ndarray, Nx: int, Nz: int) -> np.ndarray:
    """Spectral field from physical data on the unpadded I/O grid.

    Follows FlowField::readNetCDF + addPaddedModes (flowfield.cpp:3605-3826,
    2991-3213): ``phys_io`` is [i][nz][ny][nx] as stored in the file, on the
    2(Nx/3) x Ny x 2(Nz/3) grid; its r2c transform is copied into the
    Nx x Nz spectral grid (kx >= 0 block, then the kx < 0 block shifted up),
    the remaining modes are zero, then scaled by 1/(Nx_io Nz_io) and
    transformed in y.
    """
    Nd, Nz_io, Ny, Nx_io = phys_io.shape
    p = phys_io.transpose(0, 2, 3, 1)  # [i][ny][nx][nz]
    c = np.fft.rfft2(p, axes=(2, 3))
    Mz_io = Nz_io // 2 + 1
    Mz = Nz // 2 + 1
    out = np.zeros((Nd, Ny, Nx, Mz), dtype=complex)
    out[:, :, : Nx_io // 2 + 1, :Mz_io] = c[:, :, : Nx_io // 2 + 1, :]
    out[:, :, Nx_io // 2 + 1 + (Nx - Nx_io): Nx, :Mz_io] = c[:, :, Nx_io // 2 + 1:, :]
    out *= 1.0 / (Nx_io * Nz_io)
    return chebyfft(out, axis=1)


def cfl_factor(u: np.ndarray, g: Grid, Ubase: np.ndarray, Wbase: np.ndarray) -> float:
    """FlowField::CFLfactor(Ubase, Wbase) (flowfield.cpp:4035-4068): signed max of (u_i + U_i)/dx_i."""
    up = make_physical(u, g)
    Ub = ichebyfft(Ubase)
    Wb = ichebyfft(Wbase)
    y = chebypoints(g.Ny, g.a, g.b)
    dx = [g.Lx / g.Nx, None, g.Lz / g.Nz]
    cfl = 0.0
    for i in range(3):
        for ny in range(g.Ny):
            d = dx[i] if i != 1 else ((y[0] - y[1]) if ny in (0, g.Ny - 1) else (y[ny - 1] - y[ny + 1]) / 2.0)
            Ui = Ub[ny] if i == 0 else (Wb[ny] if i == 2 else 0.0)
            cfl = max(cfl, float(np.max((up[i, ny] + Ui) / d)))
    return cfl


# ---------------------------------------------------------------------------
# Binary FlowField files (.ff): FlowField::binarySave (flowfield.cpp:2642-2723)
# and the binary branch of FlowField(filebase) (flowfield.cpp:216-356), with
# the big-endian primitives of cfbasics/cfbasics.h:368-470.
# ---------------------------------------------------------------------------

def ff_write(path, u: np.ndarray, g: Grid, padded: bool):
    """Write a spectral FlowField [Nd, Ny, Nx, Mz] the way binarySave does (version 2.0.9)."""
    import struct
    Nd = u.shape[0]
    out = [struct.pack(">7i", 2, 0, 9, g.Nx, g.Ny, g.Nz, Nd), b"SS", struct.pack(">4d", g.Lx, g.Lz, g.a, g.b),
           b"1" if padded else b"0"]
    if padded:
        Nxd, Nzd = 2 * (g.Nx // 6), 2 * (g.Nz // 3) + 1
        xs = list(range(0, Nxd + 1)) + list(range(g.Nx - Nxd, g.Nx))
        sel = u[:, :, xs, : Nzd // 2 + 1]
    else:
        sel = u
    pairs = np.stack([sel.real, sel.imag], axis=-1).astype(">f8")
    out.append(pairs.tobytes())
    with open(path, "wb") as f:
        f.write(b"".join(out))


def ff_read(path):
    """Read a spectral-state .ff file; returns (u [Nd, Ny, Nx, Mz], Grid, padded)."""
    import struct
    b = open(path, "rb").read()
    major, minor, update, Nx, Ny, Nz, Nd = struct.unpack(">7i", b[:28])
    xz, ys = b[28:29], b[29:30]
    Lx, Lz, a, bb = struct.unpack(">4d", b[30:62])
    padded = b[62:63] != b"0"
    if xz != b"S" or ys != b"S":
        raise ValueError("physical-state .ff files are not read here")
    g = Grid(Nx, Ny, Nz, Lx, Lz, a, bb)
    u = np.zeros((Nd, Ny, Nx, Nz // 2 + 1), complex)
    data = np.frombuffer(b[63:], dtype=">f8")
    if padded:
        Nxd, Nzd = 2 * (Nx // 6), 2 * (Nz // 3) + 1
        xs = list(range(0, Nxd + 1)) + list(range(Nx - Nxd, Nx))
        nz = Nzd // 2 + 1
        v = data[: Nd * Ny * len(xs) * nz * 2].reshape(Nd, Ny, len(xs), nz, 2)
        u[:, :, xs, :nz] = v[..., 0] + 1j * v[..., 1]
    else:
        v = data[: Nd * Ny * Nx * (Nz // 2 + 1) * 2].reshape(Nd, Ny, Nx, Nz // 2 + 1, 2)
        u[:] = v[..., 0] + 1j * v[..., 1]
    return u, g, padded


# ---------------------------------------------------------------------------
# FieldSymmetry (symmetry.h) on spectral fields: FlowField::operator*= and
# FlowField::project (flowfield.cpp:1095-1272).
# ---------------------------------------------------------------------------

def apply_symmetry(u, g: Grid, sym, project=False, dealias=True):
    """sym = (s, sx, sy, sz, ax, az).  Acts on |kx| <= Kx, kz <= Kz (the 2/3 set when dealias, else all but
    Nyquist), as the reference does for the stored half of the spectrum; other modes are left as they are."""
    s, sx, sy, sz, ax, az = sym
    Nd = u.shape[0]
    Kx = g.Nx // 3 - 1 if dealias else g.Nx // 2 - 1
    Kz = g.Nz // 3 - 1 if dealias else g.Nz // 2 - 1
    out = u.copy()
    n = np.arange(g.Ny)
    syl = np.where((sy == -1) & (n % 2 == 1), -1.0, 1.0)
    for i in range(Nd):
        si = (sx, sy, sz)[i] if Nd == 3 else 1
        for kx in range(-Kx, Kx + 1):
            for kz in range(0, Kz + 1):
                src = u[i, :, (sx * sz * kx) % g.Nx, kz]
                if sz == -1:
                    src = np.conj(src)
                c = s * si * syl * np.exp(1j * (2 * PI * ax * sx * kx + 2 * PI * az * sz * kz))
                img = c * src
                if project:
                    img = 0.5 * (u[i, :, kx % g.Nx, kz] + img)
                out[i, :, kx % g.Nx, kz] = img
    return out
