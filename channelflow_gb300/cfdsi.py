"""cfDSI's residual and Jacobian for Newton-Krylov searches, over the GPU library.

A search vector x is field2vector(u) (the independent reals of a divergence-free no-slip field,
flowfield.cpp:4448-4760); T, the shifts and the symmetry are fixed here (cfDSI with Tsearch, xrelative
and zrelative off).  Reference behaviour restated:

* cfDSI::eval (channelflow/cfdsi.cpp:52-61) with G (cfdsi.cpp:691-703):
  G(u) = sigma f^T(u) - u, divided by T when Tnormalize;
* DSI::Jacobian (nsolver/dsi.cpp:66-88): finite-difference directional derivative
  (G(x + eps dx) - G(x)) / eps with eps = epsDx / |dx| (1 when |dx| < epsDx), or the centred form.

The f^T(u) evaluations run on the GPU (cfgpu_ft, a DNS per call as cfDSI::f builds one, or the request
server, which evaluates a whole set of them concurrently: eval_many / jacobian_many).  The Arnoldi step of
GMRES is done in FP64 on the GPU (cfgpu_orthogonalize).  newton_gmres is a minimal host driver for these
pieces (Newton with GMRES and backtracking), not the reference's hookstep algorithm.
"""

from __future__ import annotations

import copy

import numpy as np

from . import _lib as L
from .dns import DNSFlags, Grid
from .dsi import TimeStep, field2vector, ft, vector2field
from .symmetry import FieldSymmetry, apply


def orthogonalize(V: np.ndarray, w: np.ndarray):
    """Arnoldi step in FP64 on the GPU: returns (w orthonormalised against the rows of V, h) with
    h[j] = projections (j < k) and h[k] = |w| before normalisation."""
    V = np.ascontiguousarray(np.atleast_2d(V) if np.size(V) else np.zeros((0, w.shape[0])), dtype=np.float64)
    w = np.array(w, dtype=np.float64, copy=True)
    k, n = V.shape[0], w.shape[0]
    if k and V.shape[1] != n:
        raise ValueError("basis rows and w differ in length")
    h = np.zeros(k + 1)
    L.check(L.load().cfgpu_orthogonalize(n, k, L.dptr(V) if k else None, L.dptr(w), L.dptr(h)))
    return w, h


class CFDSI:
    """G(x) = field2vector((sigma f^T(u) - u) [/ T]) with u = vector2field(x)."""

    def __init__(self, grid: Grid, flags: DNSFlags, timestep: TimeStep, T: float, sigma: FieldSymmetry | None = None,
                 Tnormalize: bool = True, precision: str = "fp64", server=None):
        self.grid, self.flags, self.timestep, self.T = grid, flags, timestep, float(T)
        self.sigma, self.Tnormalize, self.precision, self.server = sigma, Tnormalize, precision, server
        self.fcount = 0

    def _G_from_fu(self, u: np.ndarray, fu: np.ndarray) -> np.ndarray:
        if self.sigma is not None:
            fu = apply(fu, self.grid, self.sigma)
        Gu = fu - u
        if self.Tnormalize:
            Gu = Gu * (1.0 / self.T)
        return field2vector(np.ascontiguousarray(Gu), self.grid)

    def eval(self, x: np.ndarray) -> np.ndarray:
        """cfDSI::eval (cfdsi.cpp:52-61)."""
        u = vector2field(x, self.grid)
        fu, _ = ft(u, self.grid, self.flags, copy.copy(self.timestep), self.T, precision=self.precision)
        self.fcount += 1
        return self._G_from_fu(u, fu)

    def eval_many(self, xs) -> list:
        """cfDSI::eval of every x in xs; with a server, all f^T evaluations are submitted at once and run
        concurrently (batched per grid)."""
        if self.server is None:
            return [self.eval(x) for x in xs]
        from .server import DONE
        us = [vector2field(x, self.grid) for x in xs]
        ids = [self.server.submit_ft(self.grid, self.flags, copy.copy(self.timestep), self.T, u) for u in us]
        self.server.run()
        out = []
        for u, rid in zip(us, ids):
            st, fu, _ = self.server.poll(rid)
            if st != DONE:
                raise RuntimeError("f^T(u) request %d did not finish" % rid)
            self.server.release(rid)
            out.append(self._G_from_fu(u, fu))
        self.fcount += len(xs)
        return out

    @staticmethod
    def _eps(dx, epsDx):
        m = float(np.linalg.norm(dx))
        return 1.0 if m < epsDx else epsDx / m

    def jacobian(self, x, dx, Gx, epsDx: float = 1e-7, centdiff: bool = False) -> np.ndarray:
        """DSI::Jacobian (nsolver/dsi.cpp:66-88)."""
        eps = self._eps(dx, epsDx)
        if centdiff:
            gp, gm = self.eval_many([x + 0.5 * eps * dx, x - 0.5 * eps * dx])
            return (gp - gm) / eps
        return (self.eval(x + eps * dx) - Gx) / eps

    def jacobian_many(self, x, dxs, Gx, epsDx: float = 1e-7) -> list:
        """DSI::Jacobian along every direction in dxs (forward differences), all f^T evaluations at once."""
        eps = [self._eps(dx, epsDx) for dx in dxs]
        gs = self.eval_many([x + e * dx for e, dx in zip(eps, dxs)])
        return [(g - Gx) / e for g, e in zip(gs, eps)]


def newton_gmres(dsi: CFDSI, x0: np.ndarray, tol: float = 1e-12, maxit: int = 10, kmax: int = 40,
                 gmres_rtol: float = 1e-6, epsDx: float = 1e-7):
    """Newton iterations on G(x) = 0 with GMRES for J dx = -G (Arnoldi in FP64 on the GPU) and backtracking
    on |G|.  Returns (x, G(x), [|G| per iteration])."""
    x = np.array(x0, dtype=np.float64, copy=True)
    Gx = dsi.eval(x)
    hist = [float(np.linalg.norm(Gx))]
    for _ in range(maxit):
        r = hist[-1]
        if r < tol:
            break
        basis = [-Gx / r]
        H = np.zeros((kmax + 1, kmax))
        y = np.zeros(0)
        for j in range(kmax):
            w = dsi.jacobian(x, basis[j], Gx, epsDx)
            w, h = orthogonalize(np.array(basis), w)
            H[: j + 2, j] = h
            e1 = np.zeros(j + 2)
            e1[0] = r
            y = np.linalg.lstsq(H[: j + 2, : j + 1], e1, rcond=None)[0]
            res = float(np.linalg.norm(e1 - H[: j + 2, : j + 1] @ y))
            basis.append(w)
            if res <= gmres_rtol * r or h[-1] == 0.0:
                break
        dx = np.array(basis[: y.shape[0]]).T @ y
        lam = 1.0
        while True:
            xn = x + lam * dx
            Gn = dsi.eval(xn)
            if np.linalg.norm(Gn) < r or lam < 1e-3:
                break
            lam *= 0.5
        x, Gx = xn, Gn
        hist.append(float(np.linalg.norm(Gx)))
    return x, Gx, hist
