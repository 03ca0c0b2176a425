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
pieces (Newton with GMRES and backtracking); hookstep_search is nsolver's Newton-Krylov-hookstep algorithm
(NewtonAlgorithm::solve with GMRES and NewtonAlgorithm::hookstep, nsolver/newtonalgorithm.cpp:334-789,
895-1346), with the x phase shift of a travelling wave as an optional extra unknown (cfDSI with xrelative,
cfdsi.cpp:555-615).
"""

from __future__ import annotations

import copy
import math
from dataclasses import dataclass

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
    """G(x) = field2vector((sigma f^T(u) - u) [/ T]) with u = vector2field(x).

    With xrelative, x carries the x phase shift ax of sigma as one more unknown after the field's reals
    (cfDSI::extractVector, cfdsi.cpp:555-580) and G's last entry is zero (cfdsi.cpp:52-61)."""

    def __init__(self, grid: Grid, flags: DNSFlags, timestep: TimeStep, T: float, sigma: FieldSymmetry | None = None,
                 Tnormalize: bool = True, precision: str = "fp64", server=None, xrelative: bool = False):
        self.grid, self.flags, self.timestep, self.T = grid, flags, timestep, float(T)
        self.sigma, self.Tnormalize, self.precision, self.server = sigma, Tnormalize, precision, server
        self.xrelative = bool(xrelative)
        self.fcount = 0

    def make_vector(self, u: np.ndarray, ax: float | None = None) -> np.ndarray:
        """x from a field (and, with xrelative, the x shift; default: sigma's)."""
        v = field2vector(np.ascontiguousarray(u), self.grid)
        if not self.xrelative:
            return v
        if ax is None:
            ax = self.sigma.ax if self.sigma is not None else 0.0
        return np.concatenate([v, [float(ax)]])

    def _split(self, x: np.ndarray):
        """(u, sigma) of x (cfDSI::extractVector)."""
        n = x.shape[0] - (1 if self.xrelative else 0)
        u = vector2field(np.ascontiguousarray(x[:n]), self.grid)
        sig = self.sigma
        if self.xrelative:
            b = sig if sig is not None else FieldSymmetry()
            sig = FieldSymmetry(b.sx, b.sy, b.sz, float(x[n]), b.az, b.s)
        return u, sig

    def _G_from_fu(self, u: np.ndarray, fu: np.ndarray, sig) -> np.ndarray:
        if sig is not None:
            fu = apply(fu, self.grid, sig)
        Gu = fu - u
        if self.Tnormalize:
            Gu = Gu * (1.0 / self.T)
        g = field2vector(np.ascontiguousarray(Gu), self.grid)
        return np.concatenate([g, [0.0]]) if self.xrelative else g

    def eval(self, x: np.ndarray) -> np.ndarray:
        """cfDSI::eval (cfdsi.cpp:52-61)."""
        u, sig = self._split(x)
        fu, _ = ft(u, self.grid, self.flags, copy.copy(self.timestep), self.T, precision=self.precision)
        self.fcount += 1
        return self._G_from_fu(u, fu, sig)

    def eval_many(self, xs) -> list:
        """cfDSI::eval of every x in xs; with a server, all f^T evaluations are submitted at once and run
        concurrently (batched per grid)."""
        if self.server is None:
            return [self.eval(x) for x in xs]
        from .server import DONE
        parts = [self._split(x) for x in xs]
        ids = [self.server.submit_ft(self.grid, self.flags, copy.copy(self.timestep), self.T, u) for u, _ in parts]
        self.server.run()
        out = []
        for (u, sig), rid in zip(parts, ids):
            st, fu, _ = self.server.poll(rid)
            if st != DONE:
                raise RuntimeError("f^T(u) request %d did not finish" % rid)
            self.server.release(rid)
            out.append(self._G_from_fu(u, fu, sig))
        self.fcount += len(xs)
        return out

    def xdiff(self, x: np.ndarray) -> np.ndarray:
        """cfDSI::xdiff (cfdsi.cpp:606-615): field2vector of du/dx, normalised; zero in the shift entry."""
        n = x.shape[0] - (1 if self.xrelative else 0)
        u = vector2field(np.ascontiguousarray(x[:n]), self.grid)
        Nx = self.grid.Nx
        kx = np.array([m if m <= Nx // 2 else m - Nx for m in range(Nx)], dtype=float)
        kx[Nx // 2] = 0.0  # the Nyquist mode has no derivative
        du = u * (2j * math.pi * kx / self.grid.Lx)[None, None, :, None]
        d = field2vector(np.ascontiguousarray(du), self.grid)
        d = d / np.linalg.norm(d)
        return np.concatenate([d, [0.0]]) if self.xrelative else d

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


# ---------------------------------------------------------------------------------------------------------------
# Newton-Krylov-hookstep (nsolver)
# ---------------------------------------------------------------------------------------------------------------

@dataclass
class NewtonSearchFlags:
    """The options of nsolver's NewtonSearchFlags with their defaults (nsolver/newtonalgorithm.cpp:62-120)."""
    epsSearch: float = 1e-13      # stop when L2Norm(G(x)) < epsSearch
    epsKrylov: float = 1e-14      # minimum norm of a new Krylov vector (GMRES benign breakdown)
    epsDx: float = 1e-7           # relative size of dx in the finite-difference Jacobian
    epsSolver: float = 1e-3       # GMRES stops when |Ax - b|/|b| < epsSolver
    epsSolverF: float = 0.05      # accept the last GMRES iterate below this residual
    centdiff: bool = False        # centred differences for the Jacobian
    Nnewton: int = 20
    Nsolver: int = 500            # GMRES iterations per Newton step
    Nhook: int = 20               # iterations of the search for the hookstep's mu
    delta: float = 0.01           # initial trust-region radius
    deltaMin: float = 1e-12
    deltaMax: float = 0.1
    deltaFuzz: float = 1e-6
    lambdaMin: float = 0.2
    lambdaMax: float = 1.5
    lambdaRequiredReduction: float = 0.5
    improvReq: float = 1e-3
    improvOk: float = 0.10
    improvGood: float = 0.75
    improvAcc: float = 0.10


def _adjust_delta(delta, rate, dmin, dmax):
    """adjustDelta (cfbasics/cfbasics.h:964-988)."""
    if delta == dmin and delta * rate < dmin:
        return dmin
    delta *= rate
    if delta <= dmin:
        delta = 0.5 * dmin
    if delta > dmax:
        delta = dmax
    return delta


def _adjust_lambda(lam, lmin, lmax):
    """adjustLambda (cfbasics/cfbasics.h:990-999).  The reference's second test repeats lam < lmin, so lam is
    never capped at lmax; kept as it is."""
    if lam < lmin:
        lam = lmin
    return lam


class GMRES:
    """nsolver's GMRES (nsolver/gmres.cpp:19-100): Arnoldi on Q with the (n+1) x n Hessenberg H, least-squares
    solution in the Krylov space; the Gram-Schmidt step is `ortho` (by default the FP64 GPU step)."""

    def __init__(self, b: np.ndarray, nmax: int, min_condition: float, ortho=None, rng=None):
        self.M, self.nmax, self.cond = b.shape[0], int(nmax), float(min_condition)
        self.bnorm = float(np.linalg.norm(b))
        self.Q = [b / self.bnorm]
        self.H = np.zeros((self.nmax + 1, self.nmax))
        self.n = 0
        self.residual = 1.0
        self.x = np.zeros(self.M)
        self.ortho = ortho or orthogonalize
        self.rng = rng or np.random.default_rng(0)

    def test_vector(self) -> np.ndarray:
        return self.Q[self.n]

    def iterate(self, Aq: np.ndarray):
        n = self.n
        V = np.array(self.Q)
        w, h = self.ortho(V, Aq)
        retries = 0
        while abs(h[-1]) < self.cond and retries < 10:   # benign breakdown: a random vector instead
            retries += 1
            w, h2 = self.ortho(V, self.rng.standard_normal(self.M))
            h = np.concatenate([h[:-1], [h2[-1]]])
        self.H[: n + 1, n] = h[:-1]
        self.H[n + 1, n] = h[-1]
        self.Q.append(w)
        Hn = self.H[: n + 2, : n + 1]
        bk = np.zeros(n + 2)
        bk[0] = self.bnorm
        y = np.linalg.lstsq(Hn, bk, rcond=None)[0]
        self.residual = float(np.linalg.norm(Hn @ y - bk) / self.bnorm)
        self.x = np.array(self.Q[: n + 1]).T @ y
        self.n = n + 1


def _numpy_ortho(V: np.ndarray, w: np.ndarray):
    """Gram-Schmidt twice on the host (the same step as cfgpu_orthogonalize), for host-only use."""
    w = np.array(w, dtype=np.float64, copy=True)
    k = V.shape[0] if V.size else 0
    h = np.zeros(k + 1)
    for _ in range(2):
        if k:
            p = V @ w
            w -= V.T @ p
            h[:k] += p
    h[k] = float(np.linalg.norm(w))
    if h[k] > 0:
        w /= h[k]
    return w, h


def hookstep_search(dsi, x0: np.ndarray, flags: NewtonSearchFlags | None = None, ortho=None, log=None):
    """Newton-Krylov-hookstep search for G(x) = 0: NewtonAlgorithm::solve with the GMRES solver and hookstep
    optimization (nsolver/newtonalgorithm.cpp:334-789, 895-1346).  dsi provides eval(x), jacobian(x, dx, Gx,
    epsDx, centdiff) and, when dsi.xrelative, xdiff(x) (the phase condition: the Krylov rows of the shift
    unknown are (dx, du0/dx), newtonalgorithm.cpp:540-550, 612-620).

    Returns (x, G(x), info) with info = {"gx": [L2Norm(G) per Newton step], "fcount": f evaluations,
    "converged": bool, "reason": why the search stopped, "gmres": [Krylov dimension per step],
    "delta": [trust radius per step]}.
    """
    f = flags or NewtonSearchFlags()
    say = log or (lambda *a: None)
    xrel = bool(getattr(dsi, "xrelative", False))
    ncut = 1 if xrel else 0  # the field part of x: norms and trust region exclude the shift unknown

    def fnorm(v):
        return float(np.linalg.norm(v[: v.shape[0] - ncut] if ncut else v))

    x = np.array(x0, dtype=np.float64, copy=True)
    E = dsi.xdiff(x0) if xrel else None
    Gx = dsi.eval(x)
    nunk = x.shape[0]
    nsolver = min(nunk, f.Nsolver)
    delta = f.delta
    info = {"gx": [], "fcount": 1, "converged": False, "reason": "", "gmres": [], "delta": []}

    def jac(xx, dx, G, cd):
        info["fcount"] += 2 if cd else 1
        return dsi.jacobian(xx, dx, G, f.epsDx, cd)

    def ev(xx):
        info["fcount"] += 1
        return dsi.eval(xx)

    for nnewton in range(f.Nnewton + 1):
        rx = 0.5 * float(Gx @ Gx)
        gx = float(np.linalg.norm(Gx))
        info["gx"].append(gx)
        info["delta"].append(delta)
        say("Newton %d: L2Norm(G(x)) = %.6e, delta = %.3e" % (nnewton, gx, delta))
        if gx < f.epsSearch:
            info["converged"], info["reason"] = True, "L2Norm(G(x)) < epsSearch"
            return x, Gx, info
        if nnewton == f.Nnewton:
            info["reason"] = "maximum number of Newton steps"
            return x, Gx, info
        # GMRES for DG(x) dx = -G(x)
        b = -Gx
        gm = GMRES(b, nsolver, f.epsKrylov, ortho=ortho)
        dxN = None
        for n in range(nsolver):
            q = gm.test_vector()
            Lq = jac(x, q, Gx, f.centdiff)
            if xrel:
                Lq = Lq.copy()
                Lq[-1] = float(q @ E)
            gm.iterate(Lq)
            if gm.residual < f.epsSolver or (n == nsolver - 1 and gm.residual < f.epsSolverF):
                dxN = gm.x
                break
        info["gmres"].append(gm.n)
        if dxN is None:
            info["reason"] = "GMRES failed to converge"
            return x, Gx, info
        # hookstep (newtonalgorithm.cpp:895-1346)
        Nk = gm.n
        Hn = gm.H[: Nk + 1, :Nk]
        Q = np.array(gm.Q[: Nk + 1]).T  # M x (Nk+1)
        U, D, Vt = np.linalg.svd(Hn, full_matrices=False)
        bh = U.T @ (Q.T @ b)
        have_backup = False
        backup = None
        delta_max_local = f.deltaMax
        while True:
            dxn = fnorm(dxN)
            if dxn <= delta:
                newton_inside = True
                dxH = dxN
            else:
                newton_inside = False
                mu = 0.0
                found = False
                for hs in range(f.Nhook):
                    dxHmu = bh / (D + mu)
                    nd = float(np.linalg.norm(dxHmu))
                    phi = nd * nd - delta * delta
                    if nd < delta or ((1 - f.deltaFuzz) * delta < nd < (1 + f.deltaFuzz) * delta):
                        found = True
                        break
                    if hs < f.Nhook - 1:
                        dphi = -2.0 * float(np.sum(bh * bh / (D + mu) ** 3))
                        mu -= (nd / delta) * (phi / dphi)
                if not found:
                    info["reason"] = "no hookstep of radius delta"
                    return x, Gx, info
                dxH = Q[:, :Nk] @ (Vt.T @ dxHmu)
            GxH = ev(x + dxH)
            rH = 0.5 * float(GxH @ GxH)
            d_rH = rH - rx
            DG = jac(x, dxH, Gx, f.centdiff)
            d_rL = float(Gx @ DG)
            if rx + d_rL >= rx:
                if f.centdiff:
                    info["reason"] = "local linear model of the residual is increasing"
                    return x, Gx, info
                DG = jac(x, dxH, Gx, True)
                d_rL = float(Gx @ DG)
                if rx + d_rL >= rx:
                    info["reason"] = "local linear model of the residual is increasing (centred differences)"
                    return x, Gx, info
            rQ = 0.5 * float(np.linalg.norm(DG + Gx) ** 2)
            d_rQ = rQ - rx
            dxHnorm = fnorm(dxH)
            drdx = d_rL / dxHnorm
            lam = -0.5 * drdx * dxHnorm / (rH - rx - drdx * dxHnorm)
            req = f.improvReq * drdx * dxHnorm
            ok = f.improvOk * d_rQ
            good = f.improvGood * d_rQ
            acc = abs(f.improvAcc * d_rQ)
            if d_rH > req:
                imp = "unacceptable"
            elif d_rH > ok:
                imp = "poor"
            elif d_rH < ok and d_rH > good:
                imp = "ok"
            else:
                imp = "good"
                if d_rQ - acc <= d_rH <= d_rQ + acc:
                    imp = "accurate"
                elif d_rH < d_rL:
                    imp = "negacurve"
            recompute = False
            if imp == "unacceptable":
                if have_backup:
                    dxH, GxH, rH, dxHnorm, delta = backup
                else:
                    delta_max_local = delta
                    lam = _adjust_lambda(lam, f.lambdaMin, f.lambdaRequiredReduction)
                    delta = _adjust_delta(delta, lam, f.deltaMin, f.deltaMax)
                    if delta < f.deltaMin:
                        delta = f.deltaMin
                        info["reason"] = "trust region below deltaMin"
                        return x, Gx, info
                    if delta > dxHnorm:
                        delta = 0.5 * dxHnorm
                        if delta < f.deltaMin:
                            info["reason"] = "trust region below deltaMin"
                            return x, Gx, info
                    recompute = True
            elif imp in ("negacurve", "accurate") and not (have_backup and backup[2] < rH) and not newton_inside \
                    and not delta >= f.deltaMax:
                new_delta = _adjust_delta(delta, f.lambdaMax, f.deltaMin, f.deltaMax)
                if new_delta < delta_max_local:
                    have_backup = True
                    backup = (dxH, GxH, rH, dxHnorm, delta)
                    recompute = True
                    delta = new_delta
                else:
                    delta = delta_max_local
            else:
                if have_backup and backup[2] < rH:
                    dxH, GxH, rH, dxHnorm, delta = backup
                elif have_backup:
                    pass
                elif imp == "poor":
                    lam = _adjust_lambda(lam, f.lambdaMin, 1.0)
                    delta = _adjust_delta(delta, lam, f.deltaMin, f.deltaMax)
                    if delta < f.deltaMin:
                        info["reason"] = "trust region below deltaMin"
                        return x, Gx, info
                elif imp == "ok" or newton_inside or delta >= f.deltaMax:
                    pass
                else:
                    lam = _adjust_lambda(lam, 1.0, f.lambdaMax)
                    delta = _adjust_delta(delta, lam, f.deltaMin, f.deltaMax)
            if not recompute:
                break
        x = x + dxH
        Gx = GxH
    return x, Gx, info


class Arnoldi:
    """nsolver's Arnoldi iteration (nsolver/arnoldi.cpp:24-133): eigenvalue estimates of a linear operator A
    known only through products A q.  Q holds the orthonormal Krylov basis, H the (n+1) x n Hessenberg matrix;
    ew() are the eigenvalues of H_n sorted by decreasing modulus (sort_by_abs, cfbasics/cfbasics.h:1261-1276),
    ev() the Ritz vectors Q_n W, rd() the residual estimates |q_n| |W[n-1, j]| (arnoldi.cpp:108-127; q_n is a
    unit vector, so the estimate is |W[n-1, j]|, as in the reference).  The Gram-Schmidt step is `ortho` (the
    FP64 GPU step by default; the reference's single modified Gram-Schmidt pass differs from it by rounding).
    A breakdown (|w| below min_condition), where the reference exits, raises RuntimeError; an iteration past
    niter, where the reference writes past H, raises ValueError."""

    def __init__(self, b: np.ndarray, niter: int, min_condition: float = 1e-13, ortho=None):
        b = np.asarray(b, dtype=np.float64)
        self.M, self.niter, self.cond = b.shape[0], int(niter), float(min_condition)
        self.H = np.zeros((self.niter + 1, self.niter))
        self.Q = [b / np.linalg.norm(b)]
        self.n = 0
        self.ortho = ortho or orthogonalize
        self._eig = None

    def test_vector(self) -> np.ndarray:
        return self.Q[self.n]

    def iterate(self, Aq: np.ndarray):
        n = self.n
        if n == self.niter:
            raise ValueError("Arnoldi: all %d iterations done" % self.niter)
        w, h = self.ortho(np.array(self.Q), np.asarray(Aq, dtype=np.float64))
        if abs(h[-1]) < self.cond:
            raise RuntimeError("Arnoldi breakdown: |w| = %.3e below %.3e after %d iterations" % (abs(h[-1]), self.cond,
                                                                                               n))
        self.H[: n + 1, n] = h[:-1]
        self.H[n + 1, n] = h[-1]
        self.Q.append(w)
        self.n = n + 1
        self._eig = None

    def _eigencalc(self):
        if self._eig is None:
            n = self.n
            lam, W = np.linalg.eig(self.H[:n, :n])
            order = np.argsort(-np.abs(lam), kind="stable")
            lam, W = lam[order], W[:, order]
            V = np.array(self.Q[:n]).T @ W
            rd = np.linalg.norm(self.Q[n]) * np.abs(W[n - 1, :])
            self._eig = (lam, V, rd)
        return self._eig

    def ew(self) -> np.ndarray:
        return self._eigencalc()[0]

    def ev(self) -> np.ndarray:
        return self._eigencalc()[1]

    def rd(self) -> np.ndarray:
        return self._eigencalc()[2]


class Lanczos(Arnoldi):
    """nsolver's Lanczos iteration for normal (self-adjoint) operators (nsolver/lanczos.cpp:23-93): the
    tridiagonal T with T[n, n] = <q_n, A q_n - T[n-1, n] q_{n-1}> and T[n+1, n] = T[n, n+1] = |w|, w
    reorthogonalised against every earlier q (the reference's full modified Gram-Schmidt pass); ew() from the
    symmetric eigenproblem of T_n, sorted by decreasing modulus; ev() and rd() as for Arnoldi."""

    def iterate(self, Aq: np.ndarray):
        n = self.n
        if n == self.niter:
            raise ValueError("Lanczos: all %d iterations done" % self.niter)
        v = np.array(Aq, dtype=np.float64, copy=True)
        if n != 0:
            v -= self.H[n - 1, n] * self.Q[n - 1]
        self.H[n, n] = float(self.Q[n] @ v)
        for q in self.Q:
            v -= float(q @ v) * q
        vnorm = float(np.linalg.norm(v))
        if vnorm < self.cond:
            raise RuntimeError("Lanczos breakdown: |w| = %.3e below %.3e after %d iterations" % (vnorm, self.cond, n))
        if n + 1 < self.niter:
            self.H[n, n + 1] = vnorm
        self.H[n + 1, n] = vnorm
        self.Q.append(v / vnorm)
        self.n = n + 1
        self._eig = None

    def _eigencalc(self):
        if self._eig is None:
            n = self.n
            lam, W = np.linalg.eigh(self.H[:n, :n])
            order = np.argsort(-np.abs(lam), kind="stable")
            lam, W = lam[order].astype(complex), W[:, order]
            V = (np.array(self.Q[:n]).T @ W).astype(complex)
            rd = np.linalg.norm(self.Q[n]) * np.abs(W[n - 1, :])
            self._eig = (lam, V, rd)
        return self._eig


@dataclass
class EigenvalsFlags:
    """EigenvalsFlags (nsolver/eigenvals.h:16-44, the defaults of nsolver/eigenvals.cpp:46-59): Arnoldi
    iterations, stable eigenvalues kept beyond the unstable and marginal ones (or exactly Nstable when
    fixedNs), Krylov breakdown threshold, centred differences, the margin below which Re(lambda) counts as
    stable; isnormal selects the Lanczos iteration (self-adjoint operators)."""
    isnormal: bool = False
    Narnoldi: int = 100
    Nstable: int = 5
    fixedNs: bool = False
    EPS_kry: float = 1e-10
    centdiff: bool = False
    EPS_stab: float = 1e-6


def eigenvals(dsi, x: np.ndarray, dx: np.ndarray, T: float, eps: float = 1e-7,
              flags: EigenvalsFlags | None = None, ortho=None, log=None) -> dict:
    """Eigenvals::solve (nsolver/eigenvals.cpp:118-279), the Arnoldi iteration behind findeigenvals: the
    eigenvalues Lambda of the linearised map Df^T at a fixed point x of f^T (G(x) = 0), from products
        A q = (f^T(x + eps q) - f^T(x)) / eps,
    which DSI::Jacobian gives with Gx = -eps q (G = f^T(u) - u, so G(x + eps q) + eps q = f^T(x + eps q) - x);
    with centred differences Jacobian returns (f^T(x + eps q/2) - f^T(x - eps q/2)) / eps - q and q is added
    back.  Each iteration is one f^T evaluation (two with centdiff, submitted together to the server when dsi
    has one) and depends on the previous one, so the iteration itself is sequential.  Growth rates
    lambda = log(Lambda) / T.

    Returns {"Lambda", "lambda", "residual" (the last iteration's), "Nnonstable", "Nsave", "eigvecs": the
    saved eigenfunctions as vectors (a complex pair as its real and imaginary parts, eigenvals.cpp:250-271),
    "history": per iteration the leading Lambda and their residuals, "fcount"}."""
    f = flags or EigenvalsFlags()
    say = log or (lambda *a: None)
    dx = np.asarray(dx, dtype=np.float64)
    dx = dx / np.linalg.norm(dx)
    arn = Lanczos(dx, f.Narnoldi, f.EPS_kry) if f.isnormal else Arnoldi(dx, f.Narnoldi, f.EPS_kry, ortho=ortho)
    history = []
    fcount0 = getattr(dsi, "fcount", 0)
    for n in range(f.Narnoldi):
        q = arn.test_vector()
        Gx = -eps * q
        Aq = dsi.jacobian(x, q, Gx, eps, f.centdiff)
        if f.centdiff:
            Aq = Aq + q
        arn.iterate(Aq)
        Lam, rd = arn.ew(), arn.rd()
        lam = np.log(Lam.astype(complex)) / T
        nns = int(np.sum(lam.real >= -f.EPS_stab))
        nsave = min(Lam.shape[0], f.Nstable if f.fixedNs else nns + f.Nstable)
        history.append({"Lambda": Lam[:nsave].copy(), "residual": rd[:nsave].copy()})
        say("Arnoldi %d: |Lambda_0| = %.12g, residual %.3e" % (n, abs(Lam[0]), rd[0]))
    Lam, V, rd = arn.ew(), arn.ev(), arn.rd()
    lam = np.log(Lam.astype(complex)) / T
    nns = int(np.sum(lam.real >= -f.EPS_stab))
    nsave = min(Lam.shape[0], f.Nstable if f.fixedNs else nns + f.Nstable)
    eigvecs = []
    j = 0
    while j < nsave:
        if Lam[j].imag == 0.0:
            eigvecs.append((j, V[:, j].real.copy()))
        elif j + 1 < Lam.shape[0]:
            eigvecs.append((j, V[:, j].real.copy()))
            eigvecs.append((j + 1, V[:, j].imag.copy()))
            j += 1
        j += 1
    return {"Lambda": Lam, "lambda": lam, "residual": rd, "Nnonstable": nns, "Nsave": nsave, "eigvecs": eigvecs,
            "history": history, "fcount": getattr(dsi, "fcount", 0) - fcount0}
