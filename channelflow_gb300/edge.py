"""Edge-tracking bisection (programs/edgetracking.cpp) on the host, with the candidate trajectories of a
bisection round classified together in one batched GPU ensemble.

Restated from the reference:

* attractor (edgetracking.cpp:836-893): a field is turbulent if its cross-flow energy Ecf and/or its L2 norm
  are at or above the high thresholds, laminar if at or below the low ones (only the criteria whose two
  thresholds are both set count), and laminar as well once Ecf has not grown for more than tMaxDecay time
  units; both at once is an error, neither is "no attractor";
* Ecf (diffops.cpp:3931): the squared L2 norm of v and w, integrated over y without normalisation;
* RelL2Diff (edgetracking.cpp:110): L2Dist(u1, u2) / (L2Norm(u1) + L2Norm(u2));
* Bisection (edgetracking.cpp:363-455): with one trajectory per round the midpoint of uL and uH replaces
  whichever of them has its attractor; with n > 1, candidates (1 - alpha) uL + alpha uH at alpha = j / (n + 1)
  are tried for j = 1, 2, ... until one is not laminar (j <= n + 11), uH becomes that candidate and, for
  j >= 3, uL the candidate of j - 2.  The reference integrates the candidates one after the other; here the
  n of a round run as one ensemble (the next block of candidates only if all were laminar), which gives
  the same choice because the trajectories are independent;
* CalcAttractor (edgetracking.cpp:767-818): integrate one time unit at a time until the attractor is known
  (after tMin) or tMax is reached.  The ensemble shares one dt, so each candidate runs at the flags' fixed dt
  where the reference adapts each trajectory's dt to its CFL number.

* ChooseNewLH (edgetracking.cpp:659-715), AdvanceLH (:472-657) with its equilibrium and periodic-orbit
  checks on Ecf, and the tracking loop EdgeStateTracking (:284-327); uL and uH advance as the two slots of one
  ensemble.

Not restated: the output files (energies, saved fields, continuation) and the symmetry projection of the
initial field.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .fields import l2norm

LAMINAR, TURBULENT = "laminar", "turbulent"


@dataclass
class AttractorFlags:
    """AttractorFlags (edgetracking.cpp:34-47; options at :126-137, all thresholds 0 = unset by default)."""
    EcfH: float = 0.0
    EcfL: float = 0.0
    L2H: float = 0.0
    L2L: float = 0.0
    normToHeight: bool = False
    tMaxDecay: int = 0


@dataclass
class BisectionFlags:
    """The EdgetrackingFlags the bisection reads (edgetracking.cpp:138-148): separation at which it stops,
    candidate trajectories per round, time window of the attractor classification."""
    epsilonBisection: float = 1e-6
    nBisectTrajectories: int = 1
    tMinAttractor: int = 0
    tMaxAttractor: int = 10000


def ecf(u: np.ndarray, Nx: int, Nz: int, a: float = -1.0, b: float = 1.0) -> float:
    """Ecf(u) (diffops.cpp:3931): L2Norm_uvw(u, v and w only)^2, the y integral not normalised."""
    return (b - a) * l2norm(u[1:3], Nx, Nz) ** 2


def attractor(l2: float, ecf_value: float, flags: AttractorFlags, height: float = 2.0, tdecay: int = 0,
              last_ecf: float = 0.0):
    """attractor(u, tDecay, lastEcf, flags) (edgetracking.cpp:836-893) from the field's L2 norm and Ecf.
    Returns (LAMINAR, TURBULENT or None, the updated decay counter)."""
    use_ecf = flags.EcfH > 1e-12 and flags.EcfL > 1e-12
    use_l2 = flags.L2H > 1e-12 and flags.L2L > 1e-12
    if not (use_ecf or use_l2):
        raise ValueError("no valid attractor thresholds: set EcfH and EcfL, or L2H and L2L")
    laminar = turbulent = True
    if use_ecf:
        val = ecf_value / height if flags.normToHeight else ecf_value
        if val < flags.EcfH:
            turbulent = False
        if val > flags.EcfL:
            laminar = False
    if use_l2:
        val = l2 / np.sqrt(height) if flags.normToHeight else l2
        if val < flags.L2H:
            turbulent = False
        if val > flags.L2L:
            laminar = False
    if flags.tMaxDecay > 0:
        tdecay = tdecay + 1 if ecf_value <= last_ecf else 0
        if tdecay > flags.tMaxDecay:
            laminar = True
    if laminar and turbulent:
        raise RuntimeError("field classified as both laminar and turbulent")
    return (TURBULENT if turbulent else LAMINAR if laminar else None), tdecay


def rel_l2_diff(u1: np.ndarray, u2: np.ndarray, Nx: int, Nz: int) -> float:
    """RelL2Diff (edgetracking.cpp:110)."""
    return l2norm(u1 - u2, Nx, Nz) / (l2norm(u1, Nx, Nz) + l2norm(u2, Nx, Nz))


class EnsembleClassifier:
    """CalcAttractor for many candidate fields at once: the fields are the slots of one ensemble (one set of
    kernel launches per step for all of them), advanced `steps_per_unit` steps per time unit; after each unit
    the per-slot L2 norms come from one device pass, Ecf from the slots' downloaded v and w (only when the
    flags use it).  `make_ensemble(n)` builds the ensemble (default: channelflow_gb300.Ensemble over `grid`
    and `flags` in `precision`); anything with set_field, advance_resident, l2norm, get_field and close
    serves."""

    def __init__(self, grid, flags, aflags: AttractorFlags, steps_per_unit: int, tmin: int = 0,
                 tmax: int = 10000, precision: str = "fp64", make_ensemble=None):
        self.grid, self.flags, self.aflags = grid, flags, aflags
        self.steps_per_unit, self.tmin, self.tmax = int(steps_per_unit), int(tmin), int(tmax)
        self.precision = precision
        self.make_ensemble = make_ensemble
        self.units = 0           # time units integrated, summed over calls (one per ensemble step block)

    def _ensemble(self, n):
        if self.make_ensemble is not None:
            return self.make_ensemble(n)
        from .dns import Ensemble
        return Ensemble(self.grid, self.flags, n, precision=self.precision)

    def __call__(self, fields) -> list:
        g, af = self.grid, self.aflags
        n = len(fields)
        need_ecf = (af.EcfH > 1e-12 and af.EcfL > 1e-12) or af.tMaxDecay > 0
        height = g.b - g.a
        ens = self._ensemble(n)
        try:
            for i, u in enumerate(fields):
                ens.set_field(i, np.ascontiguousarray(u))
            res = [None] * n
            tdecay = [0] * n
            u = np.zeros_like(fields[0])
            q = np.zeros((1,) + fields[0].shape[1:], dtype=fields[0].dtype)

            def ecfs(which):
                out = {}
                for i in which:
                    ens.get_field(i, u, q)
                    out[i] = ecf(u, g.Nx, g.Nz, g.a, g.b)
                return out

            last = ecfs(range(n)) if need_ecf else {}
            t = 0
            while t < self.tmax and any(r is None for r in res):
                t += 1
                ens.advance_resident(self.steps_per_unit)
                self.units += 1
                l2 = ens.l2norm(0)
                open_ = [i for i in range(n) if res[i] is None]
                cur = ecfs(open_) if need_ecf else {}
                if t > self.tmin:
                    for i in open_:
                        res[i], tdecay[i] = attractor(float(l2[i]), cur.get(i, 0.0), af, height, tdecay[i],
                                                      last.get(i, 0.0))
                last.update(cur)
            return res
        finally:
            ens.close()


def bisection(uL: np.ndarray, uH: np.ndarray, classify, Nx: int, Nz: int, flags: BisectionFlags | None = None,
              log=None):
    """Bisection (edgetracking.cpp:363-455) between uL (known to end laminar) and uH (known to end turbulent)
    until RelL2Diff(uL, uH) <= epsilonBisection.  classify(list of fields) -> list of LAMINAR / TURBULENT /
    None (e.g. an EnsembleClassifier).  Returns (uL, uH, info) with info = {"lambdaL", "lambdaH" (the
    one-trajectory interpolation parameters, as the reference reports them), "rounds", "l2diff": RelL2Diff
    after each round, "candidates": trajectories classified}."""
    f = flags or BisectionFlags()
    say = log or (lambda *a: None)
    uL, uH = np.array(uL, copy=True), np.array(uH, copy=True)
    lamL, lamH = 0.0, 1.0
    l2d = rel_l2_diff(uL, uH, Nx, Nz)
    ntraj = int(f.nBisectTrajectories)
    info = {"rounds": 0, "l2diff": [], "candidates": 0}
    while l2d > f.epsilonBisection:
        info["rounds"] += 1
        if ntraj == 1:
            lam = 0.5 * (lamL + lamH)
            uT = 0.5 * (uH + uL)
            a = classify([uT])[0]
            info["candidates"] += 1
            if a == TURBULENT:
                lamH, uH = lam, uT
            elif a == LAMINAR:
                lamL, uL = lam, uT
            else:
                raise RuntimeError("bisection: a candidate reached no attractor within the time window")
        else:
            step = 1.0 / (ntraj + 1)
            found = None
            for j0, j1 in ((1, ntraj), (ntraj + 1, ntraj + 11)):
                js = list(range(j0, j1 + 1))
                cands = [(1.0 - j * step) * uL + (j * step) * uH for j in js]
                results = classify(cands)
                info["candidates"] += len(cands)
                for j, c, r in zip(js, cands, results):
                    if r != LAMINAR:      # the reference's loop stops at the first candidate that is not laminar
                        found = (j, c, r)
                        break
                if found:
                    break
            if found is None:
                raise RuntimeError("bisection: no candidate became turbulent")
            j, uT, _ = found
            if j >= 3:
                aL = (j - 2) * step
                uL = (1.0 - aL) * uL + aL * uH
            uH = uT
        l2d = rel_l2_diff(uL, uH, Nx, Nz)
        info["l2diff"].append(l2d)
        say("bisection round %d: RelL2Diff %.3e" % (info["rounds"], l2d))
    info["lambdaL"], info["lambdaH"] = lamL, lamH
    return uL, uH, info


@dataclass
class TrackingFlags(BisectionFlags):
    """The remaining EdgetrackingFlags of the tracking loop (edgetracking.cpp:138-160, defaults :724-748):
    separation at which advancing stops, lambda step of the choice of new fields, whether to keep integrating
    after separation to verify the attractors, whether the new fields are built from uL instead of uH, and
    the equilibrium / periodic-orbit detection on the cross-flow energy."""
    epsilonAdvance: float = 1e-4
    lambdaStep: float = 0.1
    verifyLH: bool = False
    keepUL: bool = False
    checkConvergence: bool = False


def choose_new_lh(u0: np.ndarray, classify, lamL: float, lamH: float, lambda_step: float):
    """ChooseNewLH (edgetracking.cpp:659-715): raise lambdaH until lambdaH u0 is turbulent (a laminar one
    becomes the new lambdaL), then lower lambdaL until lambdaL u0 is laminar (a turbulent one becomes the new
    lambdaH; with lambdaL == lambdaH on entry lambdaL starts one step lower).  Returns (lambdaL, lambdaH)."""
    if lamL > lamH:
        raise ValueError("lambdaL > lambdaH")
    equal = lamH == lamL
    aH, aL = None, None
    while aH != TURBULENT:
        aH = classify([lamH * u0])[0]
        if aH == LAMINAR:
            lamL = lamH
            lamH += lambda_step
            aL = LAMINAR
        elif aH is None:
            raise RuntimeError("choose_new_lh: lambda = %g reaches no attractor" % lamH)
    while aL != LAMINAR:
        if equal:
            lamL -= lambda_step
            equal = False
        aL = classify([lamL * u0])[0]
        if aL == TURBULENT:
            lamH = lamL
            lamL -= lambda_step
        elif aL is None:
            raise RuntimeError("choose_new_lh: lambda = %g reaches no attractor" % lamL)
    return lamL, lamH


class EnsemblePair:
    """uL and uH as the two slots of one ensemble (one set of launches for both), advanced one time unit
    (`steps_per_unit` steps) per call; `make_ensemble(2)` as for EnsembleClassifier."""

    def __init__(self, grid, flags, uL, uH, steps_per_unit: int, precision: str = "fp64", make_ensemble=None):
        if make_ensemble is None:
            from .dns import Ensemble

            def make_ensemble(n):
                return Ensemble(grid, flags, n, precision=precision)
        self.ens = make_ensemble(2)
        self.steps = int(steps_per_unit)
        self.ens.set_field(0, np.ascontiguousarray(uL))
        self.ens.set_field(1, np.ascontiguousarray(uH))
        self._u = np.zeros_like(uL)
        self._q = np.zeros((1,) + uL.shape[1:], dtype=uL.dtype)

    def advance(self):
        self.ens.advance_resident(self.steps)

    def fields(self):
        out = []
        for i in (0, 1):
            self.ens.get_field(i, self._u, self._q)
            out.append(self._u.copy())
        return out[0], out[1]

    def close(self):
        self.ens.close()


def advance_lh(uL0: np.ndarray, uH0: np.ndarray, t: int, T: float, grid, flags: TrackingFlags,
               aflags: AttractorFlags, pair, cd: dict | None = None, log=None):
    """AdvanceLH (edgetracking.cpp:472-657): advance uL and uH (pair, e.g. an EnsemblePair started from them)
    one time unit at a time while RelL2Diff(uL, uH) < epsilonAdvance, counting t; uL0, uH0 follow the last
    states on the edge.  After the separation, with verifyLH, keep going (at most tMaxAttractor units) until uL
    is laminar and uH turbulent; without it, either reaching its attractor is an error (the thresholds are
    wrong), as is reaching it within two units.  With checkConvergence, a constant Ecf over 100 units (a
    relative equilibrium) or repeating Ecf extrema (a periodic orbit) ends the call early (the states of that
    unit are not kept, as in the reference).  Returns (uL0, uH0, t, finished: t == T or converged, cd), cd the
    extrema record kept across calls."""
    say = log or (lambda *a: None)
    g = grid
    cd = cd if cd is not None else {"EcfMax": [0.0] * 4, "EcfMin": [0.0] * 4, "tEcfMin": [0] * 4}

    def push(a, b):
        a[:] = a[1:] + [b]

    t0 = t
    t2 = float(t)
    t_att = flags.tMaxAttractor + t
    turbulent = laminar = False
    on_edge = True
    ecf0 = ecf1 = ecf2 = 0.0
    ring = [0.0] * 100
    try:
        while (not turbulent or not laminar) and t <= T and (on_edge or (flags.verifyLH and t2 <= t_att)):
            t2 += 1
            pair.advance()
            fL, fH = pair.fields()
            if on_edge:
                l2d = rel_l2_diff(fL, fH, g.Nx, g.Nz)
                if l2d < flags.epsilonAdvance:
                    t += 1
                    ecf2, ecf1, ecf0 = ecf1, ecf0, ecf(fH, g.Nx, g.Nz, g.a, g.b)
                    ecf_min = ecf1 < ecf2 and ecf1 <= ecf0
                    ecf_max = ecf1 > ecf2 and ecf1 >= ecf0
                    if flags.checkConvergence:
                        ring[t % len(ring)] = ecf0
                        if all(e >= 1e-16 and abs(e - ring[0]) / ring[0] <= flags.epsilonBisection for e in ring):
                            say("Ecf is constant: converged to a (relative) equilibrium")
                            return uL0, uH0, t, True, cd
                        if ecf_max:
                            push(cd["EcfMax"], ecf0)
                        if ecf_min:
                            push(cd["EcfMin"], ecf0)
                            push(cd["tEcfMin"], t)
                            mx, mn, tm = cd["EcfMax"], cd["EcfMin"], cd["tEcfMin"]
                            eps = 1e-3
                            if (abs(mx[0] - mx[2]) / ecf0 < eps and abs(mx[1] - mx[3]) / ecf0 < eps and
                                    abs(mn[0] - mn[2]) / ecf0 < eps and abs(mn[1] - mn[3]) / ecf0 < eps and
                                    abs((tm[3] - tm[1]) - (tm[2] - tm[0])) < 5):
                                say("converged to a periodic orbit")
                                return uL0, uH0, t, True, cd
                    uL0, uH0 = fL, fH
                else:
                    on_edge = False
                    say("fields separated by %.3e at t = %d" % (l2d, t))
            if not turbulent and attractor(l2norm(fH, g.Nx, g.Nz), ecf(fH, g.Nx, g.Nz, g.a, g.b), aflags,
                                           g.b - g.a)[0] == TURBULENT:
                turbulent = True
                if not flags.verifyLH:
                    raise RuntimeError("uH is turbulent, check the thresholds")
                if t2 - t0 <= 2:
                    raise RuntimeError("uH turbulent within two time units, check the thresholds")
            if not laminar and attractor(l2norm(fL, g.Nx, g.Nz), ecf(fL, g.Nx, g.Nz, g.a, g.b), aflags,
                                         g.b - g.a)[0] == LAMINAR:
                laminar = True
                if not flags.verifyLH:
                    raise RuntimeError("uL is laminar, check the thresholds")
                if t2 - t0 <= 2:
                    raise RuntimeError("uL laminar within two time units, check the thresholds")
    finally:
        pair.close()
    if flags.verifyLH and not laminar:
        raise RuntimeError("verifyLH: uL does not become laminar")
    if flags.verifyLH and not turbulent:
        raise RuntimeError("verifyLH: uH does not become turbulent")
    return uL0, uH0, t, t == T, cd


def edge_tracking(uL: np.ndarray, uH: np.ndarray, t0: int, T: float, grid, flags: TrackingFlags,
                  aflags: AttractorFlags, classify, make_pair, log=None) -> dict:
    """EdgeStateTracking (edgetracking.cpp:284-327): bisect uL, uH to the edge, advance them along it until
    they separate, choose new fields lambda u from the last edge state (uH, or uL with keepUL), repeat until
    t > T.  make_pair(uL, uH) builds the pair advance_lh integrates (e.g. an EnsemblePair).  As in the
    reference, whose `finished` is redeclared inside the loop, a converged or finished advance only skips the
    choice of new fields; the loop ends with t > T.  Returns {"uL", "uH", "t", "bisections": [(t, rounds)],
    "lambdas": [(lambdaL, lambdaH)]}."""
    say = log or (lambda *a: None)
    g = grid
    t = int(t0)
    out = {"bisections": [], "lambdas": []}
    cd = None
    while t <= T:
        uL, uH, info = bisection(uL, uH, classify, g.Nx, g.Nz, flags, log)
        out["bisections"].append((t, info["rounds"]))
        uL, uH, t, finished, cd = advance_lh(uL, uH, t, T, g, flags, aflags, make_pair(uL, uH), cd, log)
        if not finished:
            u = uL if flags.keepUL else uH
            lamL, lamH = choose_new_lh(u, classify, 1.0, 1.0, flags.lambdaStep)
            out["lambdas"].append((lamL, lamH))
            say("t = %d: new lambdaL %.4g, lambdaH %.4g" % (t, lamL, lamH))
            uL, uH = lamL * u, lamH * u
    out.update(uL=uL, uH=uH, t=t)
    return out
