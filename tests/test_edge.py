"""Edge-tracking bisection (programs/edgetracking.cpp:363-455, 766-893) on the host.

The attractor classification is checked against the reference's rules; the bisection and the batched
classifier run on a toy bistable system behind the ensemble interface (set_field, advance_resident, l2norm,
get_field, close): a field grows towards a turbulent amplitude when its L2 norm is above an edge value and
decays otherwise, so the bisection must end on the edge.  CPU only.
"""

import math

import numpy as np
import pytest

from channelflow_gb300.edge import (LAMINAR, TURBULENT, AttractorFlags, BisectionFlags, EnsembleClassifier,
                                    attractor, bisection, ecf, rel_l2_diff)
from channelflow_gb300.fields import l2norm

NX, NY, NZ = 4, 9, 4
EDGE = 0.1


class ToyGrid:
    Nx, Ny, Nz, a, b = NX, NY, NZ, -1.0, 1.0


class ToyEnsemble:
    """Slots of fields whose norm grows (above EDGE, up to 1) or decays (below) by a factor per step."""

    def __init__(self, n):
        self.u = [None] * n
        self.closed = False
        self.steps = 0

    def set_field(self, i, u, q=None):
        self.u[i] = np.array(u, copy=True)

    def advance_resident(self, nsteps):
        self.steps += nsteps
        for i, u in enumerate(self.u):
            for _ in range(nsteps):
                a = l2norm(u, NX, NZ)
                u = u * (min(1.2, 1.0 / a) if a > EDGE else 0.8)
            self.u[i] = u

    def l2norm(self, field=0):
        return np.array([l2norm(u, NX, NZ) for u in self.u])

    def get_field(self, i, u, q):
        u[...] = self.u[i]
        q[...] = 0.0

    def close(self):
        self.closed = True


def unit_field(seed):
    rng = np.random.default_rng(seed)
    u = np.zeros((3, NY, NX, NZ // 2 + 1), complex)
    u[:, :, 1, 1] = rng.standard_normal((3, NY)) + 1j * rng.standard_normal((3, NY))
    return u / l2norm(u, NX, NZ)


def test_attractor_rules():
    fl = AttractorFlags(L2H=0.5, L2L=0.01)
    assert attractor(0.6, 0.0, fl)[0] == TURBULENT
    assert attractor(0.005, 0.0, fl)[0] == LAMINAR
    assert attractor(0.1, 0.0, fl)[0] is None
    # both criteria must agree for a verdict (edgetracking.cpp:859-878)
    fl2 = AttractorFlags(L2H=0.5, L2L=0.01, EcfH=1e-2, EcfL=1e-5)
    assert attractor(0.6, 1e-3, fl2)[0] is None
    assert attractor(0.6, 2e-2, fl2)[0] == TURBULENT
    # normalised to the box height: L2 by sqrt(h), Ecf by h
    fl3 = AttractorFlags(L2H=0.5, L2L=0.01, normToHeight=True)
    assert attractor(0.6, 0.0, fl3, height=2.0)[0] is None            # 0.6 / sqrt(2) < 0.5
    # monotone Ecf decay for more than tMaxDecay units counts as laminar
    fl4 = AttractorFlags(L2H=0.5, L2L=0.01, tMaxDecay=2)
    td = 0
    out = []
    for e_last, e in ((1.0, 0.9), (0.9, 0.8), (0.8, 0.7)):
        r, td = attractor(0.1, e, fl4, tdecay=td, last_ecf=e_last)
        out.append(r)
    assert out == [None, None, LAMINAR]
    r, td = attractor(0.1, 0.95, fl4, tdecay=td, last_ecf=0.7)           # growth resets the counter
    assert r is None and td == 0
    with pytest.raises(ValueError):
        attractor(0.1, 0.0, AttractorFlags())
    with pytest.raises(RuntimeError):
        attractor(0.3, 0.0, AttractorFlags(L2H=0.2, L2L=0.4))


def test_ecf_is_the_unnormalised_cross_flow_energy():
    u = unit_field(3)
    u[0] *= 3.0
    e = ecf(u, NX, NZ)
    assert math.isclose(e, 2.0 * l2norm(u[1:], NX, NZ) ** 2, rel_tol=1e-14)
    v = u.copy()
    v[0] = 0
    assert math.isclose(ecf(v, NX, NZ), e, rel_tol=1e-14)


def test_classifier_runs_all_candidates_as_one_ensemble():
    made = []

    def make(n):
        made.append(ToyEnsemble(n))
        return made[-1]

    cls = EnsembleClassifier(ToyGrid(), None, AttractorFlags(L2H=0.5, L2L=0.01), steps_per_unit=2, tmax=200,
                             make_ensemble=make)
    e = unit_field(1)
    res = cls([0.05 * e, 0.3 * e, 0.099 * e, 0.101 * e])
    assert res == [LAMINAR, TURBULENT, LAMINAR, TURBULENT]
    assert len(made) == 1 and made[0].closed
    # tMax reached with the field still between the thresholds: no attractor
    res = EnsembleClassifier(ToyGrid(), None, AttractorFlags(L2H=0.5, L2L=0.01), steps_per_unit=1, tmax=3,
                             make_ensemble=ToyEnsemble)([0.09 * e])
    assert res == [None]


@pytest.mark.parametrize("ntraj", [1, 4])
def test_bisection_ends_on_the_edge(ntraj):
    e1, e2 = unit_field(11), unit_field(12)
    uL, uH = 0.05 * e1, 0.3 * e2
    cls = EnsembleClassifier(ToyGrid(), None, AttractorFlags(L2H=0.5, L2L=0.01), steps_per_unit=1, tmax=500,
                             make_ensemble=ToyEnsemble)
    fl = BisectionFlags(epsilonBisection=1e-6, nBisectTrajectories=ntraj)
    L, H, info = bisection(uL, uH, cls, NX, NZ, fl)
    assert rel_l2_diff(L, H, NX, NZ) <= 1e-6
    assert l2norm(L, NX, NZ) <= EDGE <= l2norm(H, NX, NZ)
    assert abs(l2norm(H, NX, NZ) - EDGE) < 1e-6
    assert info["l2diff"] == sorted(info["l2diff"], reverse=True)
    if ntraj == 1:
        assert info["candidates"] == info["rounds"]
        assert 0.0 < info["lambdaL"] < info["lambdaH"] < 1.0
    else:
        # a round narrows the interval to two candidate spacings, 2 / (n + 1) of it, against 1/2 one at a time
        base = bisection(uL, uH, cls, NX, NZ, BisectionFlags(epsilonBisection=1e-6))[2]["rounds"]
        assert info["rounds"] < base
        l2d0 = rel_l2_diff(uL, uH, NX, NZ)
        assert info["rounds"] <= math.ceil(math.log(1e-6 / l2d0) / math.log(2.0 / (ntraj + 1))) + 2


def test_bisection_without_a_turbulent_candidate_fails():
    e = unit_field(5)
    cls = EnsembleClassifier(ToyGrid(), None, AttractorFlags(L2H=0.5, L2L=0.01), steps_per_unit=1, tmax=500,
                             make_ensemble=ToyEnsemble)
    with pytest.raises(RuntimeError):
        bisection(0.01 * e, 0.02 * e, cls, NX, NZ, BisectionFlags(nBisectTrajectories=3))


class SlowEdgeEnsemble(ToyEnsemble):
    """Norm a -> EDGE + G (a - EDGE) per step, clipped to [0, 1]: the edge |u| = EDGE is unstable, so a pair
    started on it stays together for a number of steps before it separates."""
    G = 1.5

    def advance_resident(self, nsteps):
        self.steps += nsteps
        for i, u in enumerate(self.u):
            for _ in range(nsteps):
                a = l2norm(u, NX, NZ)
                a2 = min(1.0, max(0.0, EDGE + self.G * (a - EDGE)))
                u = u * (a2 / a) if a > 0 else u
            self.u[i] = u


def slow_classifier(tmax=400):
    return EnsembleClassifier(ToyGrid(), None, AttractorFlags(L2H=0.5, L2L=0.01), steps_per_unit=1, tmax=tmax,
                              make_ensemble=SlowEdgeEnsemble)


def test_choose_new_lh_brackets_the_edge():
    from channelflow_gb300.edge import choose_new_lh
    e = unit_field(21)
    # u0 on the turbulent side: lambdaH = 1 is turbulent, lambdaL steps down to the first laminar value
    lamL, lamH = choose_new_lh(0.15 * e, slow_classifier(), 1.0, 1.0, 0.1)
    assert math.isclose(lamH, 1.0 - 0.3, abs_tol=1e-12) and math.isclose(lamL, 1.0 - 0.4, abs_tol=1e-12)
    # u0 on the laminar side: lambdaH steps up until turbulent, the last laminar one becomes lambdaL
    lamL, lamH = choose_new_lh(0.07 * e, slow_classifier(), 1.0, 1.0, 0.1)
    assert math.isclose(lamL, 1.4, abs_tol=1e-12) and math.isclose(lamH, 1.5, abs_tol=1e-12)
    with pytest.raises(ValueError):
        choose_new_lh(e, slow_classifier(), 2.0, 1.0, 0.1)


def test_edge_tracking_follows_the_edge():
    from channelflow_gb300.edge import EnsemblePair, TrackingFlags, edge_tracking
    e1, e2 = unit_field(31), unit_field(32)
    fl = TrackingFlags(epsilonBisection=1e-7, epsilonAdvance=1e-4, lambdaStep=0.1)

    def make_pair(uL, uH):
        return EnsemblePair(ToyGrid(), None, uL, uH, 1, make_ensemble=SlowEdgeEnsemble)

    out = edge_tracking(0.05 * e1, 0.3 * e2, 0, 40, ToyGrid(), fl, AttractorFlags(L2H=0.5, L2L=0.01),
                        slow_classifier(), make_pair)
    assert out["t"] > 40
    assert len(out["bisections"]) >= 2 and len(out["lambdas"]) >= 1
    # every cycle ends near the edge: the last states bracket it
    assert l2norm(out["uL"], NX, NZ) < EDGE < l2norm(out["uH"], NX, NZ) + 1e-9
    assert abs(l2norm(out["uH"], NX, NZ) - EDGE) < 1e-3
    for lamL, lamH in out["lambdas"]:
        assert lamL < lamH


def test_advance_lh_detects_a_relative_equilibrium_and_misplaced_thresholds():
    from channelflow_gb300.edge import EnsemblePair, TrackingFlags, advance_lh

    class Still(SlowEdgeEnsemble):
        G = 1.05

    e = unit_field(41)
    uH = EDGE * e                       # exactly on the edge: stays there, Ecf constant
    uL = EDGE * (1 - 1e-10) * e
    fl = TrackingFlags(epsilonBisection=1e-6, epsilonAdvance=1e-4, checkConvergence=True)
    pair = EnsemblePair(ToyGrid(), None, uL, uH, 1, make_ensemble=Still)
    _, _, t, finished, _ = advance_lh(uL, uH, 0, 1000, ToyGrid(), fl, AttractorFlags(L2H=0.5, L2L=0.01), pair)
    assert finished and 100 <= t <= 101
    # thresholds that call the edge state turbulent are an error without verifyLH
    pair = EnsemblePair(ToyGrid(), None, uL, uH, 1, make_ensemble=Still)
    with pytest.raises(RuntimeError):
        advance_lh(uL, uH, 0, 1000, ToyGrid(), TrackingFlags(), AttractorFlags(L2H=0.05, L2L=0.01), pair)


def test_advance_lh_detects_a_periodic_orbit():
    """Ecf of uH oscillating with period 10 on the edge: after four maxima and four minima at equal spacing
    AdvanceLH's periodic-orbit check ends the advance (edgetracking.cpp:562-580)."""
    from channelflow_gb300.edge import EnsemblePair, TrackingFlags, advance_lh

    class Periodic(ToyEnsemble):
        def advance_resident(self, nsteps):
            self.steps += nsteps
            a = EDGE * (1.0 + 0.05 * math.sin(2 * math.pi * self.steps / 10.0))
            self.u = [u * (a / l2norm(u, NX, NZ)) for u in self.u]

    e = unit_field(51)
    fl = TrackingFlags(checkConvergence=True)
    pair = EnsemblePair(ToyGrid(), None, EDGE * e, EDGE * e, 1, make_ensemble=Periodic)
    _, _, t, finished, cd = advance_lh(EDGE * e, EDGE * e, 0, 1000, ToyGrid(), fl,
                                       AttractorFlags(L2H=0.5, L2L=0.01), pair)
    assert finished and t < 60
    assert all(x > 0 for x in cd["EcfMin"]) and cd["tEcfMin"][3] - cd["tEcfMin"][2] == 10
