"""TimeStep and f^T(u) (cfDSI's f, channelflow/cfdsi.cpp:705-775) against the oracle.

The TimeStep arithmetic (channelflow/dnsflags.cpp:752-965) runs in the
library's host code, so its tests need no GPU; f^T(u) itself steps on the GPU.
"""

import math

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, rel_l2, to_cflags, to_cgrid


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _timestep_cases(seed, n):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        dtmin = float(rng.choice([0.0, 1e-3, 0.01]))
        dtmax = float(rng.choice([0.05, 0.2, 1.0]))
        dt = float(rng.uniform(max(dtmin, 1e-3), dtmax))
        dT = float(rng.uniform(max(dtmin, dt * 0.5), 4.0))
        lo = float(rng.uniform(0.0, 0.6))
        hi = float(lo + rng.uniform(0.0, 0.6))
        yield dict(dt=dt, dtmin=dtmin, dtmax=dtmax, dT=dT, CFLmin=lo, CFLmax=hi, variable=bool(rng.integers(0, 2)))


def _pair(p):
    from channelflow_gb300.dsi import TimeStep
    return TimeStep(**p), O.TimeStep(p["dt"], p["dtmin"], p["dtmax"], p["dT"], p["CFLmin"], p["CFLmax"], p["variable"])


def test_timestep_adjust_for_T_matches_oracle():
    rng = np.random.default_rng(3)
    for p in _timestep_cases(1, 300):
        mine, ref = _pair(p)
        T = float(rng.choice([rng.uniform(0.01, 50.0), 0.0, p["dT"] * 3]))
        n, N, dt = mine.adjust_for_T(T)
        ref.adjust_for_T(T)
        assert (n, N) == (ref.n, ref.N)
        if T == 0:
            assert mine.dt == 0 and mine.dT == 0
            continue
        assert mine.dt == ref.dt and mine.dT == ref.dT     # same arithmetic, bit for bit
        assert dt == ref.value()


def test_timestep_adjust_matches_oracle():
    rng = np.random.default_rng(4)
    changed = 0
    for p in _timestep_cases(2, 300):
        mine, ref = _pair(p)
        for cfl in rng.uniform(0.0, 1.5, size=4):
            a = mine.adjust(float(cfl))
            b = ref.adjust(float(cfl))
            assert a == b and mine.dt == ref.dt
            changed += a
    assert changed > 50


def test_timestep_rejects_bad_parameters():
    from channelflow_gb300._lib import CfgpuError
    from channelflow_gb300.dsi import TimeStep
    for bad in (dict(dt=0.3, dtmax=0.2), dict(dt=0.01, dtmin=0.02), dict(CFLmin=0.7, CFLmax=0.6),
                dict(dT=0.0005, dtmin=0.001, dt=0.001)):
        with pytest.raises(CfgpuError):
            TimeStep(**bad).adjust_for_T(1.0)


def test_ft_nonpositive_T_needs_no_steps():
    """T < 0 returns (1+|T|) u and T == 0 returns u (cfdsi.cpp:718-728), before any DNS is built."""
    from channelflow_gb300.dsi import TimeStep, ft
    g = O.Grid(8, 9, 8, *COUETTE_BOX)
    u = O.random_divfree_field(g, seed=1, norm=0.1)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    fu, _ = ft(u, to_cgrid(g), to_cflags(fl), TimeStep(), -0.5)
    assert np.array_equal(fu, u * 1.5)
    fu, _ = ft(u, to_cgrid(g), to_cflags(fl), TimeStep(), 0.0)
    assert np.array_equal(fu, u)


FT_CASES = [
    # scheme, initial dt, CFL range: both runs adjust dt after the probe step and at least once mid-run
    ("sbdf3_var", O.SBDF3, 0.02, 0.3, 0.5, True),
    ("sbdf3_var_shrink", O.SBDF3, 0.05, 0.2, 0.3, True),
    ("cnab2_var", O.CNAB2, 0.02, 0.3, 0.5, True),
    ("smrk2_var", O.SMRK2, 0.02, 0.3, 0.5, True),
    ("cnrk2_var", O.CNRK2, 0.02, 0.3, 0.5, True),
    ("sbdf3_fixed", O.SBDF3, 0.04, 0.3, 0.5, False),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,scheme,dt,lo,hi,variable", FT_CASES, ids=[c[0] for c in FT_CASES])
def test_ft_matches_oracle(name, scheme, dt, lo, hi, variable):
    from channelflow_gb300.dsi import TimeStep, ft
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=dt, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, timestepping=scheme)
    u0 = O.random_divfree_field(g, seed=5, norm=0.3)
    T = 2.0
    ref_u, ref_cfl = O.ft(u0, g, fl, O.TimeStep(dt, 0.001, 0.2, 0.25, lo, hi, variable), T)
    fu, cfl = ft(np.ascontiguousarray(u0), to_cgrid(g), to_cflags(fl),
                 TimeStep(dt, 0.001, 0.2, 0.25, lo, hi, variable), T)
    assert rel_l2(fu, ref_u, g) <= 1e-10
    assert abs(cfl - ref_cfl) <= 1e-10 * ref_cfl
    assert math.isfinite(cfl)
