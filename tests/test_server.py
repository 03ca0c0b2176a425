"""Request server: continuous batching of mixed-grid, mixed-Reynolds requests.

Every served result must equal the same request run alone through a
single-field DNS (1e-13 relative L2, FP64 path), whatever else was in the
batch and whenever the request joined it.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, rel_l2, to_cflags, to_cgrid


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _requests(rng, n):
    grids = [O.Grid(16, 17, 16, *COUETTE_BOX), O.Grid(24, 33, 24, *COUETTE_BOX), O.Grid(16, 25, 24, *COUETTE_BOX)]
    out = []
    for k in range(n):
        g = grids[k % len(grids)]
        re = float(rng.uniform(300, 2000))
        if rng.random() < 0.5:
            p = dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
            zm = False
        else:
            p = dict(baseflow=O.LaminarBase, ulowerwall=0.0, uupperwall=0.0, constraint=O.BulkVelocity, Ubulk=2 / 3)
            zm = True
        fl = O.DNSFlags(nu=1 / re, dt=0.02, **p)   # SBDF3 with SMRK2 start-up: cfDSI's default scheme
        u = np.ascontiguousarray(O.random_divfree_field(g, seed=1000 + k, norm=float(rng.uniform(0.05, 0.3)),
                                                        zero_mean_u=zm))
        out.append((g, fl, int(rng.integers(3, 40)), u))
    return out


def _alone(g, fl, n, u):
    from channelflow_gb300 import DNS
    u = u.copy()
    q = np.zeros((1,) + u.shape[1:], complex)
    d = DNS(u, to_cgrid(g), to_cflags(fl))
    d.advance(u, q, n)
    d.close()
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("max_bytes", [8 << 30, 40 << 20], ids=["roomy", "tight_memory"])
def test_served_results_equal_alone(max_bytes):
    from channelflow_gb300.server import DONE, Server
    rng = np.random.default_rng(5)
    reqs = _requests(rng, 14)
    srv = Server(max_bytes=max_bytes, slots=3)
    ids = [srv.submit(to_cgrid(g), to_cflags(fl), n, u) for (g, fl, n, u) in reqs[:9]]
    for _ in range(3):
        srv.pump(4)
    ids += [srv.submit(to_cgrid(g), to_cflags(fl), n, u) for (g, fl, n, u) in reqs[9:]]   # arrive while running
    srv.run(4)
    st = srv.stats()
    assert st["queued"] == 0 and st["running"] == 0
    for rid, (g, fl, n, u) in zip(ids, reqs):
        status, res, times = srv.poll(rid)
        assert status == DONE
        assert times[0] <= times[1] <= times[2]
        ref = _alone(g, fl, n, u)
        assert rel_l2(res, ref, g) <= 1e-13, (rid, rel_l2(res, ref, g))
    srv.close()


def test_server_argument_errors():
    """Host-side checks (no GPU needed)."""
    from channelflow_gb300._lib import CfgpuError
    from channelflow_gb300.server import Server
    with pytest.raises(CfgpuError):
        Server(max_bytes=0)
    srv = Server(max_bytes=1 << 20, slots=2)
    g = O.Grid(8, 9, 8, *COUETTE_BOX)
    u = np.zeros((3, 9, 8, 5), complex)
    with pytest.raises(CfgpuError, match="ArbitraryBase"):
        srv.submit(to_cgrid(g), to_cflags(O.DNSFlags(baseflow=O.ArbitraryBase)), 5, u)
    rid = srv.submit(to_cgrid(g), to_cflags(O.DNSFlags()), 0, u)   # zero steps: done at once
    status, res, _ = srv.poll(rid)
    assert status == 2 and np.array_equal(res, u)
    with pytest.raises(CfgpuError):
        srv.poll(rid + 100)
    srv.release(rid)
    srv.close()


@pytest.mark.gpu
def test_served_ft_equals_ft_alone():
    """f^T(u) requests with variable TimeSteps (CFL probe, dt changes every dT) served in shared
    ensembles equal cfDSI-style f^T(u) evaluated alone (cfgpu_ft)."""
    from channelflow_gb300.dsi import TimeStep, ft
    from channelflow_gb300.server import DONE, Server
    rng = np.random.default_rng(17)
    reqs = _requests(rng, 10)
    srv = Server(slots=3)
    cases = []
    for k, (g, fl, n, u) in enumerate(reqs):
        ts = TimeStep(dt=0.02, dtmin=0.001, dtmax=0.05, dT=0.1, CFLmin=0.15 + 0.05 * (k % 3), CFLmax=0.3,
                      variable=k % 4 != 3)
        T = 0.2 * (1 + k % 5)
        cases.append((g, fl, ts, T, u, srv.submit_ft(to_cgrid(g), to_cflags(fl), ts, T, u)))
    srv.run(3)
    for g, fl, ts, T, u, rid in cases:
        status, res, _ = srv.poll(rid)
        assert status == DONE
        ref, _ = ft(u, to_cgrid(g), to_cflags(fl), TimeStep(**{k: getattr(ts, k) for k in ts.__dataclass_fields__}),
                    T)
        assert rel_l2(res, ref, g) <= 1e-13, (rid, rel_l2(res, ref, g))
    srv.close()
