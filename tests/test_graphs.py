"""Steady-state steps replayed from CUDA graphs give the same fields as eager launches.

The graph of a step records the same kernels with the same arguments as the
eager step of the same buffer-rotation state, so the results are identical
bit for bit; reset_dt must drop the graphs (its tables and coefficients change).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _run(g, fl, graphs, nsteps, precision, reset_at=None):
    from channelflow_gb300 import DNS
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=8, norm=0.2))
    q = np.zeros((1,) + u.shape[1:], complex)
    d = DNS(u, to_cgrid(g), to_cflags(fl), precision=precision)
    d.set_graphs(graphs)
    d.set_fields(u, q)
    if reset_at is None:
        d.advance_resident(nsteps)
    else:
        d.advance_resident(reset_at)
        d.reset_dt(fl.dt * 0.5)
        d.advance_resident(nsteps - reset_at)
    d.get_fields(u, q)
    launches = d.kernel_launches()
    d.close()
    return u, q, launches


@pytest.mark.parametrize("scheme", [O.SBDF3, O.SBDF4, O.CNAB2, O.SMRK2, O.CNRK2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_is_bit_identical(scheme, precision):
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0,
                    timestepping=scheme)
    ue, qe, le = _run(g, fl, False, 17, precision)
    ug, qg, lg = _run(g, fl, True, 17, precision)
    assert np.array_equal(ue, ug) and np.array_equal(qe, qg)
    assert le == lg   # graph replays count the kernels they launch


def test_graphs_dropped_by_reset_dt():
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    ue, qe, _ = _run(g, fl, False, 20, "fp64", reset_at=9)
    ug, qg, _ = _run(g, fl, True, 20, "fp64", reset_at=9)
    assert np.array_equal(ue, ug) and np.array_equal(qe, qg)


def test_autotuned_block_shapes_do_not_change_results():
    """The FFT passes' block shapes (autotuned above ~200k plane-columns) leave every column's arithmetic
    unchanged: tuned and default runs are identical."""
    from channelflow_gb300 import _lib as L
    g = O.Grid(128, 65, 128, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.01, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    lib = L.load()
    try:
        lib.cfgpu_set_autotune(0)
        ud, qd, _ = _run(g, fl, True, 4, "mixed")
        lib.cfgpu_set_autotune(1)
        ut, qt, _ = _run(g, fl, True, 4, "mixed")
    finally:
        lib.cfgpu_set_autotune(1)
    assert np.array_equal(ud, ut) and np.array_equal(qd, qt)
