"""Host FlowField buffers read and written by the GPU directly (pageable memory through the host page
tables) give the same fields as the staged path (host gathers + pinned copies): data movement only, so
the results are identical bit for bit."""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, to_cflags, to_cgrid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _run(direct, g, fl, fields, steps, precision):
    from channelflow_gb300 import DNS, Ensemble
    from channelflow_gb300.dns import set_host_access
    set_host_access(direct)
    try:
        out = []
        u = fields[0].copy()
        q = np.zeros((1,) + u.shape[1:], complex)
        d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision=precision)
        used = d.host_access()
        for _ in range(3):
            d.advance(u, q, steps)          # the e2e path: host buffers in, host buffers out
        out += [u.copy(), q.copy()]
        d.close()
        ens = Ensemble(to_cgrid(g), to_cflags(fl), len(fields), precision=precision)
        U = np.ascontiguousarray(np.stack(fields))
        Q = np.zeros((len(fields), 1) + fields[0].shape[1:], complex)
        ens.advance(U, Q, steps)
        out += [U.copy(), Q.copy()]
        ens.set_field(1, fields[0], q)      # one slot from host buffers
        ens.advance_resident(steps)
        u1, q1 = np.zeros_like(fields[0]), np.zeros_like(q)
        ens.get_field(1, u1, q1)
        out += [u1, q1]
        ens.close()
        return used, out
    finally:
        set_host_access(True)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_direct_host_access_equals_staged(precision):
    g = O.Grid(18, 17, 12, *COUETTE_BOX)   # NKz odd: 16-byte alignment of rows varies
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    fields = [np.ascontiguousarray(O.random_divfree_field(g, seed=900 + k, norm=0.2)) for k in range(3)]
    used_d, a = _run(True, g, fl, fields, 4, precision)
    used_s, b = _run(False, g, fl, fields, 4, precision)
    assert not used_s
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    if not used_d:
        pytest.skip("device kernels cannot access pageable host memory: only the staged path ran")


def test_direct_host_access_unaligned_buffers():
    """Buffers that are not 16-byte aligned (a view one double into a larger array) take the scalar path."""
    from channelflow_gb300 import DNS
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=5, norm=0.2))
    raw = np.zeros(u0.size * 2 + 1)
    uv = raw[1:].view(np.complex128).reshape(u0.shape)   # 8-byte offset
    uv[...] = u0
    q = np.zeros((1,) + u0.shape[1:], complex)
    d = DNS(u0.copy(), to_cgrid(g), to_cflags(fl))
    d.set_fields(uv, q)
    out, qo = np.zeros_like(u0), np.zeros_like(q)
    d.get_fields(out, qo)
    m = np.abs(out) > 0
    assert np.array_equal(out[m], u0[m])
    d.close()


def test_pinned_host_buffers_equal_pageable():
    """Page-locked FlowField buffers (cfgpu_host_register) go through the same kernels: identical results; the
    registration is undone on leaving the block, and a second registration of the same buffer is refused."""
    from channelflow_gb300 import DNS
    from channelflow_gb300 import _lib as L
    from channelflow_gb300.dns import PinnedHost
    g = O.Grid(18, 17, 12, *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=77, norm=0.2))
    outs = []
    for pinned in (True, False):
        u, q = u0.copy(), np.zeros((1,) + u0.shape[1:], complex)
        d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision="mixed")
        if pinned:
            with PinnedHost(u, q):
                with pytest.raises(L.CfgpuError):
                    with PinnedHost(u):
                        pass
                for _ in range(3):
                    d.advance(u, q, 4)
        else:
            for _ in range(3):
                d.advance(u, q, 4)
        outs.append((u, q))
        d.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    # unregistered on exit: registering again works
    with PinnedHost(outs[0][0]):
        pass
