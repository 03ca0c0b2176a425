"""FlowField handles on the GPU (cfgpu_field_*) and device-to-device field exchange with a DNS.

upload -> download reproduces the 2/3-dealiased modes and zeroes the rest (zeroPaddedModes,
flowfield.cpp:2235-2255); a DNS loaded from device fields and read back into device fields gives the same
results as the host-buffer path (to round-off: a slot of a two-field batch against a lone DNS).
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, solved_mask, to_cflags, to_cgrid


@pytest.mark.gpu
@pytest.mark.parametrize("Nd", [1, 3])
def test_device_field_roundtrip(Nd):
    from channelflow_gb300 import build
    from channelflow_gb300.dns import DeviceField
    build.build()
    g = O.Grid(18, 17, 12, *COUETTE_BOX)
    rng = np.random.default_rng(Nd)
    u = rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz)) + 1j * rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz))
    f = DeviceField(to_cgrid(g), Nd)
    f.upload(np.ascontiguousarray(u))
    out = f.download()
    m = solved_mask(g)
    assert np.array_equal(out[:, :, m], u[:, :, m])
    assert not np.any(out[:, :, ~m])
    f.close()


@pytest.mark.gpu
def test_dns_fields_through_device_handles():
    from channelflow_gb300 import DNS, Ensemble, build
    from channelflow_gb300.dns import DeviceField, get_fields_device, set_fields_device
    build.build()
    g = O.Grid(16, 17, 16, *COUETTE_BOX)
    cg = to_cgrid(g)
    fl = to_cflags(O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0))
    u0 = np.ascontiguousarray(O.random_divfree_field(g, seed=3, norm=0.2))
    q0 = np.zeros((1,) + u0.shape[1:], complex)
    ref = DNS(u0.copy(), cg, fl)
    ur, qr = u0.copy(), q0.copy()
    ref.advance(ur, qr, 7)
    fu, fq = DeviceField(cg, 3), DeviceField(cg, 1)
    fu.upload(u0)
    fq.upload(q0)
    ens = Ensemble(cg, fl, 2)
    set_fields_device(ens, fu, fq, slot=1)
    ens.advance_resident(7)
    get_fields_device(ens, fu, fq, slot=1)
    out = fu.download()
    assert np.abs(out - ur).max() <= 1e-14 * np.abs(ur).max()   # batched slot vs a lone DNS
    with pytest.raises(Exception):
        set_fields_device(ens, fq, None, slot=0)    # a 1-component field as velocity
    ens.close()
    ref.close()
