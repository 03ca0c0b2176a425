""".ff binary FlowField I/O (host code in libcfgpu.so) against the oracle's restatement of the format.

FlowField::binarySave (channelflow/flowfield.cpp:2642-2723) and the binary
branch of FlowField(filebase) (:216-356); big-endian primitives
(cfbasics/cfbasics.h:368-470).  No GPU needed.
"""

import os
import struct

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, solved_mask, to_cgrid


@pytest.fixture(scope="module", autouse=True)
def built():
    from channelflow_gb300 import build
    build.build()


def _field(g, seed, Nd=3, aliased_zero=True):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz)) + 1j * rng.standard_normal((Nd, g.Ny, g.Nx, g.Mz))
    if aliased_zero:
        # zero the modes a padded file omits: |kx| > 2(Nx/6) or kz > Nz/3
        Nxd, Nzd = 2 * (g.Nx // 6), 2 * (g.Nz // 3) + 1
        kx = np.array([g.kx(m) for m in range(g.Nx)])
        keep = (np.abs(kx)[:, None] <= Nxd) & (np.arange(g.Mz)[None, :] <= Nzd // 2)
        u = u * keep[None, None]
    return np.ascontiguousarray(u)


@pytest.mark.parametrize("padded", [True, False])
@pytest.mark.parametrize("dims", [(32, 33, 32), (24, 17, 18), (4, 9, 4)])
def test_ff_roundtrip_matches_oracle(tmp_path, padded, dims):
    from channelflow_gb300 import ffio
    g = O.Grid(dims[0], dims[1], dims[2], *COUETTE_BOX)
    u = _field(g, seed=sum(dims), aliased_zero=padded)
    p1, p2 = str(tmp_path / "lib.ff"), str(tmp_path / "oracle.ff")
    ffio.save(p1, u, to_cgrid(g), padded=padded)
    O.ff_write(p2, u, g, padded)
    assert open(p1, "rb").read() == open(p2, "rb").read()      # byte-identical files
    v, g2, pad2 = ffio.load(p2)
    assert pad2 == padded and (g2.Nx, g2.Ny, g2.Nz) == dims and g2.Lx == g.Lx and g2.Lz == g.Lz
    assert np.array_equal(v, u)
    w, _, _ = O.ff_read(p1)
    assert np.array_equal(w, u)


def test_ff_header_bytes(tmp_path):
    from channelflow_gb300 import ffio
    g = O.Grid(12, 9, 12, 2.0, 3.0, -1.0, 1.0)
    p = str(tmp_path / "h.ff")
    ffio.save(p, _field(g, 1), to_cgrid(g), padded=True)
    b = open(p, "rb").read()
    assert b[:63] == struct.pack(">7i", 2, 0, 9, 12, 9, 12, 3) + b"SS" + struct.pack(">4d", 2.0, 3.0, -1.0, 1.0) + b"1"
    Nxd, Nzd = 2 * (12 // 6), 2 * (12 // 3) + 1
    assert len(b) == 63 + 3 * 9 * (2 * Nxd + 1) * (Nzd // 2 + 1) * 16


def test_ff_padded_file_zero_fills_omitted_modes(tmp_path):
    from channelflow_gb300 import ffio
    g = O.Grid(32, 17, 32, *COUETTE_BOX)
    u = _field(g, 7, aliased_zero=False)
    p = str(tmp_path / "p.ff")
    O.ff_write(p, u, g, True)
    v, _, _ = ffio.load(p)
    Nxd, Nzd = 2 * (g.Nx // 6), 2 * (g.Nz // 3) + 1
    kx = np.array([g.kx(m) for m in range(g.Nx)])
    keep = (np.abs(kx)[:, None] <= Nxd) & (np.arange(g.Mz)[None, :] <= Nzd // 2)
    assert solved_mask(g)[~keep].sum() == 0        # every solved mode is stored
    assert np.array_equal(v[:, :, keep], u[:, :, keep])
    assert not np.any(v[:, :, ~keep])


def test_ff_errors(tmp_path):
    from channelflow_gb300 import ffio
    from channelflow_gb300._lib import CfgpuError
    with pytest.raises(CfgpuError):
        ffio.load(str(tmp_path / "missing.ff"))
    g = O.Grid(8, 9, 8, *COUETTE_BOX)
    p = str(tmp_path / "t.ff")
    O.ff_write(p, _field(g, 3), g, False)
    b = open(p, "rb").read()
    open(p, "wb").write(b[: len(b) // 2])
    with pytest.raises(CfgpuError, match="truncated"):
        ffio.load(p)
    phys = bytearray(b)
    phys[28:30] = b"PP"
    open(p, "wb").write(bytes(phys))
    with pytest.raises(CfgpuError, match="spectral"):
        ffio.load(p)
    assert os.path.exists(p)
