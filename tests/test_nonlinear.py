"""The nonlinear term alone: cfgpu_dns_nonlinear against the oracle's navierstokesNL + zeroPaddedModes.

navierstokesNL (channelflow/nse.cpp:12-91): base flow and Vsuck added to the
(0,0) mode, rotational / convection / skew-symmetric / divergence forms
(diffops.cpp:2229-2880), linearizedNL (diffops.cpp:3288-3361), the rotation
term (nse.cpp:62-78); NSE::nonlinear zeroes the padded modes (nse.cpp:383-391).
Tolerances: FP64 path 1e-12 relative L2 of f; mixed path (FP32 transforms and
products) 1e-5.
"""

import numpy as np
import pytest

from oracle import cf_oracle as O
from tests.helpers import COUETTE_BOX, POISEUILLE_BOX, rel_l2, to_cflags, to_cgrid

CASES = [
    ("couette_rotational", (16, 17, 16), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Rotational)),
    ("couette_convection", (18, 17, 12), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Convection)),
    ("poiseuille_skew", (24, 33, 24), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3, nonlinearity=O.SkewSymmetric)),
    ("poiseuille_divergence_vsuck", (16, 25, 16), POISEUILLE_BOX,
     dict(baseflow=O.SuctionBase, Vsuck=0.01, nonlinearity=O.Divergence)),
    ("couette_linearized", (16, 17, 16), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.LinearAboutProfile)),
    ("couette_rotation", (16, 17, 16), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Rotational, rotation=0.3)),
    # x and z lengths with prime factors 7 and 11 (direct-DFT stages of the generic FFT)
    ("couette_rotational_radix7_11", (28, 17, 22), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, nonlinearity=O.Rotational)),
    ("poiseuille_skew_radix13_7", (26, 17, 14), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3, nonlinearity=O.SkewSymmetric)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
@pytest.mark.parametrize("name,dims,box,fkw", CASES, ids=[c[0] for c in CASES])
def test_nonlinear_matches_oracle(name, dims, box, fkw, precision, tol):
    from channelflow_gb300 import DNS, build
    build.build()
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, **fkw)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=77, norm=0.2))
    q = np.zeros((1,) + u.shape[1:], complex)
    ref, _ = O.NSE(g, fl, None, u).nonlinear(u)
    d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision=precision)
    f = d.nonlinear(u)
    assert rel_l2(f, ref, g) <= tol, rel_l2(f, ref, g)
    # the DNS's own state is untouched
    u2, q2 = np.zeros_like(u), np.zeros_like(q)
    d.get_fields(u2, q2)
    m = np.abs(u2) > 0
    assert np.array_equal(u2[m], u[m])
    d.close()


FUSED_GRIDS = [(32, 33, 32), (48, 25, 64), (128, 33, 128), (96, 17, 48), (64, 21, 96)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,tol_pair", [("fp64", 1e-12, 1e-13), ("mixed", 1e-5, 3e-6)])
@pytest.mark.parametrize("dims", FUSED_GRIDS, ids=["%dx%dx%d" % d for d in FUSED_GRIDS])
def test_fused_xz_pass_matches_oracle_and_three_kernel_path(dims, precision, tol, tol_pair):
    """The rotational form's fused x/z kernel (one thread-block cluster per y-plane) against the oracle and
    against the three-kernel path (x inverse, z pass, x forward) on the same field."""
    from channelflow_gb300 import DNS, build
    from channelflow_gb300 import _lib as L
    build.build()
    lib = L.load()
    g = O.Grid(dims[0], dims[1], dims[2], *POISEUILLE_BOX)
    fl = O.DNSFlags(nu=1 / 2000, dt=0.01, baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=sum(dims), norm=0.3, zero_mean_u=True))
    ref, _ = O.NSE(g, fl, None, u).nonlinear(u)
    out = {}
    try:
        # 2: the fused kernel wherever the grid allows (1 would keep the three kernels where they time faster)
        for fused in (2, 0):
            L.check(lib.cfgpu_set_fused_xz(fused))
            d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision=precision)
            out[fused] = d.nonlinear(u)
            d.close()
    finally:
        L.check(lib.cfgpu_set_fused_xz(1))
    assert rel_l2(out[2], ref, g) <= tol
    assert rel_l2(out[2], out[0], g) <= tol_pair


CHEB_FFT_CASES = [
    ("poiseuille_33", (16, 33, 16), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3)),
    ("couette_49", (24, 49, 18), COUETTE_BOX, dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)),
    ("suction_65", (16, 65, 16), POISEUILLE_BOX, dict(baseflow=O.SuctionBase, Vsuck=0.01)),
    ("poiseuille_97", (32, 97, 32), POISEUILLE_BOX,
     dict(baseflow=O.LaminarBase, constraint=O.BulkVelocity, Ubulk=2 / 3)),
    ("couette_rotation_129", (16, 129, 12), COUETTE_BOX,
     dict(baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0, rotation=0.3)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,tol_pair", [("fp64", 1e-12, 1e-13), ("mixed", 1e-5, 3e-6)])
@pytest.mark.parametrize("name,dims,box,fkw", CHEB_FFT_CASES, ids=[c[0] for c in CHEB_FFT_CASES])
def test_cheb_fft_matches_oracle_and_matrix_path(name, dims, box, fkw, precision, tol, tol_pair):
    """The rotational form with its Chebyshev transforms through the FFT (spectral curl, inverse and forward
    DCT-I as one complex FFT of length Ny - 1 per mode) against the oracle and against the dense matrix
    products on the same field."""
    from channelflow_gb300 import DNS, build
    from channelflow_gb300 import _lib as L
    build.build()
    lib = L.load()
    g = O.Grid(dims[0], dims[1], dims[2], *box)
    fl = O.DNSFlags(nu=1 / 1000, dt=0.01, nonlinearity=O.Rotational, **fkw)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=dims[1], norm=0.3))
    ref, _ = O.NSE(g, fl, None, u).nonlinear(u)
    out = {}
    try:
        for mode in (2, 0):
            L.check(lib.cfgpu_set_cheb_fft(mode))
            d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision=precision)
            used = ctypes_int()
            L.check(lib.cfgpu_dns_cheb_fft(d._h, used))
            assert used.value == (1 if mode == 2 else 0)
            out[mode] = d.nonlinear(u)
            d.close()
    finally:
        L.check(lib.cfgpu_set_cheb_fft(1))
    assert rel_l2(out[2], ref, g) <= tol, rel_l2(out[2], ref, g)
    assert rel_l2(out[2], out[0], g) <= tol_pair, rel_l2(out[2], out[0], g)


@pytest.mark.gpu
def test_cheb_fft_not_used_where_the_length_does_not_factor():
    """Ny - 1 = 34 has the factor 17: the FFT form is unavailable and the DNS keeps the matrix products."""
    from channelflow_gb300 import DNS, build
    from channelflow_gb300 import _lib as L
    build.build()
    lib = L.load()
    g = O.Grid(16, 35, 16, *POISEUILLE_BOX)
    fl = O.DNSFlags(nu=1 / 1000, dt=0.01, baseflow=O.LaminarBase)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=5, norm=0.1))
    L.check(lib.cfgpu_set_cheb_fft(2))
    try:
        d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision="fp64")
    finally:
        L.check(lib.cfgpu_set_cheb_fft(1))
    used = ctypes_int()
    L.check(lib.cfgpu_dns_cheb_fft(d._h, used))
    assert used.value == 0
    d.close()


def ctypes_int():
    import ctypes
    return ctypes.c_int(-1)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,tol_pair", [("mixed", 1e-5, 3e-6)])
@pytest.mark.parametrize("dims", FUSED_GRIDS, ids=["%dx%dx%d" % d for d in FUSED_GRIDS])
def test_register_zpass_matches_generic_and_oracle(dims, precision, tol, tol_pair):
    """The mixed path's three-kernel x/z path with the register-FFT z pass (csrc/z_reg.cu) against the same
    path with the generic Stockham z pass and against the oracle's rotationalNL."""
    from channelflow_gb300 import DNS, build
    from channelflow_gb300 import _lib as L
    build.build()
    lib = L.load()
    g = O.Grid(dims[0], dims[1], dims[2], *COUETTE_BOX)
    fl = O.DNSFlags(nu=1 / 400, dt=0.02, baseflow=O.LaminarBase, ulowerwall=-1.0, uupperwall=1.0)
    u = np.ascontiguousarray(O.random_divfree_field(g, seed=3 * sum(dims), norm=0.3))
    ref, _ = O.NSE(g, fl, None, u).nonlinear(u)
    out = {}
    try:
        L.check(lib.cfgpu_set_fused_xz(0))
        for reg in (1, 0):
            L.check(lib.cfgpu_set_register_zpass(reg))
            d = DNS(u.copy(), to_cgrid(g), to_cflags(fl), precision=precision)
            out[reg] = d.nonlinear(u)
            d.close()
    finally:
        L.check(lib.cfgpu_set_register_zpass(1))
        L.check(lib.cfgpu_set_fused_xz(1))
    assert rel_l2(out[1], ref, g) <= tol
    assert rel_l2(out[1], out[0], g) <= tol_pair
