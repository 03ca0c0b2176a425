"""Python mirror of the reference's DNS / DNSFlags API over the C ABI.

Mirrors channelflow's ``DNS`` (channelflow/dns.h:30-97) and ``DNSFlags``
(channelflow/dnsflags.h:81-198): same field names, same enum values, and
``DNS.advance(u, q, nsteps)`` overwrites the fields in place like
``DNS::advance(fields, nSteps)``.  Fields are NumPy complex128 arrays shaped
(Nd, Ny, Nx, Nz//2+1) -- byte-identical to the reference's serial spectral
FlowField layout.  All arithmetic runs in libcfgpu.so on the GPU; errors
raise ``CfgpuError`` (the reference exits via cferror instead).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, fields as dc_fields

import numpy as np

from . import _lib as L

# Enumerations (channelflow/dnsflags.h:24-38)
ZeroBase, LinearBase, ParabolicBase, LaminarBase, SuctionBase, ArbitraryBase = range(6)
PressureGradient, BulkVelocity = range(2)
CNFE1, CNAB2, CNRK2, SMRK2, SBDF1, SBDF2, SBDF3, SBDF4 = range(8)
Rotational, Convection, Divergence, SkewSymmetric, Alternating, Alternating_, LinearAboutProfile = range(7)
NoDealiasing, DealiasXZ, DealiasY, DealiasXYZ = range(4)


@dataclass
class DNSFlags:
    """DNSFlags members used by the time step, with the reference's defaults (dnsflags.h:84-92)."""
    nu: float = 0.0025
    dPdx: float = 0.0
    dPdz: float = 0.0
    Ubulk: float = 0.0
    Wbulk: float = 0.0
    ulowerwall: float = 0.0
    uupperwall: float = 0.0
    wlowerwall: float = 0.0
    wupperwall: float = 0.0
    Vsuck: float = 0.0
    t0: float = 0.0
    dt: float = 0.03125
    baseflow: int = LaminarBase
    constraint: int = PressureGradient
    timestepping: int = SBDF3
    initstepping: int = SMRK2
    nonlinearity: int = Rotational
    dealiasing: int = DealiasXZ
    taucorrection: bool = True
    rotation: float = 0.0

    def to_c(self) -> L.Flags:
        f = L.Flags()
        for fld in dc_fields(self):
            setattr(f, fld.name, int(getattr(self, fld.name)) if fld.name in (
                "baseflow", "constraint", "timestepping", "initstepping", "nonlinearity", "dealiasing",
                "taucorrection") else float(getattr(self, fld.name)))
        return f


@dataclass
class Grid:
    Nx: int
    Ny: int
    Nz: int
    Lx: float
    Lz: float
    a: float = -1.0
    b: float = 1.0

    def to_c(self) -> L.Grid:
        return L.Grid(self.Nx, self.Ny, self.Nz, self.Lx, self.Lz, self.a, self.b)

    @property
    def Mz(self):
        return self.Nz // 2 + 1

    def field(self, Nd: int) -> np.ndarray:
        """Zero spectral FlowField buffer (Nd, Ny, Nx, Mz) complex128."""
        return np.zeros((Nd, self.Ny, self.Nx, self.Mz), dtype=np.complex128)


def _as_field(a: np.ndarray, g: Grid, Nd: int) -> np.ndarray:
    if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"] or a.shape != (Nd, g.Ny, g.Nx, g.Mz):
        raise ValueError("field must be C-contiguous complex128 of shape %s" % ((Nd, g.Ny, g.Nx, g.Mz),))
    return a


class DNS:
    """GPU DNS with the reference's DNS interface (channelflow/dns.h:30-97).

    ``precision`` is "fp64" (plain path) or "mixed" (FP32 transforms and
    nonlinear term, FP64 state and tau solves).
    """

    def __init__(self, u: np.ndarray, grid: Grid, flags: DNSFlags, base=None, precision: str = "fp64"):
        lib = L.load()
        self.grid, self.flags = grid, flags
        _as_field(u, grid, 3)
        prec = {"fp64": L.CFGPU_FP64, "mixed": L.CFGPU_MIXED}[precision]
        h = C.c_void_p()
        Ub = Wb = None
        if base is not None:
            Ub = np.ascontiguousarray(base[0], dtype=np.float64)
            Wb = np.ascontiguousarray(base[1], dtype=np.float64)
        gc, fc = grid.to_c(), flags.to_c()
        L.check(lib.cfgpu_dns_create(C.byref(gc), C.byref(fc), L.dptr(Ub), L.dptr(Wb), L.dptr(u), prec,
                                     C.byref(h)))
        self._h = h
        self._lib = lib

    def advance(self, u: np.ndarray, q: np.ndarray, nsteps: int):
        """DNS::advance(fields, nSteps): u (3,...) and q (1,...) updated in place."""
        _as_field(u, self.grid, 3)
        _as_field(q, self.grid, 1)
        L.check(self._lib.cfgpu_dns_advance(self._h, L.dptr(u), L.dptr(q), int(nsteps)))

    def set_fields(self, u, q):
        L.check(self._lib.cfgpu_dns_set_fields(self._h, L.dptr(_as_field(u, self.grid, 3)),
                                               L.dptr(_as_field(q, self.grid, 1))))

    def advance_resident(self, nsteps: int):
        L.check(self._lib.cfgpu_dns_advance_resident(self._h, int(nsteps)))

    def get_fields(self, u, q):
        L.check(self._lib.cfgpu_dns_get_fields(self._h, L.dptr(_as_field(u, self.grid, 3)),
                                               L.dptr(_as_field(q, self.grid, 1))))

    def cheb_fft(self) -> bool:
        """True when the nonlinear term's Chebyshev transforms run through the FFT (else matrix products)."""
        v = C.c_int()
        L.check(self._lib.cfgpu_dns_cheb_fft(self._h, C.byref(v)))
        return bool(v.value)

    def cheb_tensor(self) -> bool:
        """True when the mixed path's forward Chebyshev transform runs on the tensor cores."""
        v = C.c_int()
        L.check(self._lib.cfgpu_dns_cheb_tensor(self._h, C.byref(v)))
        return bool(v.value)

    def advance_timed(self, nsteps: int) -> float:
        """Resident advance bracketed by CUDA events on the library's stream; device milliseconds."""
        ms = C.c_double()
        L.check(self._lib.cfgpu_dns_advance_timed(self._h, int(nsteps), C.byref(ms)))
        return ms.value

    def field2vector(self, slot: int = 0) -> np.ndarray:
        """field2vector of the resident velocity (of field `slot` of an ensemble), computed on the GPU."""
        from .dsi import field2vector_size
        v = np.zeros(field2vector_size(self.grid))
        L.check(self._lib.cfgpu_ensemble_field2vector(self._h, int(slot), L.dptr(v)))
        return v

    def vector2field(self, v: np.ndarray, slot: int = 0):
        """Set the resident velocity (of field `slot`) to vector2field(v), on the GPU; the pressure is kept."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        L.check(self._lib.cfgpu_ensemble_vector2field(self._h, int(slot), L.dptr(v)))

    def reset_time(self, t: float):
        """DNS::reset_time (dns.cpp:199-205)."""
        L.check(self._lib.cfgpu_dns_reset_time(self._h, float(t)))

    def reset_gradp(self, dPdx: float, dPdz: float = 0.0):
        """DNS::reset_gradp (dns.cpp:221-226): pressure-gradient constraint from the next step on."""
        L.check(self._lib.cfgpu_dns_reset_gradp(self._h, float(dPdx), float(dPdz)))

    def reset_bulkv(self, Ubulk: float, Wbulk: float = 0.0):
        """DNS::reset_bulkv (dns.cpp:227-232): bulk-velocity constraint from the next step on."""
        L.check(self._lib.cfgpu_dns_reset_bulkv(self._h, float(Ubulk), float(Wbulk)))

    def constraint(self) -> dict:
        """DNS::Ubulk, Wbulk, UbulkRef, WbulkRef, dPdxRef, dPdzRef (dns.cpp:298-330)."""
        v = np.zeros(6)
        L.check(self._lib.cfgpu_dns_constraint(self._h, L.dptr(v)))
        return dict(zip(("Ubulk", "Wbulk", "UbulkRef", "WbulkRef", "dPdxRef", "dPdzRef"), v.tolist()))

    def host_access(self) -> bool:
        """True when this DNS reads and writes host FlowField buffers with its own kernels (no staging)."""
        v = C.c_int()
        L.check(self._lib.cfgpu_dns_host_access(self._h, C.byref(v)))
        return bool(v.value)

    def set_graphs(self, enable: bool):
        """Replay steady-state steps from captured CUDA graphs (default) or launch every kernel."""
        L.check(self._lib.cfgpu_dns_set_graphs(self._h, int(bool(enable))))

    def set_profiling(self, enable: bool):
        L.check(self._lib.cfgpu_dns_set_profiling(self._h, int(bool(enable))))

    def phase_times(self):
        """(nl_ms, nl_count, tau_ms, tau_count) accumulated since the last call."""
        a, c = C.c_double(), C.c_double()
        b, d = C.c_longlong(), C.c_longlong()
        L.check(self._lib.cfgpu_dns_phase_times(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value

    def reset_dt(self, dt: float):
        L.check(self._lib.cfgpu_dns_reset_dt(self._h, float(dt)))
        self.flags.dt = dt

    def time(self) -> float:
        t = C.c_double()
        L.check(self._lib.cfgpu_dns_time(self._h, C.byref(t)))
        return t.value

    def dPdx(self) -> float:
        v = C.c_double()
        L.check(self._lib.cfgpu_dns_dPdx(self._h, C.byref(v)))
        return v.value

    def CFL(self) -> float:
        """DNS::CFL of the current velocity (dnsalgo.cpp:63-67)."""
        v = C.c_double()
        L.check(self._lib.cfgpu_dns_cfl(self._h, C.byref(v)))
        return v.value

    def nonlinear(self, u) -> np.ndarray:
        """navierstokesNL(u) + zeroPaddedModes (nse.cpp:12-91, 383-391) with this DNS's flags and precision;
        the DNS's own fields are untouched."""
        u = np.ascontiguousarray(_as_field(u, self.grid, 3))
        f = np.zeros_like(u)
        L.check(self._lib.cfgpu_dns_nonlinear(self._h, L.dptr(u), L.dptr(f)))
        return f

    def l2norm(self, field: int = 0) -> float:
        """L2Norm (normalize=true) of the current u (field 0) or q (field 1)."""
        v = C.c_double()
        L.check(self._lib.cfgpu_dns_l2norm(self._h, int(field), C.byref(v)))
        return v.value

    def base(self):
        U = np.zeros(self.grid.Ny)
        W = np.zeros(self.grid.Ny)
        L.check(self._lib.cfgpu_dns_base(self._h, L.dptr(U), L.dptr(W)))
        return U, W

    def num_modes(self) -> int:
        n = C.c_int()
        L.check(self._lib.cfgpu_dns_num_modes(self._h, C.byref(n)))
        return n.value

    def device_bytes(self) -> int:
        n = C.c_longlong()
        L.check(self._lib.cfgpu_dns_device_bytes(self._h, C.byref(n)))
        return n.value

    def kernel_launches(self) -> int:
        n = C.c_longlong()
        L.check(self._lib.cfgpu_dns_kernel_launches(self._h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cfgpu_dns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble(DNS):
    """nfields fields with one grid and one set of flags, advanced by shared kernel launches.

    Whole-ensemble buffers are shaped (nfields, 3, Ny, Nx, Nz//2+1) for u and
    (nfields, 1, ...) for q; set_field/get_field address one slot.  Every
    field's result equals a single-field DNS of that field.
    """

    def __init__(self, grid: Grid, flags: DNSFlags, nfields: int, precision: str = "fp64"):
        lib = L.load()
        self.grid, self.flags, self.nfields = grid, flags, int(nfields)
        prec = {"fp64": L.CFGPU_FP64, "mixed": L.CFGPU_MIXED}[precision]
        h = C.c_void_p()
        gc, fc = grid.to_c(), flags.to_c()
        L.check(lib.cfgpu_ensemble_create(C.byref(gc), C.byref(fc), self.nfields, prec, C.byref(h)))
        self._h = h
        self._lib = lib

    def _all(self, a, Nd):
        shape = (self.nfields, Nd, self.grid.Ny, self.grid.Nx, self.grid.Mz)
        if a.dtype != np.complex128 or not a.flags["C_CONTIGUOUS"] or a.shape != shape:
            raise ValueError("ensemble buffer must be C-contiguous complex128 of shape %s" % (shape,))
        return a

    def advance(self, u, q, nsteps: int):
        L.check(self._lib.cfgpu_dns_advance(self._h, L.dptr(self._all(u, 3)), L.dptr(self._all(q, 1)),
                                            int(nsteps)))

    def set_fields(self, u, q):
        L.check(self._lib.cfgpu_dns_set_fields(self._h, L.dptr(self._all(u, 3)), L.dptr(self._all(q, 1))))

    def get_fields(self, u, q):
        L.check(self._lib.cfgpu_dns_get_fields(self._h, L.dptr(self._all(u, 3)), L.dptr(self._all(q, 1))))

    def set_field(self, slot: int, u, q=None):
        L.check(self._lib.cfgpu_ensemble_set_field(self._h, int(slot), L.dptr(_as_field(u, self.grid, 3)),
                                                   L.dptr(None if q is None else _as_field(q, self.grid, 1))))

    def get_field(self, slot: int, u, q):
        L.check(self._lib.cfgpu_ensemble_get_field(self._h, int(slot), L.dptr(_as_field(u, self.grid, 3)),
                                                   L.dptr(_as_field(q, self.grid, 1))))

    def set_params(self, slot: int, flags: DNSFlags, base=None):
        """Field `slot` gets the nu, base flow and constraint of `flags` (dt and schemes stay shared)."""
        fc = flags.to_c()
        Ub = Wb = None
        if base is not None:
            Ub = np.ascontiguousarray(base[0], dtype=np.float64)
            Wb = np.ascontiguousarray(base[1], dtype=np.float64)
        L.check(self._lib.cfgpu_ensemble_set_params(self._h, int(slot), C.byref(fc), L.dptr(Ub), L.dptr(Wb)))

    def load_slot(self, slot: int, dns: DNS):
        """Move the time-stepping state of a started single-field DNS into field `slot`."""
        L.check(self._lib.cfgpu_ensemble_load_slot(self._h, int(slot), dns._h))

    def CFL(self) -> np.ndarray:
        v = np.zeros(self.nfields)
        L.check(self._lib.cfgpu_ensemble_cfl(self._h, L.dptr(v)))
        return v

    def l2norm(self, field: int = 0) -> np.ndarray:
        v = np.zeros(self.nfields)
        L.check(self._lib.cfgpu_ensemble_l2norm(self._h, int(field), L.dptr(v)))
        return v

    def dPdx(self) -> np.ndarray:
        v = np.zeros(self.nfields)
        L.check(self._lib.cfgpu_ensemble_dPdx(self._h, L.dptr(v)))
        return v


def tau_solve_batched(N, kx, kz, Lx, Lz, a, b, lambda_t, nu, Rx, Ry, Rz, taucorrection=True):
    """Batched TauSolver solve; R* complex arrays shaped (nmodes, N). Returns (u, v, w, P)."""
    lib = L.load()
    kx = np.ascontiguousarray(kx, dtype=np.int32)
    kz = np.ascontiguousarray(kz, dtype=np.int32)
    nm = kx.shape[0]
    Rs = [np.ascontiguousarray(r, dtype=np.complex128) for r in (Rx, Ry, Rz)]
    for r in Rs:
        assert r.shape == (nm, N)
    outs = [np.zeros((nm, N), dtype=np.complex128) for _ in range(4)]
    L.check(lib.cfgpu_tau_solve_batched(int(N), int(nm), L.iptr(kx), L.iptr(kz), float(Lx), float(Lz), float(a),
                                        float(b), float(lambda_t), float(nu), int(bool(taucorrection)),
                                        *[L.dptr(r) for r in Rs], *[L.dptr(o) for o in outs]))
    return tuple(outs)


def set_host_access(enable: bool):
    """Direct host-buffer access for DNS objects created from now on (default: on where the device
    supports it); off: host-side gathers and pinned staging copies."""
    L.check(L.load().cfgpu_set_host_access(int(bool(enable))))


class PinnedHost:
    """Page-locks host arrays for the lifetime of a `with` block (cfgpu_host_register / _unregister), e.g. the
    FlowField buffers a caller passes to DNS.advance on every step; the arrays stay ordinary NumPy arrays."""

    def __init__(self, *arrays: np.ndarray):
        for a in arrays:
            if not a.flags.c_contiguous:
                raise ValueError("pinned arrays must be C-contiguous")
        self._arrays = arrays
        self._done = []

    def __enter__(self):
        lib = L.load()
        try:
            for a in self._arrays:
                L.check(lib.cfgpu_host_register(C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes)))
                self._done.append(a)
        except BaseException:
            self.__exit__(None, None, None)
            raise
        return self

    def __exit__(self, *exc):
        lib = L.load()
        while self._done:
            a = self._done.pop()
            L.check(lib.cfgpu_host_unregister(C.c_void_p(a.ctypes.data)))
        return False


def helmholtz_solve_batched(a: float, b: float, lam, nu: float, f, ua=None, ub=None, umean=None):
    """HelmholtzSolver(N, a, b, lambda_s, nu).solve for many systems (helmholtz.cpp:18-95): f is
    [nsys][N] Chebyshev coefficients; returns u [nsys][N], or (u, mu) with umean given (the
    mean-constrained solve, helmholtz.cpp:158-213)."""
    f = np.ascontiguousarray(np.atleast_2d(np.asarray(f, dtype=np.float64)))
    nsys, N = f.shape
    lam = np.ascontiguousarray(np.broadcast_to(np.asarray(lam, dtype=np.float64), (nsys,)))
    vec = lambda v: None if v is None else np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float64), (nsys,)))
    ua, ub, umean = vec(ua), vec(ub), vec(umean)
    u = np.zeros_like(f)
    lib = L.load()
    if umean is None:
        L.check(lib.cfgpu_helmholtz_solve_batched(N, nsys, a, b, L.dptr(lam), nu, L.dptr(f), L.dptr(ua), L.dptr(ub),
                                                  L.dptr(u)))
        return u
    mu = np.zeros(nsys)
    L.check(lib.cfgpu_helmholtz_solve_mean_batched(N, nsys, a, b, L.dptr(lam), nu, L.dptr(f), L.dptr(umean),
                                                   L.dptr(ua), L.dptr(ub), L.dptr(u), L.dptr(mu)))
    return u, mu


class DeviceField:
    """FlowField on the GPU (2/3-dealiased modes of Nd components): upload / download host FlowField buffers,
    hand to and take from a DNS without a host round trip."""

    def __init__(self, grid: Grid, Nd: int = 3):
        self.grid, self.Nd = grid, Nd
        self._lib = L.load()
        h = C.c_void_p()
        gc = grid.to_c()
        L.check(self._lib.cfgpu_field_create(C.byref(gc), int(Nd), C.byref(h)))
        self._h = h

    def upload(self, u):
        L.check(self._lib.cfgpu_field_upload(self._h, L.dptr(_as_field(np.ascontiguousarray(u), self.grid, self.Nd))))

    def download(self) -> np.ndarray:
        out = np.zeros((self.Nd, self.grid.Ny, self.grid.Nx, self.grid.Nz // 2 + 1), dtype=np.complex128)
        L.check(self._lib.cfgpu_field_download(self._h, L.dptr(out)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cfgpu_field_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_fields_device(dns, u: DeviceField | None, q: DeviceField | None = None, slot: int = 0):
    """The DNS's (slot's) velocity / pressure from GPU fields, device to device."""
    L.check(dns._lib.cfgpu_dns_set_fields_device(dns._h, int(slot), u._h if u else None, q._h if q else None))


def get_fields_device(dns, u: DeviceField | None, q: DeviceField | None = None, slot: int = 0):
    """The DNS's (slot's) velocity / pressure into GPU fields, device to device."""
    L.check(dns._lib.cfgpu_dns_get_fields_device(dns._h, int(slot), u._h if u else None, q._h if q else None))
