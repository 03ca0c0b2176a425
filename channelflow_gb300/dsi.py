"""f^T(u) and TimeStep over the C ABI (the role of channelflow's cfDSI::f and TimeStep).

``ft(u, grid, flags, timestep, T)`` returns the velocity after integrating for
time T exactly as cfDSI's f(u, T) does (channelflow/cfdsi.cpp:705-775); the
time loop, CFL checks and dt adjustments run in libcfgpu.so's host code, the
steps on the GPU.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .dns import DNSFlags, Grid, _as_field


@dataclass
class TimeStep:
    """TimeStep parameters with DNSFlags' defaults (dnsflags.h:84-92)."""
    dt: float = 0.03125
    dtmin: float = 0.001
    dtmax: float = 0.2
    dT: float = 1.0
    CFLmin: float = 0.4
    CFLmax: float = 0.6
    variable: bool = True

    def to_c(self) -> L.TimeStepC:
        return L.TimeStepC(self.dt, self.dtmin, self.dtmax, self.dT, self.CFLmin, self.CFLmax, int(self.variable))

    def adjust_for_T(self, T: float):
        """TimeStep::adjust_for_T: returns (n, N, dt) and updates dt, dT."""
        c = self.to_c()
        n, N, dt = C.c_int(), C.c_int(), C.c_double()
        L.check(L.load().cfgpu_timestep_adjust_for_T(C.byref(c), float(T), C.byref(n), C.byref(N), C.byref(dt)))
        self.dt, self.dT = c.dt, c.dT
        return n.value, N.value, dt.value


    def adjust(self, cfl: float) -> bool:
        """TimeStep::adjust(CFL): returns whether dt changed; updates dt."""
        c = self.to_c()
        n, adj = C.c_int(), C.c_int()
        L.check(L.load().cfgpu_timestep_adjust(C.byref(c), float(cfl), C.byref(n), C.byref(adj)))
        self.dt = c.dt
        return bool(adj.value)


def ft(u: np.ndarray, grid: Grid, flags: DNSFlags, timestep: TimeStep, T: float, precision: str = "fp64"):
    """f^T(u) (cfdsi.cpp:705-775); returns (f^T(u), last CFL number)."""
    _as_field(u, grid, 3)
    fu = np.empty_like(u)
    cfl = C.c_double()
    gc, fc, tc = grid.to_c(), flags.to_c(), timestep.to_c()
    prec = {"fp64": L.CFGPU_FP64, "mixed": L.CFGPU_MIXED}[precision]
    L.check(L.load().cfgpu_ft(C.byref(gc), C.byref(fc), C.byref(tc), float(T), L.dptr(u), L.dptr(fu),
                              C.byref(cfl), prec))
    return fu, cfl.value


def field2vector_size(grid: Grid) -> int:
    """field2vector_size (flowfield.cpp:4448-4478): independent reals of a div-free no-slip field."""
    n = C.c_longlong()
    gc = grid.to_c()
    L.check(L.load().cfgpu_field2vector_size(C.byref(gc), C.byref(n)))
    return n.value


def field2vector(u: np.ndarray, grid: Grid) -> np.ndarray:
    """field2vector (flowfield.cpp:4480-4557), on the GPU."""
    u = np.ascontiguousarray(u)
    _as_field(u, grid, 3)
    v = np.zeros(field2vector_size(grid))
    gc = grid.to_c()
    L.check(L.load().cfgpu_field2vector(C.byref(gc), L.dptr(u.view(np.float64)), L.dptr(v)))
    return v


def vector2field(v: np.ndarray, grid: Grid) -> np.ndarray:
    """vector2field (flowfield.cpp:4559-4760), on the GPU: the div-free no-slip field with independent
    coefficients v."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    if v.shape != (field2vector_size(grid),):
        raise ValueError("vector has the wrong size")
    u = np.zeros((3, grid.Ny, grid.Nx, grid.Nz // 2 + 1), dtype=np.complex128)
    gc = grid.to_c()
    L.check(L.load().cfgpu_vector2field(C.byref(gc), L.dptr(v), L.dptr(u.view(np.float64))))
    return u
