"""channelflow .ff binary fields through the C ABI (FlowField::binarySave / FlowField(filebase))."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .dns import Grid


def save(path: str, u: np.ndarray, grid: Grid, padded: bool = True):
    """Write the spectral field u [Nd, Ny, Nx, Nz//2+1] (flowfield.cpp:2642-2723)."""
    u = np.ascontiguousarray(u, dtype=np.complex128)
    Nd = u.shape[0]
    if u.shape != (Nd, grid.Ny, grid.Nx, grid.Nz // 2 + 1):
        raise ValueError("field shape does not match the grid")
    L.check(L.load().cfgpu_ff_write(path.encode(), grid.Nx, grid.Ny, grid.Nz, Nd, grid.Lx, grid.Lz, grid.a,
                                    grid.b, int(padded), L.dptr(u)))


def load(path: str):
    """Read a spectral-state .ff file; returns (u, Grid, padded)  (flowfield.cpp:216-356)."""
    lib = L.load()
    dims = (C.c_int * 4)()
    geom = (C.c_double * 4)()
    padded = C.c_int()
    state = C.create_string_buffer(2)
    L.check(lib.cfgpu_ff_read_header(path.encode(), dims, geom, C.byref(padded), state))
    Nx, Ny, Nz, Nd = list(dims)
    u = np.zeros((Nd, Ny, Nx, Nz // 2 + 1), dtype=np.complex128)
    L.check(lib.cfgpu_ff_read(path.encode(), L.dptr(u), u.size * 2))
    return u, Grid(Nx, Ny, Nz, geom[0], geom[1], geom[2], geom[3]), bool(padded.value)
