"""FieldSymmetry on spectral fields through the C ABI (channelflow/symmetry.h, flowfield.cpp:1095-1272)."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .dns import Grid


@dataclass
class FieldSymmetry:
    """sigma (u,v,w)(x,y,z) = s (sx u, sy v, sz w)(sx x + ax Lx, sy y, sz z + az Lz)."""
    sx: int = 1
    sy: int = 1
    sz: int = 1
    ax: float = 0.0
    az: float = 0.0
    s: int = 1

    def to_c(self) -> L.SymmetryC:
        return L.SymmetryC(self.s, self.sx, self.sy, self.sz, self.ax, self.az)


def apply(u: np.ndarray, grid: Grid, sigma: FieldSymmetry, project: bool = False, dealias: bool = True):
    """sigma u (FlowField::operator*=) or (u + sigma u)/2 (FlowField::project) of a spectral field; returns a copy."""
    out = np.array(u, dtype=np.complex128, order="C", copy=True)
    if out.ndim != 4 or out.shape[0] not in (1, 3) or out.shape[1:] != (grid.Ny, grid.Nx, grid.Nz // 2 + 1):
        raise ValueError("field must be (1 or 3, Ny, Nx, Nz//2+1)")
    gc, sc = grid.to_c(), sigma.to_c()
    L.check(L.load().cfgpu_field_symmetry(C.byref(gc), int(bool(dealias)), out.shape[0], C.byref(sc),
                                          int(bool(project)), L.dptr(out)))
    return out


def set_symmetries(dns, syms, interval: int = 100):
    """DNSFlags::symmetries / symmetryprojectioninterval for a DNS or Ensemble."""
    arr = (L.SymmetryC * max(1, len(syms)))(*[s.to_c() for s in syms])
    L.check(dns._lib.cfgpu_dns_set_symmetries(dns._h, C.cast(arr, C.c_void_p), len(syms), int(interval)))


def apply_resident(dns, sigma: FieldSymmetry, project: bool = False):
    """sigma (or its projection) on the resident velocity of every field of a DNS or Ensemble."""
    sc = sigma.to_c()
    L.check(dns._lib.cfgpu_dns_symmetry(dns._h, C.byref(sc), int(bool(project))))
