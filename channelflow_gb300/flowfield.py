"""A whole FlowField on the GPU with the reference's transforms (channelflow/flowfield.h:52-345).

``FlowField(Nx, Ny, Nz, Nd, Lx, Lz, a, b)`` owns the reference's serial FlowField buffer on the device
(Nd*Ny*Nx*Nzpad doubles, Nzpad = 2*(Nz/2+1)) and mirrors its state machine: ``makePhysical``,
``makeSpectral``, ``makePhysical_xz`` / ``_y``, ``makeSpectral_xz`` / ``_y`` and ``makeState``
(channelflow/flowfield.cpp:1850-2020), computed by libcfgpu.so in FP64.  NumPy views in and out:
``set_spectral`` / ``spectral`` take and give complex (Nd, Ny, Nx, Nz//2+1) arrays, ``set_physical`` /
``physical`` real (Nd, Ny, Nx, Nz) arrays, in the reference's index order.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

Physical, Spectral = 0, 1  # fieldstate (cfbasics/mathdefs.h:77)


class FlowField:
    def __init__(self, Nx: int, Ny: int, Nz: int, Nd: int, Lx: float, Lz: float, a: float = -1.0, b: float = 1.0):
        lib = L.load()
        self.Nx, self.Ny, self.Nz, self.Nd = Nx, Ny, Nz, Nd
        self.Mz, self.Nzpad = Nz // 2 + 1, 2 * (Nz // 2 + 1)
        g = L.Grid(Nx, Ny, Nz, Lx, Lz, a, b)
        h = C.c_void_p()
        L.check(lib.cfgpu_flowfield_create(C.byref(g), int(Nd), C.byref(h)))
        self._h, self._lib = h, lib

    # --- buffer in the reference's layout ---------------------------------------------------------------
    def _raw(self) -> np.ndarray:
        a = np.empty(self.Nd * self.Ny * self.Nx * self.Nzpad)
        L.check(self._lib.cfgpu_flowfield_download(self._h, L.dptr(a)))
        return a

    def set_spectral(self, u: np.ndarray):
        """Spectral data (xzstate = ystate = Spectral), complex (Nd, Ny, Nx, Nz//2+1)."""
        u = np.ascontiguousarray(u, dtype=np.complex128)
        if u.shape != (self.Nd, self.Ny, self.Nx, self.Mz):
            raise ValueError("spectral data must have shape %s" % ((self.Nd, self.Ny, self.Nx, self.Mz),))
        L.check(self._lib.cfgpu_flowfield_upload(self._h, L.dptr(u.view(np.float64)), Spectral, Spectral))

    def set_physical(self, p: np.ndarray):
        """Physical data (xzstate = ystate = Physical), real (Nd, Ny, Nx, Nz)."""
        p = np.asarray(p, dtype=np.float64)
        if p.shape != (self.Nd, self.Ny, self.Nx, self.Nz):
            raise ValueError("physical data must have shape %s" % ((self.Nd, self.Ny, self.Nx, self.Nz),))
        buf = np.zeros((self.Nd, self.Ny, self.Nx, self.Nzpad))
        buf[..., : self.Nz] = p
        L.check(self._lib.cfgpu_flowfield_upload(self._h, L.dptr(buf), Physical, Physical))

    def set_raw(self, buf: np.ndarray, xzstate: int, ystate: int):
        buf = np.ascontiguousarray(buf, dtype=np.float64).ravel()
        if buf.size != self.Nd * self.Ny * self.Nx * self.Nzpad:
            raise ValueError("buffer must hold Nd*Ny*Nx*Nzpad doubles")
        L.check(self._lib.cfgpu_flowfield_upload(self._h, L.dptr(buf), int(xzstate), int(ystate)))

    def raw(self) -> np.ndarray:
        return self._raw()

    def spectral(self) -> np.ndarray:
        """The buffer read as xz-spectral complex data (Nd, Ny, Nx, Nz//2+1)."""
        return self._raw().view(np.complex128).reshape(self.Nd, self.Ny, self.Nx, self.Mz).copy()

    def physical(self) -> np.ndarray:
        """The buffer read as xz-physical real data (Nd, Ny, Nx, Nz)."""
        return self._raw().reshape(self.Nd, self.Ny, self.Nx, self.Nzpad)[..., : self.Nz].copy()

    # --- state machine -----------------------------------------------------------------------------------
    def state(self):
        xz, y = C.c_int(), C.c_int()
        L.check(self._lib.cfgpu_flowfield_state(self._h, C.byref(xz), C.byref(y)))
        return xz.value, y.value

    @property
    def xzstate(self):
        return self.state()[0]

    @property
    def ystate(self):
        return self.state()[1]

    def makePhysical(self):
        L.check(self._lib.cfgpu_flowfield_make_physical(self._h))

    def makeSpectral(self):
        L.check(self._lib.cfgpu_flowfield_make_spectral(self._h))

    def makePhysical_xz(self):
        L.check(self._lib.cfgpu_flowfield_make_physical_xz(self._h))

    def makeSpectral_xz(self):
        L.check(self._lib.cfgpu_flowfield_make_spectral_xz(self._h))

    def makePhysical_y(self):
        L.check(self._lib.cfgpu_flowfield_make_physical_y(self._h))

    def makeSpectral_y(self):
        L.check(self._lib.cfgpu_flowfield_make_spectral_y(self._h))

    def makeState(self, xzstate: int, ystate: int):
        """FlowField::makeState (flowfield.cpp:1999-2020)."""
        if ystate == Physical and xzstate == Physical:
            self.makePhysical()
        elif ystate == Spectral and xzstate == Spectral:
            self.makeSpectral()
        elif ystate == Physical and xzstate == Spectral:
            self.makeSpectral_xz()
            self.makePhysical_y()
        else:
            self.makeSpectral_y()
            self.makePhysical_xz()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cfgpu_flowfield_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
