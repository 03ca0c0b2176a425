"""Request server over the C ABI: continuous batching of fixed-dt DNS integrations / f^T(u) evaluations.

Requests that share a grid and the shared flags (dt, schemes, nonlinearity,
dealiasing) run as fields of one batched ensemble (per-field Reynolds number,
base flow and constraint); see cfgpu_server_* in include/cfgpu.h.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .dns import DNSFlags, Grid, _as_field

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


class Server:
    def __init__(self, max_bytes: int = 8 << 30, slots: int = 8, precision: str = "fp64"):
        self._lib = L.load()
        prec = {"fp64": L.CFGPU_FP64, "mixed": L.CFGPU_MIXED}[precision]
        h = C.c_void_p()
        L.check(self._lib.cfgpu_server_create(int(max_bytes), int(slots), prec, C.byref(h)))
        self._h = h
        self._shapes = {}

    def submit(self, grid: Grid, flags: DNSFlags, nsteps: int, u: np.ndarray) -> int:
        """Queue nsteps steps of field u (f^T(u) with T = nsteps * flags.dt); returns the request id."""
        u = np.ascontiguousarray(u)
        _as_field(u, grid, 3)
        rid = C.c_longlong()
        gc, fc = grid.to_c(), flags.to_c()
        L.check(self._lib.cfgpu_server_submit(self._h, C.byref(gc), C.byref(fc), int(nsteps), L.dptr(u),
                                              C.byref(rid)))
        self._shapes[rid.value] = u.shape
        return rid.value

    def submit_ft(self, grid: Grid, flags: DNSFlags, timestep, T: float, u: np.ndarray) -> int:
        """Queue f^T(u) with a TimeStep (channelflow_gb300.dsi.TimeStep), as cfDSI's f(u, T) evaluates it."""
        u = np.ascontiguousarray(u)
        _as_field(u, grid, 3)
        rid = C.c_longlong()
        gc, fc, tc = grid.to_c(), flags.to_c(), timestep.to_c()
        L.check(self._lib.cfgpu_server_submit_ft(self._h, C.byref(gc), C.byref(fc), C.byref(tc), float(T),
                                                 L.dptr(u), C.byref(rid)))
        self._shapes[rid.value] = u.shape
        return rid.value

    def pump(self, max_steps: int = 50) -> int:
        """One scheduling round; returns the number of queued or running requests."""
        active = C.c_int()
        L.check(self._lib.cfgpu_server_pump(self._h, int(max_steps), C.byref(active)))
        return active.value

    def poll(self, rid: int):
        """(status, result or None, (t_submit, t_start, t_done))."""
        st = C.c_int()
        shape = self._shapes.get(rid)
        out = np.zeros(shape, dtype=np.complex128) if shape else None
        t = (C.c_double * 3)()
        L.check(self._lib.cfgpu_server_poll(self._h, C.c_longlong(rid), C.byref(st), L.dptr(out), t))
        return st.value, (out if st.value == DONE else None), tuple(t)

    def release(self, rid: int):
        L.check(self._lib.cfgpu_server_release(self._h, C.c_longlong(rid)))
        self._shapes.pop(rid, None)

    def stats(self) -> dict:
        v = (C.c_longlong * 15)()
        L.check(self._lib.cfgpu_server_stats(self._h, v))
        keys = ("device_bytes", "ensembles", "slots", "running", "queued", "ensemble_steps", "field_steps", "chunks",
                "dt_changes", "admit_us", "interval_us", "create_us", "params_us", "stage_us", "load_us")
        return dict(zip(keys, list(v)))

    def run(self, max_steps: int = 50):
        while self.pump(max_steps):
            pass

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cfgpu_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
