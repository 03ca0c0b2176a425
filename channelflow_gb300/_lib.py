"""ctypes binding of the C ABI in include/cfgpu.h (libcfgpu.so, built in-tree).

There is no fallback: if the library is missing or fails to load, every
entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcfgpu.so")
HEADER = os.path.join(HERE, "..", "include", "cfgpu.h")

CFGPU_OK, CFGPU_EINVAL, CFGPU_ENOMEM, CFGPU_ECUDA, CFGPU_ENOTSUP, CFGPU_ENONFINITE = range(6)
CFGPU_FP64, CFGPU_MIXED = 0, 1


class Grid(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("Lx", C.c_double), ("Lz", C.c_double),
                ("a", C.c_double), ("b", C.c_double)]


class Flags(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("nu", "dPdx", "dPdz", "Ubulk", "Wbulk", "ulowerwall", "uupperwall",
                                          "wlowerwall", "wupperwall", "Vsuck", "t0", "dt")] + \
               [(n, C.c_int) for n in ("baseflow", "constraint", "timestepping", "initstepping", "nonlinearity",
                                       "dealiasing", "taucorrection")] + [("rotation", C.c_double)]


class TimeStepC(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dt", "dtmin", "dtmax", "dT", "CFLmin", "CFLmax")] + [("variable", C.c_int)]


class SymmetryC(C.Structure):
    _fields_ = [("s", C.c_int), ("sx", C.c_int), ("sy", C.c_int), ("sz", C.c_int), ("ax", C.c_double),
                ("az", C.c_double)]


class CfgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cfgpu error %d: %s" % (code, msg))
        self.code = code


_lib = None

_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)
_SIGS = {
    "cfgpu_flags_default": [C.POINTER(Flags)],
    "cfgpu_dns_create": [C.POINTER(Grid), C.POINTER(Flags), _PD, _PD, _PD, C.c_int, C.POINTER(C.c_void_p)],
    "cfgpu_dns_advance": [C.c_void_p, _PD, _PD, C.c_int],
    "cfgpu_dns_set_fields": [C.c_void_p, _PD, _PD],
    "cfgpu_dns_advance_resident": [C.c_void_p, C.c_int],
    "cfgpu_dns_get_fields": [C.c_void_p, _PD, _PD],
    "cfgpu_dns_reset_dt": [C.c_void_p, C.c_double],
    "cfgpu_dns_time": [C.c_void_p, _PD],
    "cfgpu_dns_dPdx": [C.c_void_p, _PD],
    "cfgpu_dns_base": [C.c_void_p, _PD, _PD],
    "cfgpu_dns_num_modes": [C.c_void_p, _PI],
    "cfgpu_dns_device_bytes": [C.c_void_p, C.POINTER(C.c_longlong)],
    "cfgpu_dns_kernel_launches": [C.c_void_p, C.POINTER(C.c_longlong)],
    "cfgpu_dns_destroy": [C.c_void_p],
    "cfgpu_dns_cfl": [C.c_void_p, _PD],
    "cfgpu_dns_nonlinear": [C.c_void_p, _PD, _PD],
    "cfgpu_set_host_access": [C.c_int],
    "cfgpu_dns_reset_time": [C.c_void_p, C.c_double],
    "cfgpu_dns_reset_gradp": [C.c_void_p, C.c_double, C.c_double],
    "cfgpu_dns_reset_bulkv": [C.c_void_p, C.c_double, C.c_double],
    "cfgpu_dns_constraint": [C.c_void_p, _PD],
    "cfgpu_field_create": [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)],
    "cfgpu_field_upload": [C.c_void_p, _PD],
    "cfgpu_field_download": [C.c_void_p, _PD],
    "cfgpu_field_destroy": [C.c_void_p],
    "cfgpu_dns_set_fields_device": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "cfgpu_dns_get_fields_device": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
    "cfgpu_field2vector_size": [C.c_void_p, C.POINTER(C.c_longlong)],
    "cfgpu_orthogonalize": [C.c_int, C.c_int, _PD, _PD, _PD],
    "cfgpu_field2vector": [C.c_void_p, _PD, _PD],
    "cfgpu_vector2field": [C.c_void_p, _PD, _PD],
    "cfgpu_ensemble_field2vector": [C.c_void_p, C.c_int, _PD],
    "cfgpu_ensemble_vector2field": [C.c_void_p, C.c_int, _PD],
    "cfgpu_helmholtz_solve_batched": [C.c_int, C.c_int, C.c_double, C.c_double, _PD, C.c_double, _PD, _PD, _PD, _PD],
    "cfgpu_helmholtz_solve_mean_batched": [C.c_int, C.c_int, C.c_double, C.c_double, _PD, C.c_double, _PD, _PD,
                                           _PD, _PD, _PD, _PD],
    "cfgpu_dns_host_access": [C.c_void_p, C.POINTER(C.c_int)],
    "cfgpu_host_register": [C.c_void_p, C.c_size_t],
    "cfgpu_host_unregister": [C.c_void_p],
    "cfgpu_measure_fp64": [_PD, _PD],
    "cfgpu_dither_versions": [C.c_double, C.POINTER(C.c_float)],
    "cfgpu_timestep_adjust_for_T": [C.c_void_p, C.c_double, _PI, _PI, _PD],
    "cfgpu_timestep_adjust": [C.c_void_p, C.c_double, _PI, _PI],
    "cfgpu_ensemble_create": [C.POINTER(Grid), C.POINTER(Flags), C.c_int, C.c_int, C.POINTER(C.c_void_p)],
    "cfgpu_ensemble_size": [C.c_void_p, _PI],
    "cfgpu_ensemble_set_field": [C.c_void_p, C.c_int, _PD, _PD],
    "cfgpu_ensemble_get_field": [C.c_void_p, C.c_int, _PD, _PD],
    "cfgpu_ensemble_cfl": [C.c_void_p, _PD],
    "cfgpu_ensemble_l2norm": [C.c_void_p, C.c_int, _PD],
    "cfgpu_ensemble_dPdx": [C.c_void_p, _PD],
    "cfgpu_ensemble_set_params": [C.c_void_p, C.c_int, C.POINTER(Flags), _PD, _PD],
    "cfgpu_ensemble_load_slot": [C.c_void_p, C.c_int, C.c_void_p],
    "cfgpu_server_create": [C.c_longlong, C.c_int, C.c_int, C.POINTER(C.c_void_p)],
    "cfgpu_server_submit": [C.c_void_p, C.POINTER(Grid), C.POINTER(Flags), C.c_int, _PD, C.POINTER(C.c_longlong)],
    "cfgpu_server_submit_ft": [C.c_void_p, C.POINTER(Grid), C.POINTER(Flags), C.POINTER(TimeStepC), C.c_double,
                               _PD, C.POINTER(C.c_longlong)],
    "cfgpu_server_pump": [C.c_void_p, C.c_int, _PI],
    "cfgpu_server_poll": [C.c_void_p, C.c_longlong, _PI, _PD, _PD],
    "cfgpu_server_release": [C.c_void_p, C.c_longlong],
    "cfgpu_server_stats": [C.c_void_p, C.POINTER(C.c_longlong)],
    "cfgpu_server_destroy": [C.c_void_p],
    "cfgpu_dns_set_graphs": [C.c_void_p, C.c_int],
    "cfgpu_set_autotune": [C.c_int],
    "cfgpu_set_fused_xz": [C.c_int],
    "cfgpu_set_pdl": [C.c_int],
    "cfgpu_set_register_zpass": [C.c_int],
    "cfgpu_set_cheb_fft": [C.c_int],
    "cfgpu_set_tau_segmented": [C.c_int],
    "cfgpu_set_cheb_tensor": [C.c_int],
    "cfgpu_dns_cheb_tensor": [C.c_void_p, C.POINTER(C.c_int)],
    "cfgpu_dns_cheb_fft": [C.c_void_p, C.POINTER(C.c_int)],
    "cfgpu_dns_set_symmetries": [C.c_void_p, C.c_void_p, C.c_int, C.c_int],
    "cfgpu_dns_symmetry": [C.c_void_p, C.POINTER(SymmetryC), C.c_int],
    "cfgpu_field_symmetry": [C.POINTER(Grid), C.c_int, C.c_int, C.POINTER(SymmetryC), C.c_int, _PD],
    "cfgpu_ff_write": [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                       C.c_double, C.c_int, _PD],
    "cfgpu_ff_read_header": [C.c_char_p, _PI, _PD, _PI, C.c_char_p],
    "cfgpu_ff_read": [C.c_char_p, _PD, C.c_size_t],
    "cfgpu_ft": [C.POINTER(Grid), C.POINTER(Flags), C.POINTER(TimeStepC), C.c_double, _PD, _PD, _PD, C.c_int],
    "cfgpu_dns_l2norm": [C.c_void_p, C.c_int, _PD],
    "cfgpu_dns_advance_timed": [C.c_void_p, C.c_int, _PD],
    "cfgpu_dns_set_profiling": [C.c_void_p, C.c_int],
    "cfgpu_dns_phase_times": [C.c_void_p, _PD, C.POINTER(C.c_longlong), _PD, C.POINTER(C.c_longlong)],
    "cfgpu_flowfield_create": [C.POINTER(Grid), C.c_int, C.POINTER(C.c_void_p)],
    "cfgpu_flowfield_destroy": [C.c_void_p],
    "cfgpu_flowfield_size": [C.c_void_p, C.POINTER(C.c_longlong)],
    "cfgpu_flowfield_data": [C.c_void_p, C.POINTER(C.c_void_p)],
    "cfgpu_flowfield_upload": [C.c_void_p, _PD, C.c_int, C.c_int],
    "cfgpu_flowfield_download": [C.c_void_p, _PD],
    "cfgpu_flowfield_state": [C.c_void_p, _PI, _PI],
    "cfgpu_flowfield_make_physical": [C.c_void_p],
    "cfgpu_flowfield_make_spectral": [C.c_void_p],
    "cfgpu_flowfield_make_physical_xz": [C.c_void_p],
    "cfgpu_flowfield_make_spectral_xz": [C.c_void_p],
    "cfgpu_flowfield_make_physical_y": [C.c_void_p],
    "cfgpu_flowfield_make_spectral_y": [C.c_void_p],
    "cfgpu_tau_solve_batched": [C.c_int, C.c_int, _PI, _PI, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_int, _PD, _PD, _PD, _PD, _PD, _PD, _PD],
    "cfgpu_tau_solve_batched_noalloc": [C.c_int, C.c_int, _PI, _PI, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_double, C.c_int, _PD, _PD, _PD, _PD, _PD, _PD, _PD],
}


def header_functions():
    """Names of all functions declared in include/cfgpu.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cfgpu_[a-z_0-9]+)\s*\(", txt)))


def load(path: str = LIB_PATH):
    """Load libcfgpu.so (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libcfgpu.so is not built: run channelflow_gb300.build.build() (needs nvcc)")
    lib = C.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.cfgpu_last_error.restype = C.c_char_p
    lib.cfgpu_version.restype = C.c_char_p
    _lib = lib
    return lib


def check(code: int):
    if code != CFGPU_OK:
        raise CfgpuError(code, load().cfgpu_last_error().decode())


def dptr(a):
    return a.ctypes.data_as(_PD) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_PI)
