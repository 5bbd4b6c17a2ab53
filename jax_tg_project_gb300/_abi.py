"""ctypes binding of libtgdns.so (declarations in include/tgdns.h).

The library is built in-tree by ``jax_tg_project_gb300._build.build()``.  There
is no fallback: if the shared library is missing or a CUDA device is absent,
every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

c_int, c_int64, c_double, c_void_p, c_uint64 = (ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                                                ctypes.c_void_p, ctypes.c_uint64)

TG_OK, TG_E_INVALID, TG_E_UNSUPPORTED, TG_E_CUDA, TG_E_NOMEM, TG_E_NONFINITE = range(6)
TG_PHYS_HYDRO, TG_PHYS_MHD = 0, 1
TG_PREC_F32, TG_PREC_F64 = 0, 1
TG_FLAG_EXPLICIT_VISC, TG_FLAG_LORENTZ_REF, TG_FLAG_AUTOTUNE = 1, 2, 4
TG_IC_TAYLOR_GREEN, TG_IC_MHD_REFERENCE, TG_IC_MHD_EQUAL_ENERGY, TG_IC_ZERO = range(4)
TG_ABSMAX_VELOCITY, TG_ABSMAX_DIVERGENCE = 0, 1
TG_DERIVED_VORTICITY, TG_DERIVED_DIVERGENCE = 0, 1
TG_DIAG_WIDTH = 8
TG_PROF_SLOTS = 12
TG_NOALLOC_MAX_RUNS = 64
TG_ADJ_HOST_TAPE = -1  # tg_adjoint: keep every step's stage data in pinned host memory
PASS_NAMES = ("kx_stage_hd", "kx_stage_mhd", "kx_load_hd", "kx_load_mhd", "kx_fwd_hd",
              "kx_fwd_mhd", "ky_inverse", "ky_forward", "kz_product_hd", "kz_product_mhd",
              "kz_c2r", "kz_r2c")
(TG_D_KINETIC, TG_D_ENSTROPHY, TG_D_DISSIPATION, TG_D_MAGNETIC, TG_D_CROSS_HELICITY,
 TG_D_TOTAL, TG_D_DIVU_MAX, TG_D_DIVB_MAX) = range(8)


class TgDesc(ctypes.Structure):
    _fields_ = [("n", c_int), ("batch", c_int), ("physics", c_int), ("precision", c_int),
                ("flags", c_int), ("cutoff", c_int)]


#: every symbol declared in include/tgdns.h with (restype, argtypes)
SIGNATURES = {
    "tg_plan_create": (c_int, [ctypes.POINTER(c_void_p), ctypes.POINTER(TgDesc)]),
    "tg_plan_destroy": (c_int, [c_void_p]),
    "tg_set_stream": (c_int, [c_void_p, c_void_p]),
    "tg_state_layout": (c_int64, [c_void_p, ctypes.POINTER(c_int)]),
    "tg_plan_scratch_bytes": (c_int64, [c_void_p]),
    "tg_set_run_params": (c_int, [c_void_p, ctypes.POINTER(c_double), ctypes.POINTER(c_double),
                                  ctypes.POINTER(c_double), c_int]),
    "tg_initial_condition": (c_int, [c_void_p, c_int, c_uint64, c_double, c_double, c_double, c_void_p]),
    "tg_forward": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_inverse": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_rhs": (c_int, [c_void_p, c_void_p, c_double, c_double, c_void_p]),
    "tg_step": (c_int, [c_void_p, c_void_p, c_double, c_double, c_double, c_int]),
    "tg_run": (c_int, [c_void_p, c_void_p, c_double, c_double, c_double, c_int, c_int, c_void_p]),
    "tg_diagnostics": (c_int, [c_void_p, c_void_p, c_double, c_double, c_void_p]),
    "tg_field_absmax": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "tg_derived": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "tg_to_full_spectrum": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_from_full_spectrum": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_physical_energy": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_profile_passes": (c_int, [c_void_p, c_void_p, c_double, c_double, c_double, c_int,
                                  ctypes.POINTER(c_double), ctypes.POINTER(c_int64)]),
    "tg_adjoint": (c_int, [c_void_p, c_void_p, c_double, c_double, c_int, c_int, c_void_p, c_void_p,
                           c_void_p]),
    "tg_spectrum_bins": (c_int, [c_void_p]),
    "tg_energy_spectrum": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tg_diagnostics_noalloc": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_double, c_double,
                                       c_void_p, c_void_p]),
    "tg_last_launch_count": (c_int64, [c_void_p]),
    "tg_pass_variant": (c_int, [c_void_p]),
    "tg_y_config": (c_int, [c_void_p, ctypes.POINTER(c_int)]),
    "tg_release_host_tape": (c_int, [c_void_p]),
    "tg_adjoint_profile": (c_int, [c_void_p, ctypes.POINTER(c_double)]),
    "tg_last_error": (ctypes.c_char_p, []),
    "tg_version": (c_int, []),
}


class TgError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[tgdns error {code}] {message}")
        self.code = code


_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libtgdns.so and declare its prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(
                f"{path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != TG_OK:
        msg = load().tg_last_error()
        raise TgError(rc, msg.decode() if msg else "unknown error")
    return rc
