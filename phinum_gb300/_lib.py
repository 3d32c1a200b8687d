"""ctypes binding of libphinum_gpu.so (include/phinum_gpu.h).

The library is the product; this module only declares its C ABI for Python
callers (tests, bench).  Loading fails loudly when the shared object is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphinum_gpu.so")

MAX_NC = 4
OK, ERR_INVALID, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT, ERR_NOMEM, ERR_UNSUPPORTED, ERR_TRUNCATED = \
    0, -1, -2, -3, -4, -5, -6, -7
FP64, FP32, FP32_KAHAN, FP32_PAIR = 0, 1, 2, 3
ISLAND_REFERENCE, ISLAND_ENERGY, ISLAND_DELTA = 0, 1, 2
PATH_AUTO, PATH_PLAIN, PATH_TMA, PATH_X4 = 0, 1, 2, 3
TRACK_ALIVE, TRACK_RETIRED, TRACK_BUBBLES = 0, 1, 2
FILTER_TOPHAT, FILTER_GAUSSIAN, FILTER_TABLE, FILTER_KTOPHAT = 0, 1, 2, 3

_D, _I = ctypes.c_double, ctypes.c_int
_PD, _PI = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)


ABI_VERSION = 4  # PHN_ABI_VERSION of include/phinum_gpu.h


class PhnParams(ctypes.Structure):
    _fields_ = [("N", _I), ("Nc", _I), ("potential", _I), ("mass_mode", _I), ("lambda_mode", _I),
                ("precision", _I), ("a", _D), ("dt", _D), ("T0", _D), ("m_sqr", _D), ("kappa", _D),
                ("h", _D), ("g", _D), ("p_mono", _D), ("m_mono_sqr", _D), ("expanding", _I),
                ("reserved_", _I), ("H0", _D)]


class PhnIcParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_long), ("justnoise", _I), ("QS", _D), ("scale2", _D), ("amplitude", _D),
                ("noise", _D), ("phi0", _D * 2), ("pi0", _D * 2), ("m2_long", _D), ("m2_trans", _D)]


class PhnIcMode(ctypes.Structure):
    _fields_ = [("init_mode", _I), ("charged", _I), ("chi", _D), ("famp", _D), ("lambda_", _D),
                ("temperature", _D), ("phi0", _D), ("pi0", _D)]


class PhnTrackIsland(ctypes.Structure):
    _fields_ = [("index", _D), ("status", _D), ("disp", _D), ("length", _D)] + [
        (f, _D * 5) for f in ("at_time", "center", "volume", "pot_en", "kin_en", "grad_en", "av_phi", "peak_value")]


class PhnAverages(ctypes.Structure):
    _fields_ = [("t", _D), ("phi", _D * MAX_NC), ("pi", _D * MAX_NC), ("phi2", _D), ("pi2", _D),
                ("phipi", _D), ("phi4", _D), ("phi6", _D), ("energy", _D), ("interaction", _D),
                ("charge", _D), ("min_phi", _D), ("max_phi", _D), ("max_abs_phi", _D), ("min_pos", _D),
                ("max_pos", _D), ("max_abs_pos", _D), ("gradient", _D), ("nonfinite", _D),
                ("scale_factor", _D)]


AVG_LEN = ctypes.sizeof(PhnAverages) // 8
ISLAND_FIELDS = ["index", "size", "volume", "pot_en", "kin_en", "grad_en", "av_phi", "peak_pos",
                 "peak_value", "seed_pos"]


class PhnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"phn error {code}: {msg}")
        self.code = code


_lib = None

# name: (restype, argtypes)
_SIGS = {
    "phn_abi_version": (_I, []),
    "phn_last_error": (ctypes.c_char_p, []),
    "phn_device_count": (_I, [_PI]),
    "phn_create": (_I, [ctypes.POINTER(PhnParams), ctypes.POINTER(ctypes.c_void_p)]),
    "phn_destroy": (_I, [ctypes.c_void_p]),
    "phn_upload": (_I, [ctypes.c_void_p, _PD, _PD]),
    "phn_download": (_I, [ctypes.c_void_p, _PD, _PD]),
    "phn_upload_f32": (_I, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "phn_download_f32": (_I, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "phn_reset": (_I, [ctypes.c_void_p]),
    "phn_evolve": (_I, [ctypes.c_void_p, _I]),
    "phn_time": (_I, [ctypes.c_void_p, _PD, _PI]),
    "phn_conformal_time": (_I, [ctypes.c_void_p, _PD, _PD]),
    "phn_volume_averages": (_I, [ctypes.c_void_p, ctypes.POINTER(PhnAverages)]),
    "phn_false_vacuum_decayed": (_I, [ctypes.POINTER(PhnAverages), _I, _PI]),
    "phn_run_loop": (_I, [ctypes.c_void_p, _I, _D, ctypes.POINTER(PhnAverages), _I, _PI]),
    "phn_spectrum_bins": (_I, [ctypes.c_void_p, _PI, _PD]),
    "phn_spectrum": (_I, [ctypes.c_void_p, _PD, _PD, _PD, _PI, _I]),
    "phn_spectrum_uniform": (_I, [ctypes.c_void_p, _I, _PD, _PD, _PD, _PI]),
    "phn_spectrum_energy": (_I, [ctypes.c_void_p, _PD, _PI, _I]),
    "phn_spectrum_timing": (_I, [ctypes.c_void_p, _PD, _PD]),
    "phn_initial_conditions": (_I, [ctypes.c_void_p, ctypes.POINTER(PhnIcParams)]),
    "phn_initial_conditions_mode": (_I, [ctypes.c_void_p, ctypes.POINTER(PhnIcParams), ctypes.POINTER(PhnIcMode)]),
    "phn_islands_lookup": (_I, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), _I, _PI]),
    "phn_save_config": (_I, [ctypes.c_void_p, ctypes.c_char_p, _I, _I, _I]),
    "phn_apply_filter": (_I, [ctypes.c_void_p, _D, _I, _PD, _I, _D]),
    "phn_wait_selftest": (_I, [ctypes.c_void_p, ctypes.c_longlong]),
    "phn_divide_selftest": (_I, [ctypes.c_void_p, _D, ctypes.c_longlong, ctypes.c_ulonglong,
                                 ctypes.POINTER(ctypes.c_longlong)]),
    "phn_load_config": (_I, [ctypes.c_void_p, ctypes.c_char_p, _I, _I, _PD, _I]),
    "phn_write_config_file": (_I, [ctypes.c_char_p, _PD, _PD, _I, _I, _I, _I]),
    "phn_read_config_file": (_I, [ctypes.c_char_p, _PD, _PD, _I, _I, _I]),
    "phn_tracker_create": (_I, [_I, ctypes.POINTER(ctypes.c_void_p)]),
    "phn_tracker_destroy": (_I, [ctypes.c_void_p]),
    "phn_tracker_reset": (_I, [ctypes.c_void_p]),
    "phn_tracker_update": (_I, [ctypes.c_void_p, ctypes.c_void_p, _D, _I, _I, _PI]),
    "phn_tracker_update_records": (_I, [ctypes.c_void_p, _D, ctypes.c_void_p, _I, _PI, _PI]),
    "phn_tracker_centers": (_I, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), _I, _PI]),
    "phn_tracker_count": (_I, [ctypes.c_void_p, _I, _PI]),
    "phn_tracker_get": (_I, [ctypes.c_void_p, _I, _I, ctypes.POINTER(PhnTrackIsland)]),
    "phn_tracker_oscillons": (_I, [ctypes.c_void_p, _I, _D, _D, _PD]),
    "phn_tracker_add_stat": (_I, [ctypes.c_void_p, _D, _D, _PI, _PI]),
    "phn_islands": (_I, [ctypes.c_void_p, _D, _I, _I, _PI, _PD, _I, _PI]),
    "phn_islands_device": (_I, [ctypes.c_void_p, _D, _I, _I, ctypes.POINTER(ctypes.c_void_p), _PI]),
    "phn_set_path": (_I, [ctypes.c_void_p, _I]),
    "phn_get_path": (_I, [ctypes.c_void_p, _PI]),
    "phn_autotune": (_I, [ctypes.c_void_p, _I, _PI, _PD]),
    "phn_num_variants": (_I, [ctypes.c_void_p, _PI]),
    "phn_set_variant": (_I, [ctypes.c_void_p, _I]),
    "phn_device_fields": (_I, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                               ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]),
    "phn_synchronize": (_I, [ctypes.c_void_p]),
    "phn_stats": (_I, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), _PD, _PI]),
    "phn_volume_averages_noalloc": (_I, [ctypes.POINTER(PhnParams), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.POINTER(PhnAverages)]),
    "phn_ensemble_create": (_I, [ctypes.POINTER(PhnParams), _I, ctypes.POINTER(ctypes.c_void_p)]),
    "phn_ensemble_destroy": (_I, [ctypes.c_void_p]),
    "phn_ensemble_upload": (_I, [ctypes.c_void_p, _I, _PD, _PD]),
    "phn_ensemble_download": (_I, [ctypes.c_void_p, _I, _PD, _PD]),
    "phn_ensemble_reset": (_I, [ctypes.c_void_p]),
    "phn_ensemble_evolve": (_I, [ctypes.c_void_p, _I]),
    "phn_ensemble_time": (_I, [ctypes.c_void_p, _PD, _PI]),
    "phn_ensemble_averages": (_I, [ctypes.c_void_p, ctypes.c_void_p]),
    "phn_ensemble_islands": (_I, [ctypes.c_void_p, _I, _D, _I, _I, _PI, _PD, _I, _PI]),
    "phn_ensemble_autotune": (_I, [ctypes.c_void_p, _I, _PI, _PD]),
    "phn_ensemble_set_tile": (_I, [ctypes.c_void_p, _I]),
    "phn_ensemble_stats": (_I, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), _PD, _PI]),
    "phn_adjoint_create": (_I, [ctypes.POINTER(PhnParams), _I, _I, _D, ctypes.POINTER(ctypes.c_void_p)]),
    "phn_adjoint_destroy": (_I, [ctypes.c_void_p]),
    "phn_adjoint_forward": (_I, [ctypes.c_void_p, _PD, _PD, _PD]),
    "phn_adjoint_backward": (_I, [ctypes.c_void_p, _PD, _PD, _PD]),
    "phn_adjoint_info": (_I, [ctypes.c_void_p, _PD, _PD, _PD]),
    "phn_adjoint_set_forward_precision": (_I, [ctypes.c_void_p, _I]),
    "phn_pin_host": (_I, [ctypes.c_void_p, ctypes.c_size_t]),
    "phn_unpin_host": (_I, [ctypes.c_void_p]),
}


def exported_symbols():
    return list(_SIGS)


def load(build_if_missing: bool = False):
    """Loads the library once.  Raises if it is not built (build() builds it)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b
            _b.build()
        else:
            raise OSError(f"{LIB_PATH} is not built; run phinum_gb300.build.build() "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.phn_abi_version() != ABI_VERSION:  # the structures above follow one layout
        raise OSError(f"{LIB_PATH} has ABI {lib.phn_abi_version()}, this binding {ABI_VERSION}: rebuild")
    _lib = lib
    return lib


def check(code: int):
    if code != OK:
        msg = _lib.phn_last_error().decode() if _lib is not None else ""
        raise PhnError(code, msg)
    return code
