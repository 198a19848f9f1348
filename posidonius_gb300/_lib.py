"""ctypes binding of libposidonius_gb300.so (the C ABI in include/posidonius_gb300.h).

The library is built in-tree by ``posidonius_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for the product path.
"""
import ctypes
import os

from . import layout as L

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libposidonius_gb300.so")

_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_intp = ctypes.POINTER(ctypes.c_int)
_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); every symbol declared in the C header.
SIGNATURES = {
    "posi_version": (ctypes.c_char_p, []),
    "posi_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "posi_last_error": (ctypes.c_char_p, []),
    "posi_device_count": (ctypes.c_int, []),
    "posi_read_case": (ctypes.c_int, [ctypes.c_char_p, _i64p, _i64p, _i64p, _f64p, _i64p, _f64p, _f64p, _f64p]),
    "posi_read_case_ias15": (ctypes.c_int, [ctypes.c_char_p, _f64p]),
    "posi_get_ias15": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "posi_set_ias15": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "posi_batch_get_ias15": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "posi_batch_set_ias15": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "posi_universe_from_json": (_vp, [ctypes.c_char_p, ctypes.c_int, _intp]),
    "posi_universe_from_arrays": (_vp, [_i64p, _f64p, _i64p, _f64p, _f64p, ctypes.c_int64, _f64p, ctypes.c_int,
                                        _intp]),
    "posi_destroy": (None, [_vp]),
    "posi_get_n_particles": (ctypes.c_int, [_vp, _i64p]),
    "posi_get_current_time": (ctypes.c_int, [_vp, _f64p]),
    "posi_get_n_historic_snapshots": (ctypes.c_int, [_vp, _i64p]),
    "posi_set_time_limit": (ctypes.c_int, [_vp, ctypes.c_double]),
    "posi_set_snapshot_periods": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double]),
    "posi_initialize_physical_values": (ctypes.c_int, [_vp]),
    "posi_iterate": (ctypes.c_int, [_vp, ctypes.c_int64, _i64p, _intp]),
    "posi_gravity_calculate_acceleration": (ctypes.c_int, [_vp, ctypes.c_int]),
    "posi_calculate_additional_effects": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                         ctypes.c_int]),
    "posi_get_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p, _f64p]),
    "posi_set_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p]),
    "posi_batch_create": (_vp, [ctypes.c_int64, ctypes.c_int64, _i64p, _f64p, _i64p, _f64p, _f64p, ctypes.c_int64,
                                _f64p, ctypes.c_int, ctypes.c_int, _intp]),
    "posi_batch_destroy": (None, [_vp]),
    "posi_batch_size": (ctypes.c_int, [_vp, _i64p, _i64p]),
    "posi_batch_initialize_physical_values": (ctypes.c_int, [_vp]),
    "posi_batch_iterate": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64]),
    "posi_batch_set_balanced": (ctypes.c_int, [_vp, ctypes.c_int]),
    "posi_batch_get_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p, _f64p]),
    "posi_batch_set_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p]),
    "posi_batch_mapping_for": (ctypes.c_int, [_vp, ctypes.c_int64]),
    "posi_batch_autotune": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]),
    "posi_batch_autotune_report": (ctypes.c_int, [_vp, ctypes.c_int64, _f64p]),
    "posi_batch_last_timing": (ctypes.c_int, [_vp, _f64p, _i64p]),
    "posi_fp64_probe": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, _f64p]),
    "posi_open_history": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int64]),
    "posi_close_history": (ctypes.c_int, [_vp]),
    "posi_write_recovery_snapshot": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "posi_convert_snapshot": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p]),
    "posi_adjoint_create": (_vp, [_vp, ctypes.c_int64, ctypes.c_int64, _intp]),
    "posi_adjoint_destroy": (None, [_vp]),
    "posi_adjoint_forward": (ctypes.c_int, [_vp]),
    "posi_adjoint_backward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "posi_adjoint_last_timing": (ctypes.c_int, [_vp, _f64p, _f64p, _f64p, _f64p]),
    "posi_large_create": (_vp, [ctypes.c_int64, _i64p, _f64p, _i64p, _f64p, _intp]),
    "posi_large_destroy": (None, [_vp]),
    "posi_large_set_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p]),
    "posi_large_get_state": (ctypes.c_int, [_vp, _i64p, _f64p, _i64p, _f64p]),
    "posi_large_initialize_physical_values": (ctypes.c_int, [_vp]),
    "posi_large_iterate": (ctypes.c_int, [_vp, ctypes.c_int64]),
    "posi_large_iterate_tangent": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int32, _i32p, _i32p, _f64p]),
    "posi_large_last_timing": (ctypes.c_int, [_vp, _f64p]),
    "posi_adjoint_vjp_static": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int64,
                                               _vp, _vp, _vp, _vp]),
}

_lib = None


class PosiError(RuntimeError):
    def __init__(self, status, detail=""):
        self.status = status
        name = lib().posi_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{name} ({status}){': ' + detail if detail else ''}")


def lib():
    """Load the library (raises when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run posidonius_gb300.build.build() (needs nvcc)")
        h = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def last_error():
    return lib().posi_last_error().decode()


def check(status, ok=(L.OK,)):
    if status not in ok:
        raise PosiError(status, last_error())
    return status


def ptr(a, kind):
    if a is None:
        return None
    return a.ctypes.data_as({"i": _i64p, "i32": _i32p}.get(kind, _f64p))
