"""ctypes binding of libspacecharge_gb300.so (the C ABI in
include/spacecharge_gb300.h).  The library is required: nothing here has a
CPU fallback, and loading fails loudly when the .so has not been built."""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
LIBPATH = os.path.join(_PKG_ROOT, "lib", "libspacecharge_gb300.so")

SC_OK = 0
SC_ERR_INVALID = 1
SC_ERR_CUDA = 2
SC_ERR_OOM = 3
SC_ERR_OUT_OF_RANGE = 4
SC_ERR_TIMEOUT = 5
SC_ERR_UNSUPPORTED = 6

SC_F32 = 0
SC_F64 = 1

SC_PREC_PLAIN64 = 0
SC_PREC_FP64 = 1
SC_PREC_MIXED = 2

SC_DEPOSIT_ATOMIC = 0
SC_DEPOSIT_SORTED = 1
SC_DEPOSIT_DETERMINISTIC = 2
SC_DEPOSIT_TILED = 3
SC_DEPOSIT_VECTOR = 4

SC_NUM_STAGES = 9
STAGES = ["deposit", "green", "fwd_x", "fwd_y", "zpass", "inv_y", "inv_x", "gather", "plain_fft"]

SC_FFT_AUTO = 0
SC_FFT_STOCKHAM = 1
SC_FP64_ARITH_FP64 = 0
SC_FP64_ARITH_DF32 = 1

SC_LAYOUT_PLANAR = 0
SC_LAYOUT_PACKED = 1


class SpaceChargeError(Exception):
    """Raised for a failing library call; the analogue of the reference's
    `error("...")` / ErrorException.  `code` is the SC_ERR_* status."""

    def __init__(self, msg: str, code: int = SC_ERR_INVALID):
        super().__init__(msg)
        self.code = code


class MeshInfo(C.Structure):
    _fields_ = [
        ("grid_size", C.c_int32 * 3),
        ("precision", C.c_int32),
        ("min_bounds", C.c_double * 3),
        ("max_bounds", C.c_double * 3),
        ("delta", C.c_double * 3),
        ("gamma", C.c_double),
        ("total_charge", C.c_double),
        ("efield_layout", C.c_int32),
        ("elem_bytes", C.c_int32),
        ("fft_shape", C.c_int32 * 3),
        ("device", C.c_int32),
    ]


_vp = C.c_void_p
_i64 = C.c_int64
_int = C.c_int
_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)

# name -> argtypes; every function returns int (status) except noted
SIGNATURES = {
    "sc_version": [],
    "sc_last_error": [],
    "sc_mesh_create": [_i32p, _dp, _dp, C.c_double, C.c_double, _int, C.POINTER(_vp)],
    "sc_auto_bounds": [_i32p, _vp, _vp, _vp, _i64, _int, _dp, _dp, _dp, _vp],
    "sc_mesh_create_from_particles": [_i32p, _vp, _vp, _vp, _i64, _int, C.c_double, C.c_double, _int, _vp,
                                      C.POINTER(_vp)],
    "sc_mesh_destroy": [_vp],
    "sc_mesh_set_bounds": [_vp, _dp, _dp],
    "sc_mesh_refit": [_vp, _vp, _vp, _vp, _i64, _int, _vp],
    "sc_mesh_get_info": [_vp, C.POINTER(MeshInfo)],
    "sc_mesh_rho": [_vp, C.POINTER(_vp)],
    "sc_mesh_efield": [_vp, C.POINTER(_vp)],
    "sc_mesh_set_green_cache": [_vp, _int],
    "sc_mesh_set_fp64_arithmetic": [_vp, _int],
    "sc_mesh_set_kick_mode": [_vp, _int],
    "sc_mesh_set_kick_graph": [_vp, _int],
    "sc_set_fft_engine": [_int],
    "sc_test_fail_allocations": [_i64],
    "sc_clear_mesh": [_vp, _vp],
    "sc_deposit": [_vp, _vp, _vp, _vp, _vp, _i64, _int, _int, _int, _vp],
    "sc_solve": [_vp, _int, _vp],
    "sc_interpolate_field": [_vp, _vp, _vp, _vp, _i64, _int, _vp, _vp, _vp, _vp],
    "sc_kick": [_vp, _vp, _vp, _vp, _vp, _i64, _int, _int, _vp, _vp, _vp, _vp],
    "sc_kick_host": [_vp, _vp, _vp, _vp, _vp, _i64, _int, _int, _vp, _vp, _vp, _vp],
    "sc_magnetic_field": [_vp, _vp, _vp, _i64, _int, _vp, _vp, _vp],
    "sc_aos_to_soa": [_vp, _i64, _int, _i32p, _int, _vp, _vp, _vp, _vp, _vp],
    "sc_soa_to_aos": [_vp, _vp, _vp, _i64, _int, _int, _i32p, _vp, _vp],
    "sc_relative_to_absolute": [_vp, _vp, _vp, _i64, _dp, _vp, _vp, _vp, _vp],
    "sc_solve_potential": [_vp, _int, _vp, _vp],
    "sc_bounds_from_extrema": [_i32p, _dp, _dp, _dp, _dp, _dp],
    "sc_track": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _int, C.c_double, C.c_double, _int, _int, _int, _vp],
    "sc_mesh_set_profiling": [_vp, _int],
    "sc_mesh_stage_times": [_vp, _dp, C.POINTER(_i64), _vp],
    "sc_mesh_launch_count": [_vp, C.POINTER(_i64)],
    "sc_kick_adjoint": [_vp, _vp, _vp, _vp, _vp, _i64, _int, _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "sc_solve_noalloc": [_i32p, _dp, C.c_double, _vp, _vp, _vp],
    "sc_batch_create": [C.POINTER(_vp), _int, _int, C.POINTER(_vp)],
    "sc_batch_kick": [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_i64), _int,
                      _int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _vp],
    "sc_batch_set_graph": [_vp, _int],
    "sc_batch_set_staged": [_vp, _int],
    "sc_batch_set_group_bytes": [_vp, _i64],
    "sc_batch_set_fused_forward": [_vp, _int],
    "sc_batch_autotune": [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_i64), _int,
                          _int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _vp, C.POINTER(_i64),
                          C.POINTER(_int)],
    "sc_batch_staged_count": [_vp, C.POINTER(_int), C.POINTER(_i64)],
    "sc_batch_graph_nodes": [_vp, C.POINTER(_i64)],
    "sc_batch_destroy": [_vp],
    "sc_autotune": [_vp, _vp, C.POINTER(_int)],
    "sc_cell_index": [_vp, _vp, _vp, _vp, _i64, _int, _vp, _vp, _vp],
    "sc_mesh_out_of_range": [_vp, C.POINTER(_i64), _vp],
}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load the library once; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIBPATH
        if not os.path.exists(p):
            raise ImportError(
                f"{p} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(p)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_char_p if name == "sc_last_error" else C.c_int
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != SC_OK:
        msg = load().sc_last_error().decode(errors="replace")
        raise SpaceChargeError(msg, status)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
