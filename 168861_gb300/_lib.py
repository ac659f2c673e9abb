"""ctypes binding of libneurite_gb300.so (include/neurite_gb300.h).

The library is the product: loading fails loudly when it is missing (no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libneurite_gb300.so")

NRT_OK, NRT_EINVAL, NRT_ETOPOLOGY, NRT_ENOMEM, NRT_ENOCONV = 0, 1, 2, 3, 4
NRT_EDEVICE, NRT_EBUDGET, NRT_ESTATE, NRT_ENOTREADY = 5, 6, 7, 8
NRT_EXPLICIT, NRT_IMPLICIT_BE = 0, 1
NRT_FP64, NRT_MIXED = 0, 1
NRT_GMRES, NRT_BICGSTAB = 0, 1
NRT_PRECOND_NONE, NRT_PRECOND_JACOBI, NRT_PRECOND_SEGMENT, NRT_PRECOND_TREE = 0, 1, 2, 3
NRT_TOL_ABS, NRT_TOL_REL = 0, 1
NRT_BACKWARD_EULER, NRT_CRANK_NICOLSON = 0, 1

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


class Problem(ctypes.Structure):
    _fields_ = [
        ("num_elem", ctypes.c_int32), ("mother", _i32p), ("dr", _i32p), ("dl", _i32p),
        ("branching", _i32p), ("num_term", ctypes.c_int32), ("terminals", _i32p),
        ("dx", _f64p), ("c_m", _f64p), ("r_a", _f64p), ("W", _f64p), ("K", _f64p),
        ("input", _f64p), ("num_hh", ctypes.c_int32), ("hh_elem", _i32p),
        ("m", _f64p), ("h", _f64p), ("n", _f64p), ("g_Na", _f64p), ("g_K", _f64p),
        ("G_L", _f64p), ("E_Na", _f64p), ("E_K", _f64p), ("E_L", _f64p), ("ls_Na", _f64p),
        ("ls_K", _f64p), ("rest", _f64p), ("V0", _f64p), ("V1", _f64p), ("dT", ctypes.c_double),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int32), ("precision", ctypes.c_int32), ("krylov", ctypes.c_int32),
        ("precond", ctypes.c_int32), ("restart", ctypes.c_int32), ("tol_mode", ctypes.c_int32),
        ("tol", ctypes.c_double), ("max_iter", ctypes.c_int32), ("device", ctypes.c_int32),
        ("use_graphs", ctypes.c_int32), ("schedule", ctypes.c_int32),
        ("tiled", ctypes.c_int32), ("scheme", ctypes.c_int32),
        ("tile_ctas_per_sm", ctypes.c_int32), ("step_threads", ctypes.c_int32),
        ("inner_tol", ctypes.c_double), ("step_launch", ctypes.c_int32),
        ("refinement", ctypes.c_int32),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_int64), ("chunk_steps", ctypes.c_int32),
                ("max_batch", ctypes.c_int32), ("max_wait_us", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 5)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("rejected", ctypes.c_int64), ("batches_created", ctypes.c_int64),
                ("compartment_steps", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("busy_seconds", ctypes.c_double), ("peak_bytes", ctypes.c_int64)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int64), ("krylov_iters", ctypes.c_int64), ("last_iters", ctypes.c_int32),
        ("nonconverged_steps", ctypes.c_int32), ("last_residual", ctypes.c_double),
        ("device_bytes", ctypes.c_int64),
    ]


class InstanceRun(ctypes.Structure):
    _fields_ = [("i_begin", ctypes.c_int64), ("i_end", ctypes.c_int64),
                ("init_time", ctypes.c_double), ("end_input", ctypes.c_double)]


class RecordConfig(ctypes.Structure):
    _fields_ = [("num_probes", ctypes.c_int32), ("instance", _i32p), ("element", _i32p),
                ("origin", ctypes.c_int64), ("interval", ctypes.c_int64),
                ("capacity", ctypes.c_int64), ("threshold", ctypes.c_double),
                ("max_spikes", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]


class StrainConfig(ctypes.Structure):
    _fields_ = [("num_elem", ctypes.c_int32), ("instance", _i32p), ("element", _i32p),
                ("kind", _i32p), ("dspec", _f64p), ("myelin", ctypes.c_int32),
                ("e_max", ctypes.c_double), ("eps0", ctypes.c_double), ("eps1", ctypes.c_double),
                ("t0", ctypes.c_double), ("t1", ctypes.c_double), ("reserved", ctypes.c_int32 * 4)]


# Every symbol include/neurite_gb300.h declares.
EXPORTS = (
    "nrt_options_default", "nrt_create", "nrt_update", "nrt_calculate", "nrt_snapshot", "nrt_run",
    "nrt_synchronize", "nrt_get_stream", "nrt_potential_device", "nrt_get_gates", "nrt_export_system",
    "nrt_get_stats", "nrt_destroy", "nrt_status_string", "nrt_last_error", "nrt_derive",
    "nrt_batch_create", "nrt_batch_set_runs", "nrt_batch_advance", "nrt_batch_synchronize", "nrt_batch_get_stream",
    "nrt_batch_snapshot", "nrt_batch_remaining", "nrt_batch_get_stats", "nrt_batch_destroy",
    "nrt_batch_instance_stats",
    "nrt_server_create", "nrt_server_submit", "nrt_server_result", "nrt_server_drain",
    "nrt_server_get_stats", "nrt_server_destroy", "nrt_solve_csr_static",
    "nrt_measurement_point", "nrt_record", "nrt_batch_record", "nrt_record_read",
    "nrt_batch_record_read", "nrt_batch_pass_counts", "nrt_get_state", "nrt_set_state",
    "nrt_batch_get_state", "nrt_batch_set_state", "nrt_batch_snapshot_all",
    "nrt_server_submit_recorded", "nrt_server_recording", "nrt_derive_batch",
    "nrt_set_strain", "nrt_batch_set_strain", "nrt_kernel_launches",
)

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the CUDA library; raises if it has not been built (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "(the solver has no CPU fallback)")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    vpp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "nrt_options_default": [ctypes.POINTER(Options)],
        "nrt_create": [ctypes.POINTER(Problem), ctypes.POINTER(Options), vpp],
        "nrt_update": [vp, ctypes.c_int],
        "nrt_calculate": [vp],
        "nrt_snapshot": [vp, _f64p],
        "nrt_run": [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double],
        "nrt_synchronize": [vp],
        "nrt_get_stream": [vp, ctypes.POINTER(ctypes.c_void_p)],
        "nrt_batch_get_stream": [vp, ctypes.POINTER(ctypes.c_void_p)],
        "nrt_potential_device": [vp, ctypes.POINTER(ctypes.c_void_p)],
        "nrt_get_gates": [vp, _f64p, _f64p, _f64p],
        "nrt_export_system": [vp, ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _i32p],
        "nrt_get_stats": [vp, ctypes.POINTER(Stats)],
        "nrt_destroy": [vp],
        "nrt_derive": [ctypes.c_int32, _i32p, _f64p, ctypes.c_int32, ctypes.c_double, _f64p, _i32p,
                       _f64p, _i32p, _f64p],
        "nrt_derive_batch": [ctypes.c_int32, _i64p, _i32p, _f64p, _i32p, _f64p, _f64p, _i32p,
                             _f64p, _i64p, _f64p],
        "nrt_batch_create": [ctypes.POINTER(Problem), ctypes.c_int32, ctypes.POINTER(Options), vpp],
        "nrt_batch_set_runs": [vp, ctypes.POINTER(InstanceRun)],
        "nrt_batch_advance": [vp, ctypes.c_int64],
        "nrt_batch_synchronize": [vp],
        "nrt_batch_snapshot": [vp, ctypes.c_int32, _f64p],
        "nrt_batch_snapshot_all": [vp, _f64p],
        "nrt_batch_remaining": [vp, _i64p],
        "nrt_batch_get_stats": [vp, ctypes.POINTER(Stats)],
        "nrt_batch_destroy": [vp],
        "nrt_batch_instance_stats": [vp, _i64p, ctypes.POINTER(ctypes.c_int32),
                                     ctypes.POINTER(ctypes.c_int32), _f64p],
        "nrt_server_create": [ctypes.POINTER(ServerConfig), ctypes.POINTER(Options),
                              ctypes.POINTER(Options), vpp],
        "nrt_server_submit": [vp, ctypes.POINTER(Problem), ctypes.c_int,
                              ctypes.POINTER(InstanceRun), _i64p],
        "nrt_server_result": [vp, ctypes.c_int64, _f64p],
        "nrt_server_submit_recorded": [vp, ctypes.POINTER(Problem), ctypes.c_int,
                                       ctypes.POINTER(InstanceRun), ctypes.POINTER(RecordConfig),
                                       _i64p],
        "nrt_server_recording": [vp, ctypes.c_int64, _i64p, _f64p, _f64p,
                                 ctypes.POINTER(ctypes.c_int32), _f64p],
        "nrt_server_drain": [vp],
        "nrt_server_get_stats": [vp, ctypes.POINTER(ServerStats)],
        "nrt_server_destroy": [vp],
        "nrt_measurement_point": [ctypes.c_int32, _f64p, ctypes.c_double,
                                  ctypes.POINTER(ctypes.c_int32)],
        "nrt_batch_pass_counts": [vp, _i64p, _i64p, _i64p, _i64p, _i64p],
        "nrt_get_state": [vp, _f64p, _f64p, _f64p, _f64p, _f64p],
        "nrt_set_state": [vp, _f64p, _f64p, _f64p, _f64p, _f64p],
        "nrt_batch_get_state": [vp, ctypes.c_int32, _f64p, _f64p, _f64p, _f64p, _f64p],
        "nrt_batch_set_state": [vp, ctypes.c_int32, _f64p, _f64p, _f64p, _f64p, _f64p],
        "nrt_record": [vp, ctypes.POINTER(RecordConfig)],
        "nrt_set_strain": [vp, ctypes.POINTER(StrainConfig)],
        "nrt_batch_set_strain": [vp, ctypes.POINTER(StrainConfig)],
        "nrt_batch_record": [vp, ctypes.POINTER(RecordConfig)],
        "nrt_record_read": [vp, _i64p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int32), _f64p],
        "nrt_batch_record_read": [vp, _i64p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int32), _f64p],
        "nrt_solve_csr_static": [ctypes.c_int32, vp, vp, vp, vp, vp, ctypes.c_int32,
                                 ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp,
                                 ctypes.POINTER(ctypes.c_int32), _f64p],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.nrt_status_string.argtypes = [ctypes.c_int]
    lib.nrt_status_string.restype = ctypes.c_char_p
    lib.nrt_last_error.argtypes = []
    lib.nrt_last_error.restype = ctypes.c_char_p
    lib.nrt_kernel_launches.argtypes = []
    lib.nrt_kernel_launches.restype = ctypes.c_int64
    _lib = lib
    return lib


class NeuriteError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = load()
        msg = lib.nrt_status_string(status).decode()
        detail = lib.nrt_last_error().decode()
        super().__init__(f"{where}: {msg} ({status}){': ' + detail if detail else ''}")
        self.status = status


def check(status: int, where: str) -> int:
    if status != NRT_OK:
        raise NeuriteError(status, where)
    return status
