"""ctypes binding of libhsrq3in_gb300.so (the C ABI in include/hsrq3in_gb300.h).

The shared library is the product; this module only declares its entry
points.  Loading fails loudly when the library has not been built -- there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

HSR_OK = 0
HSR_ERR_ARG = -1
HSR_ERR_NOMEM = -2
HSR_ERR_CUDA = -3
HSR_ERR_DEVICE = -4
HSR_ERR_NOT_CONVERGED = 1
HSR_SCALING_POW2 = 0
HSR_SCALING_DOUBLE = 1
HSR_BATCH_ENGINE_TICKS = 0
HSR_BATCH_ENGINE_QUEUE = 1

# Every symbol include/hsrq3in_gb300.h declares.
EXPORTS = [
    "hsr_last_status", "hsr_status_string", "tiled_inverse_iteration",
    "hsr_inverse_iteration_ex", "hsr_inverse_iteration_device",
    "hsr_last_launch_count", "hsr_set_kernel_timing", "hsr_last_kernel_times",
    "hsr_release_workspace", "hsr_probe_fp64_peak", "hsr_version",
    "hsr_inverse_iteration_noalloc", "hsr_residuals_device",
    "hsr_hessenberg_device", "hsr_hessenberg_apply_q_device",
    "hsr_batch_plan_create", "hsr_batch_plan_execute", "hsr_batch_plan_info", "hsr_batch_plan_destroy",
    "hsr_batch_plan_set_engine", "hsr_batch_plan_queue_info",
    "hsr_autotune_tlsz", "hsr_autotune_batch", "hsr_autotune_plain", "hsr_autotune_plain_tlsz",
    "hsr_server_create", "hsr_server_replay", "hsr_server_destroy",
    "hsr_inverse_iteration_cplx_ex", "hsr_inverse_iteration_cplx_device", "hsr_inverse_iteration_mixed",
    "hsr_selftest_bounded_wait", "hsr_selftest_arith",
]
NOALLOC_MAX_N = 256
NOALLOC_MAX_NRHS = 256
KERNEL_CLASSES = ["setup", "diag", "part1", "gemm", "finalize", "other", "h2d", "d2h", "gemm_top"]
SERVER_PHASES = ["norms", "init", "diag_first", "part1", "gemm_top", "diag_next", "gemm_rest", "finalize",
                 "normalize"]


class Options(C.Structure):
    _fields_ = [("scaling", C.c_int), ("user_rhs", C.c_int),
                ("max_restarts", C.c_int), ("hbm_budget_bytes", C.c_double)]


class ColumnInfo(C.Structure):
    _fields_ = [("status", C.POINTER(C.c_int)), ("perturbed", C.POINTER(C.c_ubyte)),
                ("scale", C.POINTER(C.c_double)), ("tile_scales", C.POINTER(C.c_double)),
                ("norm", C.POINTER(C.c_double))]


class BatchProblem(C.Structure):
    _fields_ = [("n", C.c_int), ("dH", C.c_void_p), ("lddH", C.c_int), ("nrhs", C.c_int),
                ("dwr", C.c_void_p), ("dvr", C.c_void_p), ("lddvr", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("tlsz", C.c_int), ("max_active", C.c_int),
                ("scaling", C.c_int)]


class Request(C.Structure):
    _fields_ = [("n", C.c_int), ("H", C.c_void_p), ("ldH", C.c_int), ("nrhs", C.c_int),
                ("wr", C.c_void_p), ("vr", C.c_void_p), ("ldvr", C.c_int), ("arrival_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("wall_s", C.c_double), ("ticks", C.c_long), ("launches", C.c_long),
                ("max_active", C.c_int), ("peak_bytes", C.c_double), ("phase_ms", C.c_double * 9),
                ("flops", C.c_double), ("host_wait_s", C.c_double)]


_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load the CUDA library; raise if it is missing (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError("libhsrq3in_gb300.so is not built (%s); run "
                               "__graft_entry__.build() first" % path)
    lib = C.CDLL(path)
    lib.hsr_last_status.restype = C.c_int
    lib.hsr_status_string.restype = C.c_char_p
    lib.hsr_status_string.argtypes = [C.c_int]
    lib.tiled_inverse_iteration.restype = None
    lib.tiled_inverse_iteration.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                            C.c_int, C.c_int, C.c_void_p, C.c_int]
    lib.hsr_inverse_iteration_ex.restype = C.c_int
    lib.hsr_inverse_iteration_ex.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                             C.c_int, C.c_int, C.c_void_p, C.c_int,
                                             C.POINTER(Options), C.POINTER(ColumnInfo)]
    lib.hsr_inverse_iteration_device.restype = C.c_int
    lib.hsr_inverse_iteration_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                 C.c_int, C.c_void_p, C.c_int, C.POINTER(Options),
                                                 C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hsr_inverse_iteration_cplx_ex.restype = C.c_int
    lib.hsr_inverse_iteration_cplx_ex.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                  C.c_int, C.c_int, C.c_void_p, C.c_int,
                                                  C.POINTER(Options), C.POINTER(ColumnInfo)]
    lib.hsr_inverse_iteration_cplx_device.restype = C.c_int
    lib.hsr_inverse_iteration_cplx_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                      C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                                      C.POINTER(Options), C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hsr_inverse_iteration_mixed.restype = C.c_int
    lib.hsr_inverse_iteration_mixed.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                C.c_int, C.c_int, C.c_void_p, C.c_int, C.POINTER(Options),
                                                C.c_void_p]
    lib.hsr_selftest_bounded_wait.restype = C.c_int
    lib.hsr_selftest_bounded_wait.argtypes = [C.c_void_p]
    lib.hsr_residuals_device.restype = C.c_int
    lib.hsr_residuals_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_void_p, C.c_void_p]
    lib.hsr_hessenberg_device.restype = C.c_int
    lib.hsr_hessenberg_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.hsr_hessenberg_apply_q_device.restype = C.c_int
    lib.hsr_hessenberg_apply_q_device.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                  C.c_int, C.c_void_p]
    lib.hsr_last_launch_count.restype = C.c_long
    lib.hsr_set_kernel_timing.restype = None
    lib.hsr_set_kernel_timing.argtypes = [C.c_int]
    lib.hsr_last_kernel_times.restype = C.c_int
    lib.hsr_last_kernel_times.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.hsr_release_workspace.restype = None
    lib.hsr_probe_fp64_peak.restype = C.c_int
    lib.hsr_probe_fp64_peak.argtypes = [C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.hsr_version.restype = C.c_char_p
    lib.hsr_selftest_arith.restype = C.c_int
    lib.hsr_selftest_arith.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    lib.hsr_batch_plan_create.restype = C.c_int
    lib.hsr_batch_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(BatchProblem), C.c_int,
                                          C.POINTER(Options), C.c_void_p]
    lib.hsr_batch_plan_execute.restype = C.c_int
    lib.hsr_batch_plan_execute.argtypes = [C.c_void_p, C.c_void_p]
    lib.hsr_batch_plan_info.restype = C.c_int
    lib.hsr_batch_plan_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_long)]
    lib.hsr_batch_plan_set_engine.restype = C.c_int
    lib.hsr_batch_plan_set_engine.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.hsr_batch_plan_queue_info.restype = C.c_int
    lib.hsr_batch_plan_queue_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_long),
                                              C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.hsr_batch_plan_destroy.restype = None
    lib.hsr_batch_plan_destroy.argtypes = [C.c_void_p]
    lib.hsr_autotune_tlsz.restype = C.c_int
    lib.hsr_autotune_tlsz.argtypes = [C.c_int, C.c_int]
    lib.hsr_autotune_batch.restype = C.c_int
    lib.hsr_autotune_batch.argtypes = [C.c_int, C.POINTER(BatchProblem), C.POINTER(C.c_int), C.c_int,
                                       C.POINTER(C.c_double), C.c_void_p]
    lib.hsr_autotune_plain.restype = C.c_int
    lib.hsr_autotune_plain.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                       C.c_void_p]
    lib.hsr_autotune_plain_tlsz.restype = C.c_int
    lib.hsr_autotune_plain_tlsz.argtypes = [C.c_int]
    lib.hsr_server_create.restype = C.c_int
    lib.hsr_server_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(ServerConfig)]
    lib.hsr_server_replay.restype = C.c_int
    lib.hsr_server_replay.argtypes = [C.c_void_p, C.c_int, C.POINTER(Request), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int), C.POINTER(ServerStats)]
    lib.hsr_server_destroy.restype = None
    lib.hsr_server_destroy.argtypes = [C.c_void_p]
    lib.hsr_inverse_iteration_noalloc.restype = C.c_int
    lib.hsr_inverse_iteration_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                  C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                  C.c_void_p]
    _LIB = lib
    return lib
