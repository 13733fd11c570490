"""numpy / torch front end of the C ABI.

``inverse_iteration`` mirrors the reference's tiled_inverse_iteration
(inverse_iteration.h:19-22): H and the shifts go in, the eigenvector block
comes out, shifts are reordered only when a restart was needed.  The extended
form returns the per-column status, perturbation flags and scaling factors
that the reference keeps internal.  ``inverse_iteration_device`` runs on
device-resident torch tensors (inputs already in HBM).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class HsrError(RuntimeError):
    def __init__(self, status: int):
        lib = _lib.load()
        super().__init__("hsrq3in_gb300 status %d: %s" % (status, lib.hsr_status_string(status).decode()))
        self.status = status


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def tiled_inverse_iteration(H: np.ndarray, wr: np.ndarray, tlsz: int, rhs_tlsz: int,
                            vr: np.ndarray | None = None):
    """The drop-in call, exactly as a C caller makes it.  Returns (vr, wr)."""
    lib = _lib.load()
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.array(wr, dtype=np.float64, copy=True)
    if vr is None:
        vr = np.zeros((n, wr.shape[0]), dtype=np.float64, order="F")
    lib.tiled_inverse_iteration(n, H.ctypes.data, H.shape[0], wr.shape[0], wr.ctypes.data,
                                int(tlsz), int(rhs_tlsz), vr.ctypes.data, vr.shape[0])
    st = lib.hsr_last_status()
    if st < 0:
        raise HsrError(st)
    return vr, wr


def _scaling(scaling: str) -> int:
    if scaling not in ("pow2", "double"):
        raise ValueError("scaling must be 'pow2' or 'double'")
    return _lib.HSR_SCALING_POW2 if scaling == "pow2" else _lib.HSR_SCALING_DOUBLE


def inverse_iteration(H: np.ndarray, wr: np.ndarray, tlsz: int, rhs_tlsz: int = 64,
                      scaling: str = "pow2", rhs: np.ndarray | None = None,
                      max_restarts: int = -1, hbm_budget_bytes: float = 0.0):
    """Extended call.  Returns a dict with vr, wr, status, perturbed, scale,
    tile_scales (num_tiles x nrhs), norm and the library status code.
    scaling: "pow2" (default, base-2 exponents) or "double" (the reference's
    default build)."""
    lib = _lib.load()
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.array(wr, dtype=np.float64, copy=True)
    nrhs = wr.shape[0]
    T = (n + tlsz - 1) // tlsz
    if rhs is not None:
        vr = np.array(rhs, dtype=np.float64, order="F", copy=True)
    else:
        vr = np.zeros((n, nrhs), dtype=np.float64, order="F")
    status = np.zeros(max(nrhs, 1), dtype=np.int32)
    pert = np.zeros(max(nrhs, 1), dtype=np.uint8)
    scale = np.zeros(max(nrhs, 1), dtype=np.float64)
    norm = np.zeros(max(nrhs, 1), dtype=np.float64)
    tiles = np.zeros(max(T * nrhs, 1), dtype=np.float64)
    opt = _lib.Options(_scaling(scaling), int(rhs is not None), int(max_restarts), float(hbm_budget_bytes))
    info = _lib.ColumnInfo(_ptr(status, C.c_int), _ptr(pert, C.c_ubyte), _ptr(scale, C.c_double),
                           _ptr(tiles, C.c_double), _ptr(norm, C.c_double))
    rc = lib.hsr_inverse_iteration_ex(n, H.ctypes.data, H.shape[0], nrhs, wr.ctypes.data, int(tlsz),
                                      int(rhs_tlsz), vr.ctypes.data, vr.shape[0], C.byref(opt), C.byref(info))
    if rc < 0:
        raise HsrError(rc)
    return dict(vr=vr, wr=wr, status=status[:nrhs], perturbed=pert[:nrhs].astype(bool),
                scale=scale[:nrhs], norm=norm[:nrhs], tile_scales=tiles[:T * nrhs].reshape(T, nrhs),
                rc=rc, launches=lib.hsr_last_launch_count())


def inverse_iteration_device(dH, dwr, dvr, tlsz: int, stream=None, scaling: str = "pow2",
                             user_rhs: bool = False, d_status=None, d_scale=None) -> int:
    """Device-resident call on torch tensors (column-major views: pass
    tensors whose .T is contiguous, i.e. created as (cols, rows) and
    transposed).  Returns the status code."""
    lib = _lib.load()
    n = dH.shape[0]
    ldh = dH.stride(1)
    ldv = dvr.stride(1)
    nrhs = dwr.shape[0]
    opt = _lib.Options(_scaling(scaling), int(bool(user_rhs)), -1, 0.0)
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_inverse_iteration_device(n, dH.data_ptr(), ldh, nrhs, dwr.data_ptr(), int(tlsz),
                                          dvr.data_ptr(), ldv, C.byref(opt), st,
                                          None if d_status is None else d_status.data_ptr(),
                                          None if d_scale is None else d_scale.data_ptr())
    return rc


def fp64_peak(ms_target: float = 50.0):
    """(DFMA GFLOP/s, DMMA GFLOP/s) measured on the current GPU."""
    lib = _lib.load()
    a, b = C.c_double(), C.c_double()
    rc = lib.hsr_probe_fp64_peak(float(ms_target), C.byref(a), C.byref(b))
    if rc != 0:
        raise HsrError(rc)
    return a.value, b.value


def last_launch_count() -> int:
    return int(_lib.load().hsr_last_launch_count())
