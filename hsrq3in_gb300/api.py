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
    tl = int(tlsz) if tlsz else lib.hsr_autotune_plain_tlsz(n)      # 0: the autotuned size
    T = (n + tl - 1) // tl
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
    """Device-resident call on torch tensors.  Column-major blocks are passed
    as tensors of shape (columns, ld) whose rows are the columns: dH is
    (n, ldh), dvr is (nrhs, ldvr), as BatchPlan takes them.  Returns the
    status code (0, or 1 when some columns did not converge); raises on
    errors."""
    lib = _lib.load()
    n = dH.shape[0]
    ldh = dH.stride(0)
    ldv = dvr.stride(0)
    nrhs = dwr.shape[0]
    opt = _lib.Options(_scaling(scaling), int(bool(user_rhs)), -1, 0.0)
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_inverse_iteration_device(n, dH.data_ptr(), ldh, nrhs, dwr.data_ptr(), int(tlsz),
                                          dvr.data_ptr(), ldv, C.byref(opt), st,
                                          None if d_status is None else d_status.data_ptr(),
                                          None if d_scale is None else d_scale.data_ptr())
    if rc < 0:
        raise HsrError(rc)
    return rc


def inverse_iteration_cplx(H: np.ndarray, mu: np.ndarray, tlsz: int, rhs_tlsz: int = 64,
                           scaling: str = "pow2", max_restarts: int = -1,
                           hbm_budget_bytes: float = 0.0):
    """Complex-conjugate shifts: one complex shift per pair (mu, complex array;
    the vector of conj(mu) is the conjugate).  Returns a dict with vr
    (n x 2*npairs, real part in column 2k, imaginary part in 2k+1), X (the
    complex vectors, n x npairs), per-pair status, perturbed, scale, norm and
    the library status code.  Shifts keep their order."""
    lib = _lib.load()
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    mu = np.asarray(mu, dtype=np.complex128)
    wr = np.ascontiguousarray(mu.real)
    wi = np.ascontiguousarray(mu.imag)
    npairs = mu.shape[0]
    vr = np.zeros((n, 2 * npairs), dtype=np.float64, order="F")
    status = np.zeros(max(npairs, 1), dtype=np.int32)
    pert = np.zeros(max(npairs, 1), dtype=np.uint8)
    scale = np.zeros(max(npairs, 1), dtype=np.float64)
    norm = np.zeros(max(npairs, 1), dtype=np.float64)
    opt = _lib.Options(_scaling(scaling), 0, int(max_restarts), float(hbm_budget_bytes))
    info = _lib.ColumnInfo(_ptr(status, C.c_int), _ptr(pert, C.c_ubyte), _ptr(scale, C.c_double),
                           None, _ptr(norm, C.c_double))
    rc = lib.hsr_inverse_iteration_cplx_ex(n, H.ctypes.data, H.shape[0], npairs, wr.ctypes.data, wi.ctypes.data,
                                           int(tlsz), int(rhs_tlsz), vr.ctypes.data, vr.shape[0], C.byref(opt),
                                           C.byref(info))
    if rc < 0:
        raise HsrError(rc)
    return dict(vr=vr, X=vr[:, 0::2] + 1j * vr[:, 1::2], status=status[:npairs],
                perturbed=pert[:npairs].astype(bool), scale=scale[:npairs], norm=norm[:npairs], rc=rc,
                launches=lib.hsr_last_launch_count())


def inverse_iteration_mixed(H: np.ndarray, wr: np.ndarray, wi: np.ndarray, tlsz: int, rhs_tlsz: int = 64,
                            scaling: str = "pow2", max_restarts: int = -1):
    """Real eigenvalues and conjugate pairs in one call (LAPACK dhsein layout:
    a pair is two consecutive entries (a, b), (a, -b) with b > 0).  Returns a
    dict with vr (n x m: column k for a real shift; columns k, k+1 the real and
    imaginary parts for a pair), wr (real shifts possibly reordered among the
    real positions), wi, per-column status and the library status code."""
    lib = _lib.load()
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.array(wr, dtype=np.float64, copy=True)
    wi = np.array(wi, dtype=np.float64, copy=True)
    m = wr.shape[0]
    vr = np.zeros((n, m), dtype=np.float64, order="F")
    status = np.zeros(max(m, 1), dtype=np.int32)
    opt = _lib.Options(_scaling(scaling), 0, int(max_restarts), 0.0)
    rc = lib.hsr_inverse_iteration_mixed(n, H.ctypes.data, H.shape[0], m, wr.ctypes.data, wi.ctypes.data, int(tlsz),
                                         int(rhs_tlsz), vr.ctypes.data, vr.shape[0], C.byref(opt),
                                         status.ctypes.data)
    if rc < 0:
        raise HsrError(rc)
    return dict(vr=vr, wr=wr, wi=wi, status=status[:m], rc=rc)


def inverse_iteration_cplx_device(dH, dwr, dwi, dvr, tlsz: int, stream=None, scaling: str = "pow2",
                                  d_status=None, d_scale=None) -> int:
    """Device-resident complex-shift call on torch tensors: dH (n, ldh) as in
    inverse_iteration_device, dwr/dwi (npairs,), dvr (2*npairs, ldvr) whose
    rows 2k and 2k+1 receive the real and imaginary parts.  Returns the status
    code; raises on errors."""
    lib = _lib.load()
    n = dH.shape[0]
    opt = _lib.Options(_scaling(scaling), 0, -1, 0.0)
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_inverse_iteration_cplx_device(n, dH.data_ptr(), dH.stride(0), dwr.shape[0], dwr.data_ptr(),
                                               dwi.data_ptr(), int(tlsz), dvr.data_ptr(), dvr.stride(0),
                                               C.byref(opt), st,
                                               None if d_status is None else d_status.data_ptr(),
                                               None if d_scale is None else d_scale.data_ptr())
    if rc < 0:
        raise HsrError(rc)
    return rc


def residuals_device(dH, dwr, dvr, stream=None):
    """||H x_k - wr_k x_k|| / (||H||_F ||x_k||) per column, on the device.
    Tensors as for inverse_iteration_device: dH (n, ldh), dvr (ncols, ldvr)
    with rows = columns, dwr (ncols,).  Returns a float64 device tensor."""
    import torch
    lib = _lib.load()
    n = dH.shape[0]
    ncols = dwr.shape[0]
    res = torch.empty(ncols, dtype=torch.float64, device=dH.device)
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_residuals_device(n, dH.data_ptr(), dH.stride(0), ncols, dwr.data_ptr(), dvr.data_ptr(),
                                  dvr.stride(0), res.data_ptr(), st)
    if rc < 0:
        raise HsrError(rc)
    return res


def hessenberg_device(dA, stream=None):
    """Reduce the dense matrix in dA (tensor (n, lda), rows = columns) to
    upper-Hessenberg form in place, LAPACK layout (H on and above the
    subdiagonal, reflectors below).  Returns the device tensor of tau."""
    import torch
    lib = _lib.load()
    n = dA.shape[0]
    tau = torch.empty(n, dtype=torch.float64, device=dA.device)
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_hessenberg_device(n, dA.data_ptr(), dA.stride(0), tau.data_ptr(), st)
    if rc < 0:
        raise HsrError(rc)
    return tau


def hessenberg_apply_q_device(dA, dtau, dX, stream=None):
    """X <- Q X in place for the reduction stored in dA, dtau (dX: tensor
    (ncols, ldx), rows = columns)."""
    lib = _lib.load()
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.hsr_hessenberg_apply_q_device(dA.shape[0], dA.data_ptr(), dA.stride(0), dtau.data_ptr(),
                                           dX.shape[0], dX.data_ptr(), dX.stride(0), st)
    if rc < 0:
        raise HsrError(rc)


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


# ----------------------------------------------------------------- batched
class BatchPlan:
    """Many independent problems solved together (hsr_batch_plan_*).

    problems: list of (dH, dwr, dvr) torch tensors on the device, where dH and
    dvr are column-major views (tensors of shape (cols, ld) holding columns as
    rows).  tlsz=0 uses the autotuned tile size.  engine: "ticks" (a graph of
    per-phase launches, all problems in lock step) or "queue" (one persistent
    launch over a device work queue with per-problem dependencies)."""

    def __init__(self, problems, tlsz: int = 0, scaling: str = "pow2", stream=None, engine: str = "ticks"):
        lib = _lib.load()
        self._lib = lib
        self._keep = problems
        arr = (_lib.BatchProblem * max(len(problems), 1))()
        for i, (dH, dwr, dvr) in enumerate(problems):
            n = dH.shape[0]
            arr[i] = _lib.BatchProblem(n, dH.data_ptr(), dH.stride(0), dwr.numel(), dwr.data_ptr(),
                                       dvr.data_ptr(), dvr.stride(0))
        self._arr = arr
        self._stream = stream
        opt = _lib.Options(_scaling(scaling), 0, -1, 0.0)
        h = C.c_void_p()
        rc = lib.hsr_batch_plan_create(C.byref(h), len(problems), arr, int(tlsz), C.byref(opt),
                                       None if stream is None else C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise HsrError(rc)
        self._h = h
        self.set_engine(engine)

    def set_engine(self, engine: str):
        code = {"ticks": _lib.HSR_BATCH_ENGINE_TICKS, "queue": _lib.HSR_BATCH_ENGINE_QUEUE}[engine]
        rc = self._lib.hsr_batch_plan_set_engine(self._h, code, None if self._stream is None
                                                 else C.c_void_p(self._stream.cuda_stream))
        if rc != 0:
            raise HsrError(rc)

    def queue_info(self):
        e, it, g, dw, ig = C.c_int(), C.c_long(), C.c_int(), C.c_int(), C.c_int()
        self._lib.hsr_batch_plan_queue_info(self._h, C.byref(e), C.byref(it), C.byref(g), C.byref(dw), C.byref(ig))
        return dict(engine="queue" if e.value == _lib.HSR_BATCH_ENGINE_QUEUE else "ticks", items=it.value,
                    grid=g.value, diag_warps=dw.value, in_graph=bool(ig.value))

    def execute(self) -> int:
        rc = self._lib.hsr_batch_plan_execute(self._h, None if self._stream is None
                                              else C.c_void_p(self._stream.cuda_stream))
        if rc < 0:
            raise HsrError(rc)
        return rc

    def info(self):
        t, k, n = C.c_int(), C.c_int(), C.c_long()
        self._lib.hsr_batch_plan_info(self._h, C.byref(t), C.byref(k), C.byref(n))
        return dict(tlsz=t.value, ticks=k.value, launches=n.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hsr_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_plain(dH, dwr, dvr, candidates=(64, 96, 128, 160, 200), stream=None, detail=False):
    """Time the plain device path on this problem for each candidate tile
    size, then 8/16/32 shifts per diagonal CTA at the fastest, then (with 8
    or 16) the top GEMM of each tile's rows inside the diagonal CTAs or as
    its own launch (dwr restored, dvr overwritten); records all three (used
    when tlsz=0 is passed) and returns (best tlsz, [ms per candidate]), plus
    (shifts per CTA, [ms for 8, 16, 32], fused (bool), [ms separate, ms
    fused]) when detail is set (-1 ms where the form does not apply)."""
    lib = _lib.load()
    n = dH.shape[0]
    cand = (C.c_int * len(candidates))(*candidates)
    ms = (C.c_double * len(candidates))()
    sc = C.c_int()
    scms = (C.c_double * 3)()
    fz = C.c_int()
    fzms = (C.c_double * 2)()
    best = lib.hsr_autotune_plain(n, dH.data_ptr(), dH.stride(0), dwr.numel(), dwr.data_ptr(), dvr.data_ptr(),
                                  dvr.stride(0), cand, len(candidates), ms, C.byref(sc), scms, C.byref(fz), fzms,
                                  None if stream is None else C.c_void_p(stream.cuda_stream))
    if best < 0:
        raise HsrError(best)
    if detail:
        return best, list(ms), sc.value, list(scms), bool(fz.value), list(fzms)
    return best, list(ms)


def autotune_batch(problems, candidates=(32, 48, 64, 96, 128), stream=None):
    """Time the batch for each candidate tile size; records and returns the
    fastest, with the per-candidate times in ms."""
    lib = _lib.load()
    arr = (_lib.BatchProblem * len(problems))()
    for i, (dH, dwr, dvr) in enumerate(problems):
        arr[i] = _lib.BatchProblem(dH.shape[0], dH.data_ptr(), dH.stride(0), dwr.numel(), dwr.data_ptr(),
                                   dvr.data_ptr(), dvr.stride(0))
    cand = (C.c_int * len(candidates))(*candidates)
    ms = (C.c_double * len(candidates))()
    best = lib.hsr_autotune_batch(len(problems), arr, cand, len(candidates), ms,
                                  None if stream is None else C.c_void_p(stream.cuda_stream))
    if best < 0:
        raise HsrError(best)
    return best, list(ms)


# ----------------------------------------------------------------- served
class Server:
    """The request loop with continuous batching (hsr_server_*)."""

    def __init__(self, hbm_budget_bytes: float = 0.0, tlsz: int = 0, max_active: int = 0,
                 scaling: str = "pow2"):
        lib = _lib.load()
        self._lib = lib
        cfg = _lib.ServerConfig(float(hbm_budget_bytes), int(tlsz), int(max_active), _scaling(scaling))
        h = C.c_void_p()
        rc = lib.hsr_server_create(C.byref(h), C.byref(cfg))
        if rc != 0:
            raise HsrError(rc)
        self._h = h

    def replay(self, requests):
        """requests: list of dict(H=host Fortran array, wr=host array (in/out),
        vr=host Fortran array (out), arrival_s=float).  Host arrays should be
        pinned for copy/compute overlap.  Returns (latencies_s, statuses, stats)."""
        n = len(requests)
        arr = (_lib.Request * max(n, 1))()
        def ld(a):
            # column-major view: unit row stride, column stride = leading dimension
            if a.strides[0] != 8:
                raise ValueError("request blocks must be column-major float64 views")
            return a.strides[1] // 8 if a.shape[1] > 1 else a.shape[0]

        for i, r in enumerate(requests):
            H, wr, vr = r["H"], r["wr"], r["vr"]
            arr[i] = _lib.Request(H.shape[0], H.ctypes.data, ld(H), wr.shape[0], wr.ctypes.data, vr.ctypes.data,
                                  ld(vr), float(r["arrival_s"]))
        lat = (C.c_double * max(n, 1))()
        st = (C.c_int * max(n, 1))()
        stats = _lib.ServerStats()
        rc = self._lib.hsr_server_replay(self._h, n, arr, lat, st, C.byref(stats))
        if rc < 0:
            raise HsrError(rc)
        return (list(lat)[:n], list(st)[:n],
                dict(wall_s=stats.wall_s, ticks=stats.ticks, launches=stats.launches,
                     max_active=stats.max_active, peak_bytes=stats.peak_bytes))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hsr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
