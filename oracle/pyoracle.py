"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``.  Provides:

* ``oracle_inverse_iteration`` / ``oracle_solve_rhs`` -- the C restatement in
  ``oracle/hsro.c`` (variants ``ref``, ``fma``, ``ref_fast``);
* ``reference_inverse_iteration`` -- the unmodified reference compiled into
  ``oracle/_ref`` (only where its sources were present at build time), with
  the protection decisions its shim recorded;
* ``residuals`` / ``eigvec_angles`` -- the check of validation.c:145-166
  restated with overflow-safe (scaled) norms, and sign-fixed angles.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIBS: dict[str, C.CDLL] = {}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_dp1 = np.ctypeslib.ndpointer(dtype=np.float64, ndim=1, flags="C_CONTIGUOUS")


class Stats(C.Structure):
    _fields_ = [("perturbations", C.c_long), ("div_rescales", C.c_long),
                ("solve_rescales", C.c_long), ("part1_rescales", C.c_long),
                ("part2_rescales", C.c_long), ("consistency_rescales", C.c_long),
                ("restarts", C.c_long), ("nonconverged", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def _lib(variant: str) -> C.CDLL:
    if variant not in _LIBS:
        paths = _build.build_oracle()
        lib = C.CDLL(paths[variant])
        for fn in (lib.hsro_inverse_iteration, lib.hsro_solve_rhs):
            fn.restype = C.c_int
        lib.hsro_dlange_inf.restype = C.c_double
        lib.hsro_dlange_inf.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int]
        lib.hsro_protect_update.restype = C.c_double
        lib.hsro_protect_update.argtypes = [C.c_double] * 3 + [C.c_int]
        lib.hsro_dlartg.restype = None
        lib.hsro_dlartg.argtypes = [C.c_double, C.c_double] + [C.POINTER(C.c_double)] * 3
        lib.hsro_set_threads.argtypes = [C.c_int]
        lib.hsro_set_pivot_log.argtypes = [C.c_void_p]
        lib.hsro_set_pivot_log.restype = None
        lib.hsro_inverse_iteration_cplx.restype = C.c_int
        lib.hsro_cgivens.restype = None
        lib.hsro_cgivens.argtypes = [C.c_double] * 3 + [C.POINTER(C.c_double)] * 3
        lib.hsro_robust_cmplx_div.restype = C.c_int
        lib.hsro_robust_cmplx_div.argtypes = [C.c_double] * 5 + [C.POINTER(C.c_double)] * 3 + [C.c_int]
        lib.hsro_csolve_1x1.restype = C.c_int
        lib.hsro_csolve_1x1.argtypes = [C.c_double] * 5 + [C.POINTER(C.c_double)] * 3 + [C.c_int]
        _LIBS[variant] = lib
    return _LIBS[variant]


def set_threads(n: int, variant: str = "ref") -> None:
    _lib(variant).hsro_set_threads(int(n))


def _call(fn_name: str, H, wr, tlsz, rhs_tlsz, vr, intscale, variant):
    lib = _lib(variant)
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.ascontiguousarray(wr, dtype=np.float64).copy()
    nrhs = wr.shape[0]
    pert = np.zeros(max(nrhs, 1), dtype=np.uint8)
    colscale = np.zeros(max(nrhs, 1), dtype=np.float64)
    status = np.zeros(max(nrhs, 1), dtype=np.int32)
    st = Stats()
    fn = getattr(lib, fn_name)
    rc = fn(C.c_int(n), H.ctypes.data_as(C.c_void_p), C.c_int(H.shape[0]),
            C.c_int(nrhs), wr.ctypes.data_as(C.c_void_p), C.c_int(tlsz),
            C.c_int(rhs_tlsz), vr.ctypes.data_as(C.c_void_p), C.c_int(vr.shape[0]),
            C.c_int(intscale), pert.ctypes.data_as(C.c_void_p),
            colscale.ctypes.data_as(C.c_void_p), status.ctypes.data_as(C.c_void_p),
            C.byref(st))
    if rc != 0:
        raise RuntimeError("%s failed with %d" % (fn_name, rc))
    return dict(vr=vr, wr=wr, perturbed=pert[:nrhs].astype(bool),
                colscale=colscale[:nrhs], status=status[:nrhs], stats=st.as_dict())


def oracle_inverse_iteration(H, wr, tlsz, rhs_tlsz, intscale=0, variant="ref", pivot_log=False):
    """pivot_log: also return ``pivot``, per output column the smallest
    |t - lambda| / smin over its 1x1 solves (< 1 exactly where the column was
    perturbed), which tells how close each perturbation decision was."""
    n = np.asarray(H).shape[0]
    vr = np.zeros((n, len(wr)), dtype=np.float64, order="F")
    if not pivot_log:
        return _call("hsro_inverse_iteration", H, wr, tlsz, rhs_tlsz, vr, intscale, variant)
    lib = _lib(variant)
    piv = np.full(max(len(wr), 1), np.inf)
    lib.hsro_set_pivot_log(piv.ctypes.data_as(C.c_void_p))
    try:
        out = _call("hsro_inverse_iteration", H, wr, tlsz, rhs_tlsz, vr, intscale, variant)
    finally:
        lib.hsro_set_pivot_log(None)
    out["pivot"] = piv[:len(wr)]
    return out


def oracle_solve_rhs(H, wr, rhs, tlsz, rhs_tlsz, intscale=0, variant="ref"):
    vr = np.array(rhs, dtype=np.float64, order="F", copy=True)
    return _call("hsro_solve_rhs", H, wr, tlsz, rhs_tlsz, vr, intscale, variant)


def oracle_dlartg(f: float, g: float):
    lib = _lib("ref")
    c, s, r = C.c_double(), C.c_double(), C.c_double()
    lib.hsro_dlartg(f, g, C.byref(c), C.byref(s), C.byref(r))
    return c.value, s.value, r.value


def oracle_inverse_iteration_cplx(H, wr, wi, tlsz, rhs_tlsz, intscale=0, max_restarts=-1,
                                  variant="fma"):
    """Complex-conjugate shifts (oracle/hsro_cplx.c): one pair per (wr[k], wi[k]);
    returns vr (n x 2*npairs, Re/Im column pairs), the complex vectors X
    (n x npairs), and per-pair flags."""
    lib = _lib(variant)
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    wi = np.ascontiguousarray(wi, dtype=np.float64)
    npairs = wr.shape[0]
    vr = np.zeros((n, 2 * npairs), dtype=np.float64, order="F")
    pert = np.zeros(max(npairs, 1), dtype=np.uint8)
    colscale = np.zeros(max(npairs, 1), dtype=np.float64)
    status = np.zeros(max(npairs, 1), dtype=np.int32)
    st = Stats()
    rc = lib.hsro_inverse_iteration_cplx(
        C.c_int(n), H.ctypes.data_as(C.c_void_p), C.c_int(n), C.c_int(npairs),
        wr.ctypes.data_as(C.c_void_p), wi.ctypes.data_as(C.c_void_p), C.c_int(tlsz),
        C.c_int(rhs_tlsz), vr.ctypes.data_as(C.c_void_p), C.c_int(n), C.c_int(intscale),
        C.c_int(max_restarts), pert.ctypes.data_as(C.c_void_p),
        colscale.ctypes.data_as(C.c_void_p), status.ctypes.data_as(C.c_void_p), C.byref(st))
    if rc != 0:
        raise RuntimeError("hsro_inverse_iteration_cplx failed with %d" % rc)
    return dict(vr=vr, X=vr[:, 0::2] + 1j * vr[:, 1::2], perturbed=pert[:npairs].astype(bool),
                colscale=colscale[:npairs], status=status[:npairs], stats=st.as_dict())


def oracle_cgivens(fr: float, fi: float, g: float):
    c, sr, si = C.c_double(), C.c_double(), C.c_double()
    _lib("fma").hsro_cgivens(fr, fi, g, C.byref(c), C.byref(sr), C.byref(si))
    return c.value, sr.value, si.value


def oracle_robust_cmplx_div(smin, a, b, c, d, intscale=0):
    xr, xi, sc = C.c_double(), C.c_double(), C.c_double()
    info = _lib("fma").hsro_robust_cmplx_div(smin, a, b, c, d, C.byref(xr), C.byref(xi),
                                             C.byref(sc), intscale)
    return info, xr.value, xi.value, sc.value


def oracle_csolve_1x1(smin, tr, ti, lr, li, xr, xi, intscale=0):
    pr, pi, sc = C.c_double(xr), C.c_double(xi), C.c_double()
    info = _lib("fma").hsro_csolve_1x1(smin, tr, ti, lr, li, C.byref(pr), C.byref(pi),
                                       C.byref(sc), intscale)
    return info, pr.value, pi.value, sc.value


# ---------------------------------------------------------------- reference
def reference_available() -> bool:
    return os.path.exists(os.path.join(_build.REF_DIR, "libhsrq3in_ref.so")) or \
        os.path.isdir(_build.REFERENCE_SRC)


def _ref_lib(intscale: int) -> C.CDLL:
    key = "reference_int" if intscale else "reference"
    if key not in _LIBS:
        paths = _build.build_reference()
        p = paths.get("ref_int" if intscale else "ref")
        if p is None:
            raise RuntimeError("reference sources are not available on this host")
        lib = C.CDLL(p)
        lib.tiled_inverse_iteration.restype = None
        lib.hsr_ref_shim_events.restype = C.c_long
        lib.hsr_ref_set_blas_threads.argtypes = [C.c_int]
        lib.hsr_ref_set_blas_threads(1)
        _LIBS[key] = lib
    return _LIBS[key]


def reference_inverse_iteration(H, wr, tlsz, rhs_tlsz, intscale=0):
    """Run the unmodified reference; returns vr, wr (possibly reordered) and
    the recorded protection decisions."""
    lib = _ref_lib(intscale)
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    wr = np.ascontiguousarray(wr, dtype=np.float64).copy()
    nrhs = wr.shape[0]
    vr = np.zeros((n, nrhs), dtype=np.float64, order="F")
    lib.hsr_ref_shim_reset()
    lib.tiled_inverse_iteration(C.c_int(n), H.ctypes.data_as(C.c_void_p), C.c_int(n),
                                C.c_int(nrhs), wr.ctypes.data_as(C.c_void_p),
                                C.c_int(tlsz), C.c_int(rhs_tlsz),
                                vr.ctypes.data_as(C.c_void_p), C.c_int(n))
    counts = (C.c_long * 6)()
    lib.hsr_ref_shim_counts(counts)
    maxev = 1 << 20
    kind = np.zeros(maxev, dtype=np.int32)
    key = np.zeros(maxev, dtype=np.float64)
    val = np.zeros(maxev, dtype=np.float64)
    nev = lib.hsr_ref_shim_events(kind.ctypes.data_as(C.c_void_p), key.ctypes.data_as(C.c_void_p),
                                  val.ctypes.data_as(C.c_void_p), C.c_long(maxev))
    return dict(vr=vr, wr=wr,
                counts=dict(solves=counts[0], perturbations=counts[1], div_rescales=counts[2],
                            solve_rescales=counts[3], part1_rescales=counts[4],
                            part2_rescales=counts[5]),
                events=(kind[:nev], key[:nev], val[:nev]))


# ------------------------------------------------------------------- checks
def scaled_fro(x: np.ndarray, axis=None) -> np.ndarray:
    """Frobenius/2-norm without overflow or underflow (scaled by the max)."""
    a = np.abs(x)
    m = np.max(a, axis=axis, keepdims=True) if axis is not None else np.max(a)
    m = np.where(m > 0, m, 1.0)
    r = m * np.sqrt(np.sum((a / m) ** 2, axis=axis, keepdims=axis is not None))
    return np.squeeze(r, axis=axis) if axis is not None else r


def residuals(H: np.ndarray, wr: np.ndarray, X: np.ndarray) -> np.ndarray:
    """||H x - lambda x|| / (||H||_F ||x||) per column, computed with scaled
    norms so inputs of magnitude 1e300 do not overflow (validation.c:145-166
    divides by (||H||_F + |lambda|) ||x||; the benchmark's acceptance bound
    omits |lambda|, which is the stricter of the two for |lambda| > 0)."""
    H = np.asarray(H)
    hmax = np.max(np.abs(H)) or 1.0
    Hs = H / hmax
    xmax = np.max(np.abs(X), axis=0)
    xmax = np.where(xmax > 0, xmax, 1.0)
    Xs = X / xmax
    R = Hs @ Xs - (wr / hmax)[None, :] * Xs
    num = scaled_fro(R, axis=0)
    den = scaled_fro(Hs) * scaled_fro(Xs, axis=0)
    with np.errstate(invalid="ignore", divide="ignore"):
        return num / den


def normalize_sign(X: np.ndarray) -> np.ndarray:
    """Unit 2-norm columns with the largest-magnitude entry made positive."""
    nrm = scaled_fro(X, axis=0)
    Y = X / np.where(nrm > 0, nrm, 1.0)
    idx = np.argmax(np.abs(Y), axis=0)
    sg = np.sign(Y[idx, np.arange(Y.shape[1])])
    sg = np.where(sg == 0, 1.0, sg)
    return Y * sg


def eigvec_angles(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Angle between corresponding columns (sign-insensitive), radians."""
    A = normalize_sign(X)
    B = normalize_sign(Y)
    c = np.abs(np.sum(A * B, axis=0))
    s = scaled_fro(A - np.sign(np.sum(A * B, axis=0))[None, :] * B, axis=0)
    # small-angle form is accurate where arccos loses digits
    return np.where(c < 0.9, np.arccos(np.clip(c, 0, 1)), 2 * np.arcsin(np.clip(s / 2, 0, 1)))


def phase_angles(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Angle between corresponding columns of complex X and Y, invariant to a
    unit-modulus phase: atan2(||x - y p||, |p|) with p = y^H x for unit x, y
    (accurate for small angles, where arccos loses half the digits)."""
    x = X / scaled_fro(X, axis=0)
    y = Y / scaled_fro(Y, axis=0)
    p = np.sum(np.conj(y) * x, axis=0)
    r = scaled_fro(x - y * p[None, :], axis=0)
    return np.arctan2(r, np.abs(p))


def eig_vectors_for(H: np.ndarray, mu: np.ndarray) -> np.ndarray:
    """Right eigenvectors from LAPACK dgeev (numpy) for the eigenvalues
    nearest each shift in mu (complex), one column per shift."""
    w, V = np.linalg.eig(np.asarray(H))
    idx = [int(np.argmin(np.abs(w - m))) for m in np.atleast_1d(mu)]
    return V[:, idx]


def eigen_sensitivity(H: np.ndarray, wr: np.ndarray) -> np.ndarray:
    """Estimated eigenvector sensitivity eps*||H||_F*kappa_i/gap_i for each
    shift (nearest eigenvalue), from LAPACK dgeev left/right vectors."""
    import scipy.linalg as sl
    w, vl, vr = sl.eig(H, left=True, right=True)
    eps = np.finfo(np.float64).eps
    hf = scaled_fro(H)
    out = np.empty(len(wr))
    for k, mu in enumerate(wr):
        i = int(np.argmin(np.abs(w - mu)))
        s = abs(np.vdot(vl[:, i], vr[:, i])) / (np.linalg.norm(vl[:, i]) * np.linalg.norm(vr[:, i]))
        others = np.delete(w, i)
        gap = np.min(np.abs(others - w[i])) if others.size else 1.0
        out[k] = eps * hf / (s * gap) if s > 0 and gap > 0 else np.inf
    return out


def reference_robust_cmplx_div(smin, a, b, c, d, intscale=0):
    """robust_cmplx_div (robust.c:639-675) of the compiled reference."""
    lib = _ref_lib(intscale)
    fn = lib.robust_cmplx_div
    fn.restype = C.c_int
    xr, xi = C.c_double(), C.c_double()
    sc = C.c_int() if intscale else C.c_double()
    info = fn(C.c_double(smin), C.c_double(a), C.c_double(b), C.c_double(c), C.c_double(d),
              C.byref(xr), C.byref(xi), C.byref(sc))
    return info, xr.value, xi.value, float(sc.value)


def reference_solve_1x1_cmplx(smin, t, lam_re, lam_im, xr, xi, intscale=0):
    """solve_1x1_cmplx_system (robust.c:677-773) of the compiled reference."""
    lib = _ref_lib(intscale)
    fn = lib.solve_1x1_cmplx_system
    fn.restype = C.c_int
    pr, pi = C.c_double(xr), C.c_double(xi)
    sc = C.c_int() if intscale else C.c_double()
    info = fn(C.c_double(smin), C.c_double(t), C.c_double(lam_re), C.c_double(lam_im),
              C.byref(pr), C.byref(pi), C.byref(sc))
    return info, pr.value, pi.value, float(sc.value)
