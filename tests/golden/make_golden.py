"""Generate the golden fixtures of tests/golden/ from the unmodified reference.

Run in a checkout where the reference sources are available (they are
compiled into oracle/_ref by oracle/build.py); the fixtures are committed and
the tests read them on any host.  Each driver fixture holds one problem (H, shifts,
tile sizes, scaling build) and the reference's output (eigenvectors, the
possibly reordered shifts, and the protection decisions its shim recorded).
cplx_kernels.npz holds operand rows and the reference's outputs of its two
complex robust kernels, which no reference driver calls.
Every reference run happens in a child process: the reference aborts on some
inputs (its restart path), which must not take this script down.

    python tests/golden/make_golden.py [--n1000-only]
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hsrq3in_gb300 import generators as G  # noqa: E402


def cases():
    H, lam = G.real_spectrum(48, 101)
    yield "real_n48_t12", H, G.perturbed_shifts(lam, 102), 12, 8, 0
    H, lam = G.real_spectrum(100, 103)
    yield "real_n100_t40_ragged", H, G.perturbed_shifts(lam, 104), 40, 16, 0
    H, lam = G.real_spectrum(100, 103)
    yield "real_n100_t40_int", H, G.perturbed_shifts(lam, 104), 40, 16, 1
    H, lam = G.stress(64, 105)
    yield "stress_n64_t16", H, lam, 16, 16, 0
    H, lam = G.well_conditioned(60, 107)
    yield "wellcond_n60_t20", H, lam, 20, 8, 0
    H, wr = G.reduced_triangular(40, 7)
    yield "reduced_n40_t12_int", H, wr, 12, 4, 1
    H, lam = G.real_spectrum(203, 109)
    yield "real_n203_t40_r13", H, G.perturbed_shifts(lam, 110), 40, 13, 0


def _run(args, q):
    name, H, wr, tlsz, rhs, isc = args
    from oracle import pyoracle as O
    r = O.reference_inverse_iteration(H, wr, tlsz, rhs, intscale=isc)
    q.put((r["vr"], r["wr"], r["counts"]))


def _kernel_operands(seed, count, k):
    """Seeded operand rows: every third row with exponents spread over the
    whole double range (subnormal to near overflow), the rest moderate, and
    an exact zero in every seventh row."""
    rng = np.random.default_rng(seed)
    out = np.empty((count, k))
    for it in range(count):
        e = rng.integers(-320, 308, size=k) if it % 3 == 0 else rng.integers(-20, 20, size=k)
        v = rng.standard_normal(k) * 10.0 ** e.astype(float)
        if it % 7 == 0:
            v[rng.integers(0, k)] = 0.0
        out[it] = v
    return out


def _run_kernels(q):
    """Reference outputs of robust_cmplx_div (robust.c:639-675) and
    solve_1x1_cmplx_system (robust.c:677-773), both scaling builds."""
    from oracle import pyoracle as O
    res = {}
    for isc in (0, 1):
        div_in = _kernel_operands(501 + isc, 1000, 5)
        div_in[:, 0] = np.abs(div_in[:, 0])
        res["div_in_%d" % isc] = div_in
        res["div_out_%d" % isc] = np.array([O.reference_robust_cmplx_div(*r, intscale=isc) for r in div_in])
        sol_in = _kernel_operands(511 + isc, 1000, 6)
        sol_in[:, 0] = np.abs(sol_in[:, 0])
        sol_in[sol_in[:, 3] == 0.0, 3] = 1e-3          # the solver passes a nonzero Im(lambda)
        res["sol_in_%d" % isc] = sol_in
        res["sol_out_%d" % isc] = np.array([O.reference_solve_1x1_cmplx(*r, intscale=isc) for r in sol_in])
    q.put(res)


def complex_kernels(ctx):
    q = ctx.Queue()
    p = ctx.Process(target=_run_kernels, args=(q,))
    p.start()
    res = q.get(timeout=600)
    p.join(60)
    out = os.path.join(HERE, "cplx_kernels.npz")
    np.savez_compressed(out, **res)
    print("cplx_kernels: %d rows per kernel and scaling build" % len(res["div_in_0"]))


def pack_hessenberg(H: np.ndarray) -> np.ndarray:
    """The upper-Hessenberg part of H, column by column (rows 0 .. j+1 of
    column j), which is all the solver reads."""
    n = H.shape[0]
    keep = np.arange(n)[:, None] <= np.arange(n)[None, :] + 1        # keep[i, j]: i <= j + 1
    return np.ascontiguousarray(np.asarray(H).T[keep.T])


def unpack_hessenberg(packed: np.ndarray, n: int) -> np.ndarray:
    keep = np.arange(n)[:, None] <= np.arange(n)[None, :] + 1
    Ht = np.zeros((n, n))
    Ht[keep.T] = packed
    return np.asfortranarray(Ht.T)


def flags_from_events(events, wr: np.ndarray, smlnum: float) -> np.ndarray:
    """Per-column perturbation flags from the reference's recorded 1x1-solve
    decisions: each event carries the smin it was taken with, and smin =
    max(eps/2 |mu|, smlnum) (solve-task.c:149) identifies the column."""
    kind, key, _ = events
    smin = np.maximum(np.finfo(np.float64).eps / 2 * np.abs(wr), smlnum)
    hit = set(key[kind == 1].tolist())
    return np.array([s in hit for s in smin], dtype=np.uint8)


def _run_n1000(args, q):
    """Reference solves of one order-1000 problem at (tlsz, rhs_tlsz) and
    (200, 64), with the oracle's pivot log taken on the same input."""
    H, wr, tlsz, rhs, cols, cols_alt = args
    from oracle import pyoracle as O
    r = O.reference_inverse_iteration(H, wr, tlsz, rhs)
    o = O.oracle_inverse_iteration(H, wr, tlsz, rhs, variant="ref", pivot_log=True)
    assert np.array_equal(o["vr"], r["vr"]) and np.array_equal(o["wr"], r["wr"])
    alt = O.reference_inverse_iteration(H, wr, 200, 64) if cols_alt is not None else None
    res = O.residuals(H, r["wr"], r["vr"])
    q.put(dict(vr=r["vr"][:, cols], wr_out=r["wr"], counts=r["counts"], events=r["events"],
               pert_oracle=o["perturbed"].astype(np.uint8), pivot=o["pivot"], residual=res,
               vr_alt=None if alt is None else alt["vr"][:, cols_alt],
               wr_alt=None if alt is None else alt["wr"]))


def n1000_fixtures(ctx):
    """Two order-1000 problems at the benchmark's tiling (tlsz 160, rhs_tlsz
    64), with the reference's output:
      n1000_real_t160: the plain small workload (real-spectrum generator,
        seed 1234, all 1000 eigenvalues with relative 1e-12 noise, seed 1235);
        128 sampled columns of the reference's eigenvectors at this tiling and
        at (200, 64), per-column perturbation flags and pivot log, and the
        eigenvalue sensitivities and relative gaps of every shift;
      n1000_wellcond_t160: the well-conditioned companion (strictly-upper
        entries scaled by 1/n, seed 1234, the exact eigenvalues as shifts);
        160 sampled columns.
    H is stored as its packed upper-Hessenberg part."""
    from oracle import pyoracle as O
    eps = np.finfo(np.float64).eps
    n = 1000
    tiny = np.finfo(np.float64).tiny
    smlnum = max(2 * tiny, tiny * (n / eps))             # shifted_Hessenberg_solve.c:71
    H, lam = G.real_spectrum(n, 1234)
    wr = G.perturbed_shifts(lam, 1235)
    cols = np.linspace(0, n - 1, 128).astype(np.int64)
    specs = [("n1000_real_t160", H, lam, wr, cols, cols)]
    H2, lam2 = G.well_conditioned(n, 1234)
    specs.append(("n1000_wellcond_t160", H2, lam2, lam2.copy(), np.linspace(0, n - 1, 160).astype(np.int64), None))
    for name, Hm, lm, w, cs, ca in specs:
        q = ctx.Queue()
        p = ctx.Process(target=_run_n1000, args=((Hm, w, 160, 64, cs, ca), q))
        p.start()
        out = q.get(timeout=1200)
        p.join(60)
        pert = flags_from_events(out["events"], out["wr_out"], smlnum)
        assert np.array_equal(pert, out["pert_oracle"]), "event flags disagree with the oracle's"
        srt = np.sort(lm)
        gaps = np.minimum(np.abs(np.diff(srt, prepend=-np.inf)), np.abs(np.diff(srt, append=np.inf)))
        idx = np.searchsorted(srt, lm)
        relgap = gaps[idx] / np.abs(lm)
        near = np.array([int(np.argmin(np.abs(lm - m))) for m in out["wr_out"]])
        sens = O.eigen_sensitivity(Hm, out["wr_out"])
        extra = {}
        if out["vr_alt"] is not None:
            assert np.array_equal(out["wr_alt"], out["wr_out"])
            extra = dict(vr_alt=out["vr_alt"], alt_tlsz=200, alt_rhs_tlsz=64)
        c = out["counts"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), Hp=pack_hessenberg(Hm), n=n, wr_in=w,
                            wr_out=out["wr_out"], cols=cs, vr=out["vr"], tlsz=160, rhs_tlsz=64, intscale=0,
                            perturbed=pert, pivot=out["pivot"], residual=out["residual"],
                            relgap=relgap[near], sensitivity=sens,
                            perturbations=c["perturbations"], div_rescales=c["div_rescales"],
                            solve_rescales=c["solve_rescales"], part1_rescales=c["part1_rescales"],
                            part2_rescales=c["part2_rescales"], **extra)
        print("%s: %s, %d perturbed columns" % (name, c, int(pert.sum())))


def main():
    ctx = mp.get_context("spawn")
    if "--n1000-only" in sys.argv:
        n1000_fixtures(ctx)
        return
    complex_kernels(ctx)
    n1000_fixtures(ctx)
    for case in cases():
        name, H, wr, tlsz, rhs, isc = case
        q = ctx.Queue()
        p = ctx.Process(target=_run, args=(case, q))
        p.start()
        try:
            vr, wr_out, counts = q.get(timeout=600)   # drain before join
        except Exception:
            vr = None
        p.join(60)
        if vr is None or p.exitcode != 0:
            print("%s: reference aborted (exit %s); no fixture" % (name, p.exitcode))
            if p.is_alive():
                p.kill()
            continue
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, H=H, wr_in=wr, wr_out=wr_out, vr=vr, tlsz=tlsz, rhs_tlsz=rhs,
                            intscale=isc, perturbations=counts["perturbations"],
                            div_rescales=counts["div_rescales"], solve_rescales=counts["solve_rescales"],
                            part1_rescales=counts["part1_rescales"], part2_rescales=counts["part2_rescales"])
        print("%s: n=%d nrhs=%d %s" % (name, H.shape[0], len(wr), counts))


if __name__ == "__main__":
    main()
