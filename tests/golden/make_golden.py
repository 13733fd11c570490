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

    python tests/golden/make_golden.py
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


def main():
    ctx = mp.get_context("spawn")
    complex_kernels(ctx)
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
