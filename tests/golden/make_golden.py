"""Generate the golden fixtures of tests/golden/ from the unmodified reference.

Run in a checkout where the reference sources are available (they are
compiled into oracle/_ref by oracle/build.py); the fixtures are committed and
the tests read them on any host.  Each fixture holds one problem (H, shifts,
tile sizes, scaling build) and the reference's output (eigenvectors, the
possibly reordered shifts, and the protection decisions its shim recorded).
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


def main():
    ctx = mp.get_context("spawn")
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
