"""The CPU oracle against the reference: golden fixtures (made from the
unmodified reference by tests/golden/make_golden.py), the live reference where
its sources are present, LAPACK's dlartg, and the numerical criteria."""
import glob
import os

import numpy as np
import pytest

from hsrq3in_gb300 import generators as G
from oracle import pyoracle as O

EPS = np.finfo(np.float64).eps
# Driver fixtures: one problem and the reference's solve each (the scalar
# kernel fixture cplx_kernels.npz is checked in test_oracle_cplx.py).
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if os.path.basename(p) != "cplx_kernels.npz" and not os.path.basename(p).startswith("n1000_"))
# Order-1000 fixtures at the benchmark tiling: packed H, sampled columns.
GOLDEN_N1000 = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "n1000_*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_reproduces_reference_golden(path):
    z = np.load(path)
    o = O.oracle_inverse_iteration(z["H"], z["wr_in"], int(z["tlsz"]), int(z["rhs_tlsz"]),
                                   intscale=int(z["intscale"]), variant="ref")
    assert np.array_equal(o["wr"], z["wr_out"])
    assert np.array_equal(o["vr"], z["vr"])                     # bit for bit
    assert o["stats"]["perturbations"] == int(z["perturbations"])
    assert o["stats"]["div_rescales"] == int(z["div_rescales"])
    assert o["stats"]["solve_rescales"] == int(z["solve_rescales"])


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 7
    assert len(GOLDEN_N1000) == 2


def unpack_hessenberg(packed, n):
    keep = np.arange(n)[:, None] <= np.arange(n)[None, :] + 1
    Ht = np.zeros((n, n))
    Ht[keep.T] = packed
    return np.asfortranarray(Ht.T)


@pytest.mark.parametrize("path", GOLDEN_N1000, ids=[os.path.basename(p)[:-4] for p in GOLDEN_N1000])
def test_oracle_reproduces_reference_n1000(path):
    """Order 1000 at tlsz 160, rhs_tlsz 64: the reference's shifts, sampled
    eigenvector columns (bit for bit), per-column perturbation flags (mapped
    from its recorded decisions) and decision counts."""
    z = np.load(path)
    n = int(z["n"])
    H = unpack_hessenberg(z["Hp"], n)
    O.set_threads(os.cpu_count() or 1, "ref")
    o = O.oracle_inverse_iteration(H, z["wr_in"], int(z["tlsz"]), int(z["rhs_tlsz"]), variant="ref",
                                   pivot_log=True)
    assert np.array_equal(o["wr"], z["wr_out"])
    assert np.array_equal(o["vr"][:, z["cols"]], z["vr"])
    assert np.array_equal(o["perturbed"], z["perturbed"].astype(bool))
    assert np.array_equal(o["pivot"], z["pivot"])
    assert o["stats"]["perturbations"] == int(z["perturbations"])
    for k in ("div_rescales", "solve_rescales", "part1_rescales", "part2_rescales"):
        assert o["stats"][k] == int(z[k]) == 0, k
    assert np.all(z["residual"] <= 10 * n * EPS)


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not on this host")
@pytest.mark.parametrize("n,tlsz,rhs,seed,isc", [
    (37, 12, 5, 1, 0), (120, 24, 32, 2, 0), (150, 40, 7, 3, 1), (250, 60, 64, 4, 0),
])
def test_oracle_matches_live_reference(n, tlsz, rhs, seed, isc):
    H, lam = G.real_spectrum(n, seed)
    wr = G.perturbed_shifts(lam, seed + 50)
    r = O.reference_inverse_iteration(H, wr, tlsz, rhs, intscale=isc)
    o = O.oracle_inverse_iteration(H, wr, tlsz, rhs, intscale=isc, variant="ref")
    assert np.array_equal(r["vr"], o["vr"]) and np.array_equal(r["wr"], o["wr"])
    for k in ("perturbations", "div_rescales", "solve_rescales", "part1_rescales", "part2_rescales"):
        assert r["counts"][k] == o["stats"][k], k


def test_dlartg_matches_lapack_bitwise():
    import scipy.linalg.lapack as L
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.standard_normal(3000),
                           rng.standard_normal(1000) * 10.0 ** rng.uniform(-300, 300, 1000),
                           [0.0, -0.0, 1e-310, -1e-310, 1e308, -1e308, 2.0 ** -511, 2.0 ** 510]])
    rng.shuffle(vals)
    f, g = vals[:2000], vals[2000:4000]
    bad = 0
    for a, b in zip(f, g):
        c1, s1, r1 = L.dlartg(a, b)
        c2, s2, r2 = O.oracle_dlartg(float(a), float(b))
        bad += not (c1 == c2 and s1 == s2 and r1 == r2)
    assert bad == 0


@pytest.mark.parametrize("variant", ["ref", "fma", "ref_fast"])
def test_residual_bound(variant):
    """Every variant, including ref_fast (the build the CPU baseline times),
    solves to the residual bound."""
    n = 300
    H, lam = G.real_spectrum(n, 11)
    wr = G.perturbed_shifts(lam, 12)
    o = O.oracle_inverse_iteration(H, wr, 60, 32, variant=variant)
    assert np.all(np.isfinite(o["vr"]))
    assert O.residuals(H, o["wr"], o["vr"]).max() <= 10 * n * EPS


def test_angle_well_conditioned():
    """ref vs fma and ref_fast arithmetic on the well-conditioned companion
    generator."""
    n = 200
    H, lam = G.well_conditioned(n, 13)
    a = O.oracle_inverse_iteration(H, lam, 40, 16, variant="ref")
    b = O.oracle_inverse_iteration(H, lam, 40, 16, variant="fma")
    c = O.oracle_inverse_iteration(H, lam, 40, 16, variant="ref_fast")
    assert np.all(a["status"] == 1) and np.all(c["status"] == 1)
    assert O.eigvec_angles(a["vr"], b["vr"]).max() <= 1e-10
    assert O.eigvec_angles(a["vr"], c["vr"]).max() <= 1e-10


def test_angle_filtered_by_sensitivity():
    """Benchmark generator: angle <= 1e-10 for every eigenpair whose estimated
    sensitivity eps*||H||_F*kappa/gap is <= 1e-12 (the rest are too
    ill-conditioned for any two roundings to agree)."""
    n = 120
    H, lam = G.real_spectrum(n, 14)
    wr = G.perturbed_shifts(lam, 15)
    a = O.oracle_inverse_iteration(H, wr, 24, 16, variant="ref")
    b = O.oracle_inverse_iteration(H, wr, 24, 16, variant="fma")
    sens = O.eigen_sensitivity(H, a["wr"])
    ang = O.eigvec_angles(a["vr"], b["vr"])
    ok = sens <= 1e-12
    assert np.all(ang[ok] <= 1e-10)
    assert np.all(O.residuals(H, b["wr"], b["vr"]) <= 10 * n * EPS)


def test_restart_reorders_stably():
    """Shifts whose single solve does not pass ||y|| > 0.1/sqrt(n) are
    restarted; converged columns come first in their original order."""
    n = 48
    H, lam = G.well_conditioned(n, 3)
    wr = G.perturbed_shifts(lam, 4)
    o = O.oracle_inverse_iteration(H, wr, 16, 16, variant="ref")
    st = o["status"]
    assert o["stats"]["restarts"] > 0
    assert np.all(np.diff(st) <= 0)                      # converged first
    assert sorted(o["wr"]) == sorted(wr)
    # the columns that converged in the first round lead, in their order
    eps3 = O._lib("ref").hsro_dlange_inf(n, n, np.asfortranarray(H).ctypes.data, n) * EPS / 2
    first = O.oracle_solve_rhs(H, wr, np.full((n, n), eps3, order="F"), 16, 16, variant="ref")
    lead = wr[first["status"] == 1]
    assert np.array_equal(o["wr"][:len(lead)], lead)


def test_power_of_two_scaling_stays_finite_where_double_does_not():
    H, wr = G.reduced_triangular(60, 5)
    d = O.oracle_inverse_iteration(H, wr, 20, 4, intscale=0, variant="ref")
    p = O.oracle_inverse_iteration(H, wr, 20, 4, intscale=1, variant="ref")
    assert not np.all(np.isfinite(d["vr"]))
    assert np.all(np.isfinite(p["vr"]))
    assert p["stats"]["div_rescales"] > 0
    assert np.nanmax(O.residuals(H, p["wr"], p["vr"])) <= 10 * 60 * EPS


def test_block_scaled_fires_tile_update_protection():
    H, wr = G.block_scaled(96, 16, 3)
    p = O.oracle_inverse_iteration(H, wr, 16, 4, intscale=1, variant="ref")
    st = p["stats"]
    assert st["part1_rescales"] > 0 and st["part2_rescales"] > 0 and st["consistency_rescales"] > 0
    assert np.all(np.isfinite(p["vr"]))
    assert np.all(O.residuals(H, p["wr"], p["vr"]) <= 10 * 96 * EPS)


def test_both_scalings_identical_without_protection():
    H, lam = G.real_spectrum(150, 16)
    wr = G.perturbed_shifts(lam, 17)
    a = O.oracle_inverse_iteration(H, wr, 32, 16, intscale=0, variant="fma")
    b = O.oracle_inverse_iteration(H, wr, 32, 16, intscale=1, variant="fma")
    assert np.array_equal(a["vr"], b["vr"])


def test_user_rhs_solve_is_residual_small():
    n = 80
    H, lam = G.real_spectrum(n, 18)
    wr = G.perturbed_shifts(lam, 19)
    rhs = G.uniform_rhs(n, n, 20)
    o = O.oracle_solve_rhs(H, wr, rhs, 20, 8, variant="ref")
    assert np.all(np.isfinite(o["vr"]))
