"""Seeded workload generators."""
import numpy as np

from hsrq3in_gb300 import generators as G


def test_jittered_eigenvalues_gap_and_range():
    lam = G.jittered_eigenvalues(5000, np.random.default_rng(0))
    s = np.sort(lam)
    assert s[0] >= -1 and s[-1] <= 1
    assert np.min(np.diff(s)) >= 1e-4


def test_real_spectrum_is_hessenberg_with_prescribed_spectrum():
    H, lam = G.real_spectrum(80, 3)
    assert np.all(np.tril(H, -2) == 0)
    assert np.all(np.diag(H, -1) != 0)
    # eigenvalues of this non-normal family are too ill-conditioned to compare
    # one by one; the trace is exact up to rounding
    assert abs(np.trace(H) - lam.sum()) < 1e-8 * 80
    Hw, lw = G.well_conditioned(80, 3)
    ev = np.sort(np.linalg.eigvals(Hw).real)
    assert np.max(np.abs(ev - np.sort(lw))) < 1e-10


def test_deterministic():
    a = G.real_spectrum(40, 9)[0]
    b = G.real_spectrum(40, 9)[0]
    assert np.array_equal(a, b)


def test_stress_clusters():
    H, lam = G.stress(200, 1)
    c = np.unique(np.round(lam, 10))
    assert len(c) <= 50
    assert np.all(np.tril(H, -2) == 0)
    assert np.max(np.abs(H)) > 1e100


def test_shift_helpers():
    lam = G.jittered_eigenvalues(100, np.random.default_rng(1))
    s = G.perturbed_shifts(lam, 2)
    assert np.max(np.abs(s - lam) / np.abs(lam)) < 1e-10
    sub = G.shift_subset(lam, np.random.default_rng(3), 0.25, 1.0)
    assert 25 <= len(sub) <= 100 and set(sub) <= set(lam)
