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


def test_complex_spectrum_pairs_and_structure():
    """2x2 blocks [[a, b r], [-b/r, a]] carry a +- ib: with a small strictly
    upper part the spectrum of H is the prescribed one; pairs come with
    positive imaginary parts in [0.1, 1]; odd orders and n_real add real
    eigenvalues; the result repeats for a seed."""
    H, pairs, lr = G.complex_spectrum(61, 5, upper_scale=0.05, n_real=3)
    assert H.shape == (61, 61) and np.all(np.tril(H, -2) == 0)
    assert len(pairs) == 29 and len(lr) == 3
    assert np.all((pairs.imag >= 0.1) & (pairs.imag <= 1.0))
    want = np.concatenate([pairs, pairs.conj(), lr.astype(complex)])
    got = np.linalg.eigvals(H)
    key = lambda z: (np.round(z.real, 6), np.round(z.imag, 6))
    a = np.array(sorted(want, key=key))
    b = np.array(sorted(got, key=key))
    assert np.max(np.abs(a - b)) < 1e-9
    H2, p2, _ = G.complex_spectrum(61, 5, upper_scale=0.05, n_real=3)
    assert np.array_equal(H, H2) and np.array_equal(pairs, p2)
    H3, p3, l3 = G.complex_spectrum(48, 6)
    assert len(p3) == 24 and len(l3) == 0 and np.all(np.tril(H3, -2) == 0)
