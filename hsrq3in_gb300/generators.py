"""Seeded synthetic inputs for the inverse-iteration workloads.

These generators build upper-Hessenberg matrices with a prescribed real
spectrum.  The reference's own generator (problemgenerator.c:305-362) draws
eigenvalues 1..n and U[0,1) strictly-upper entries and calls rand() inside
OpenMP tasks, so its output changes with the thread count; the workloads here
instead follow the published benchmark configuration:

* ``real_spectrum(n, seed)`` -- T upper triangular with diagonal lambda_i in
  [-1, 1] (distinct, minimum gap >= 1e-4, drawn as a jittered grid because n
  uniform draws on [-1, 1] have an expected minimum gap of ~2/n^2) and N(0,1)
  strictly-upper entries; H = hess(Q T Q^T) for a random orthogonal Q.
  H depends on Q only through q = Q^T e1 (implicit-Q theorem), so Q is taken
  as the Householder reflector that maps e1 to a uniformly random unit vector,
  which gives the Haar-random case at the cost of one reduction.
* ``stress(n, seed)`` -- 50 eigenvalue clusters of width 1e-13 and strictly
  upper columns scaled by 10^k, k ~ U[0, 150].
* ``well_conditioned(n, seed)`` -- the same construction with strictly-upper
  entries scaled by 1/n, so eigenvector angles are meaningful for parity.
* ``complex_spectrum(n, seed)`` -- T quasi-upper triangular with 2x2 blocks
  [[a, b r], [-b / r, a]] (eigenvalues a +- i b, a on a jittered grid in
  [-1, 1], b in [0.1, 1], r in [0.5, 2]) and N(0,1) entries above the
  blocks, reduced to Hessenberg form the same way; the shifts of the
  complex-shift path are the eigenvalues with positive imaginary part.
* shift helpers: all eigenvalues with relative 1e-12 N(0,1) noise, or a
  random subset.

The O(n^3) Hessenberg reduction runs on the host (LAPACK dgehrd through
scipy).  Inputs are returned as Fortran-ordered float64 arrays.
"""
from __future__ import annotations

import numpy as np


def jittered_eigenvalues(n: int, rng: np.random.Generator, lo: float = -1.0,
                         hi: float = 1.0, min_gap: float = 1e-4) -> np.ndarray:
    """n distinct values in [lo, hi] with pairwise gap >= min_gap, shuffled."""
    spacing = (hi - lo) / n
    if spacing <= min_gap:
        raise ValueError("cannot place %d values with gap %g in [%g, %g]" % (n, min_gap, lo, hi))
    jit = 0.5 * (spacing - min_gap)
    lam = lo + spacing * (np.arange(n) + 0.5) + rng.uniform(-jit, jit, n)
    rng.shuffle(lam)
    return lam


def _hessenberg_similarity(T: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """hess(Q T Q^T) with Q^T e1 uniform on the unit sphere."""
    import scipy.linalg as sl
    n = T.shape[0]
    q = rng.standard_normal(n)
    q /= np.linalg.norm(q)
    w = -q.copy()
    w[0] += 1.0
    nw = np.linalg.norm(w)
    A = np.array(T, dtype=np.float64, order="F")
    if nw > 0 and n > 1:
        w /= nw
        # A := P T P with P = I - 2 w w^T (P e1 = q)
        A -= 2.0 * np.outer(w, w @ A)
        A -= 2.0 * np.outer(A @ w, w)
    H = sl.hessenberg(A, overwrite_a=True, check_finite=False)
    return np.asfortranarray(np.triu(H, -1))


def real_spectrum(n: int, seed: int, upper_scale: float = 1.0):
    """(H, lambda) for the real-spectrum workload of order n."""
    rng = np.random.default_rng(seed)
    lam = jittered_eigenvalues(n, rng)
    T = np.triu(rng.standard_normal((n, n)) * upper_scale, 1)
    T[np.diag_indices(n)] = lam
    return _hessenberg_similarity(T, rng), lam


def well_conditioned(n: int, seed: int):
    """Same construction with strictly-upper entries scaled by 1/n."""
    return real_spectrum(n, seed, upper_scale=1.0 / n)


def stress(n: int, seed: int, clusters: int = 50, width: float = 1e-13,
           max_exp: float = 150.0):
    """(H, lambda): clustered spectrum, strictly-upper columns scaled 10^k."""
    rng = np.random.default_rng(seed)
    centers = jittered_eigenvalues(clusters, rng, min_gap=1e-3)
    lam = np.empty(n)
    for c in range(clusters):
        idx = np.arange(c, n, clusters)
        lam[idx] = centers[c] + rng.uniform(-0.5 * width, 0.5 * width, idx.size)
    rng.shuffle(lam)
    k = rng.uniform(0.0, max_exp, n)
    T = np.triu(rng.standard_normal((n, n)) * (10.0 ** k)[None, :], 1)
    T[np.diag_indices(n)] = lam
    return _hessenberg_similarity(T, rng), lam


def complex_spectrum(n: int, seed: int, upper_scale: float = 1.0, n_real: int = 0):
    """(H, pairs, lam_real): H of order n with (n - n_real) // 2 complex
    conjugate pairs, returned as the eigenvalues with positive imaginary part
    (complex array), and n_real (+1 when n - n_real is odd) real eigenvalues."""
    rng = np.random.default_rng(seed)
    npairs = (n - n_real) // 2
    nreal = n - 2 * npairs
    a = jittered_eigenvalues(npairs, rng) if npairs else np.zeros(0)
    b = rng.uniform(0.1, 1.0, npairs)
    r = np.exp(rng.uniform(np.log(0.5), np.log(2.0), npairs))
    lam_r = jittered_eigenvalues(nreal, rng, min_gap=1e-6) if nreal else np.zeros(0)
    # Diagonal blocks in random order: 2 = a pair, 1 = a real eigenvalue.
    kinds = np.array([2] * npairs + [1] * nreal)
    order = rng.permutation(kinds.size)
    T = np.triu(rng.standard_normal((n, n)) * upper_scale, 1)
    pos = 0
    ip = ir = 0
    for o in order:
        if kinds[o] == 2:
            T[pos, pos] = T[pos + 1, pos + 1] = a[ip]
            T[pos, pos + 1] = b[ip] * r[ip]
            T[pos + 1, pos] = -b[ip] / r[ip]
            ip += 1
            pos += 2
        else:
            T[pos, pos] = lam_r[ir]
            ir += 1
            pos += 1
    return _hessenberg_similarity(T, rng), a + 1j * b, lam_r


def block_scaled(n: int, b: int, seed: int, far: float = 1e250, diag: float = 1e-200,
                 sub: float = 1e-3):
    """Adversarial upper-Hessenberg input for the overflow-protection branches
    of the tile update: entries more than b columns right of the diagonal
    scaled by `far`, a nearly singular diagonal of magnitude `diag`, and a
    constant subdiagonal `sub`.  Returns (H, shifts) with shifts near 0."""
    rng = np.random.default_rng(seed)
    T = np.triu(rng.standard_normal((n, n)))
    I, J = np.indices((n, n))
    T = np.where(J - I > b, T * far, T)
    T[np.diag_indices(n)] = rng.uniform(0.5, 1.0, n) * diag * np.sign(rng.standard_normal(n))
    T[np.arange(1, n), np.arange(n - 1)] = sub
    H = np.asfortranarray(np.triu(T, -1))
    return H, np.array([0.0, 0.7 * diag, -0.6 * diag, 1e-300])


def reduced_triangular(n: int, seed: int, sub: float = 0.0):
    """Nearly reduced input: upper triangular with a zero diagonal (repeated
    zero eigenvalue) and subdiagonal `sub`; shifts 0.  Every 1x1 solve is
    perturbed and the division rescales fire."""
    rng = np.random.default_rng(seed)
    T = np.triu(rng.standard_normal((n, n)))
    T[np.diag_indices(n)] = 0.0
    T[np.arange(1, n), np.arange(n - 1)] = sub
    return np.asfortranarray(T), np.zeros(8)


def perturbed_shifts(lam: np.ndarray, seed: int, rel: float = 1e-12) -> np.ndarray:
    """lambda_i (1 + rel * N(0,1))."""
    rng = np.random.default_rng(seed)
    return lam * (1.0 + rel * rng.standard_normal(lam.shape[0]))


def shift_subset(lam: np.ndarray, rng: np.random.Generator, lo: float, hi: float) -> np.ndarray:
    """A random subset of lam of fraction U[lo, hi] (at least one)."""
    n = lam.shape[0]
    m = max(1, int(round(n * rng.uniform(lo, hi))))
    return np.sort(rng.choice(lam, size=m, replace=False))


def uniform_rhs(n: int, nrhs: int, seed: int) -> np.ndarray:
    """Right-hand sides uniform on [0, 1] (Fortran order)."""
    return np.asfortranarray(np.random.default_rng(seed).uniform(0.0, 1.0, (n, nrhs)))
