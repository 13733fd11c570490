"""CPU tests of the complex-shift oracle (oracle/hsro_cplx.c).

The reference ships the robust kernels for complex shifts (robust.c:486-773)
but no driver that uses them, so the oracle's complex path is pinned in two
ways: its scalar kernels bit for bit against the reference's own compiled
robust.c, and its eigenvectors against LAPACK dgeev (angles, phase-invariant)
and the residual bound ||Hx - mu x|| / (||H||_F ||x||) <= 10 n eps.
"""
import os

import numpy as np
import pytest

from hsrq3in_gb300 import generators as gen
from oracle import pyoracle as po

EPS = np.finfo(float).eps


def _same(a, b):
    return all((x == y and np.signbit(x) == np.signbit(y)) or (x != x and y != y)
               for x, y in zip(a, b))


def _extreme_operands(rng, count, k):
    out = []
    for it in range(count):
        e = rng.integers(-320, 308, size=k) if it % 3 == 0 else rng.integers(-20, 20, size=k)
        v = rng.standard_normal(k) * 10.0 ** e.astype(float)
        if it % 7 == 0:
            v[rng.integers(0, k)] = 0.0
        out.append(v)
    return out


GOLDEN_KERNELS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cplx_kernels.npz")


@pytest.mark.parametrize("intscale", [0, 1])
def test_complex_kernels_vs_golden(intscale):
    """robust_cmplx_div and the complex 1x1 solve of the oracle against the
    reference's own outputs recorded in tests/golden/cplx_kernels.npz (made
    by tests/golden/make_golden.py from the compiled robust.c:639-773): every
    output bit of 1000 operand rows per kernel, including about a third that
    take a protection branch, on hosts without the reference sources too."""
    z = np.load(GOLDEN_KERNELS)
    for row, ref in zip(z["div_in_%d" % intscale], z["div_out_%d" % intscale]):
        assert _same(po.oracle_robust_cmplx_div(*row, intscale=intscale), ref), row
    for row, ref in zip(z["sol_in_%d" % intscale], z["sol_out_%d" % intscale]):
        smin, t, lr, li, xr, xi = row
        assert _same(po.oracle_csolve_1x1(smin, t, 0.0, lr, li, xr, xi, intscale), ref), row


@pytest.mark.parametrize("intscale", [0, 1])
def test_complex_division_pinned_to_reference(intscale):
    """robust_cmplx_div (robust.c:639-675): every output bit, both scalings."""
    if not po.reference_available():
        pytest.skip("reference sources not present on this host")
    rng = np.random.default_rng(11 + intscale)
    for v in _extreme_operands(rng, 6000, 5):
        smin, a, b, c, d = abs(v[0]), v[1], v[2], v[3], v[4]
        assert _same(po.oracle_robust_cmplx_div(smin, a, b, c, d, intscale),
                     po.reference_robust_cmplx_div(smin, a, b, c, d, intscale)), v


@pytest.mark.parametrize("intscale", [0, 1])
def test_complex_1x1_solve_pinned_to_reference(intscale):
    """solve_1x1_cmplx_system (robust.c:677-773) is the complex 1x1 solve with
    a real t; nonzero imaginary parts of lambda, as the solver uses it."""
    if not po.reference_available():
        pytest.skip("reference sources not present on this host")
    rng = np.random.default_rng(21 + intscale)
    for v in _extreme_operands(rng, 6000, 6):
        smin, t, lr, li, xr, xi = abs(v[0]), v[1], v[2], v[3], v[4], v[5]
        if li == 0.0:
            li = 1e-3
        assert _same(po.oracle_csolve_1x1(smin, t, 0.0, lr, li, xr, xi, intscale),
                     po.reference_solve_1x1_cmplx(smin, t, lr, li, xr, xi, intscale)), v


def test_complex_givens():
    rng = np.random.default_rng(3)
    for v in _extreme_operands(rng, 3000, 3):
        fr, fi, g = v
        c, sr, si = po.oracle_cgivens(fr, fi, g)
        s = complex(sr, si)
        f = complex(fr, fi)
        assert c >= 0.0
        assert abs(c * c + abs(s) ** 2 - 1.0) < 8 * EPS
        m = max(abs(fr), abs(fi), abs(g))
        if m == 0 or not np.isfinite(m) or m < 1e-290 or m > 1e290:
            continue
        # sigma f + c g = 0 relative to the operands
        assert abs(s * (f / m) + c * (g / m)) < 8 * EPS
    # a real f reproduces the real rotation of reduce.c:14-24 up to rounding
    for f, g in [(3.0, 4.0), (-2.0, 1e-3), (1e-200, 5.0), (7.0, -1e10)]:
        c, sr, si = po.oracle_cgivens(f, 0.0, g)
        dl = po.oracle_dlartg(f, g)
        assert si == 0.0
        assert abs(c - dl[0]) <= 4 * EPS and abs(sr - (-dl[1])) <= 4 * EPS


@pytest.mark.parametrize("n,tlsz,rhs", [(40, 8, 4), (61, 12, 5), (101, 16, 7), (160, 20, 16)])
def test_complex_oracle_against_lapack(n, tlsz, rhs):
    """Well-conditioned complex spectra: every pair converges, residual
    <= 10 n eps, and the vector agrees with LAPACK dgeev's to <= 1e-11 rad."""
    H, pairs, _ = gen.complex_spectrum(n, n + 1, upper_scale=1.0 / n)
    o = po.oracle_inverse_iteration_cplx(H, pairs.real, pairs.imag, tlsz, rhs)
    assert o["status"].all()
    X = o["X"]
    assert np.all(po.residuals(H, pairs, X) <= 10 * n * EPS)
    assert np.max(po.phase_angles(X, po.eig_vectors_for(H, pairs))) <= 1e-11
    # unit 2-norm columns
    assert np.allclose(np.linalg.norm(X, axis=0), 1.0, atol=1e-14)


def test_complex_oracle_tiling():
    """The tile size changes rounding only; the shift-tile width changes
    nothing (every pair is computed independently)."""
    n = 97
    H, pairs, _ = gen.complex_spectrum(n, 5, upper_scale=1.0 / n)
    a = po.oracle_inverse_iteration_cplx(H, pairs.real, pairs.imag, 12, 5)
    b = po.oracle_inverse_iteration_cplx(H, pairs.real, pairs.imag, 12, 48)
    c = po.oracle_inverse_iteration_cplx(H, pairs.real, pairs.imag, 32, 3)
    assert np.array_equal(a["vr"], b["vr"])
    assert np.max(po.phase_angles(a["X"], c["X"])) <= 1e-12


def test_complex_oracle_ill_conditioned_residuals():
    """The benchmark's N(0,1) strictly-upper entries: angles are meaningless
    (kappa ~ 1e13), residuals are not."""
    n = 120
    H, pairs, _ = gen.complex_spectrum(n, 9)
    o = po.oracle_inverse_iteration_cplx(H, pairs.real, pairs.imag, 16, 8)
    assert o["status"].all()
    assert np.all(po.residuals(H, pairs, o["X"]) <= 10 * n * EPS)


@pytest.mark.parametrize("wi", [1e-300, 1e-100, 1e-20])
def test_complex_protection_reduced(wi):
    """Upper-triangular H with a zero diagonal and tiny complex shifts: the
    complex division and the diagonal-solve rescales fire; power-of-two factors
    keep every vector finite and converged within the residual bound."""
    H, _ = gen.reduced_triangular(40, 5)
    wr = np.zeros(3)
    wim = np.array([wi, 2 * wi, 0.5 * wi])
    o = po.oracle_inverse_iteration_cplx(H, wr, wim, 12, 4, intscale=1, max_restarts=1)
    st = o["stats"]
    assert st["div_rescales"] > 0
    assert np.isfinite(o["vr"]).all() and o["status"].all()
    assert np.all(po.residuals(H, wr + 1j * wim, o["X"]) <= 10 * 40 * EPS)


def test_complex_protection_tile_update():
    """Block-scaled input (entries far right of the diagonal ~1e250): the
    Part-0/1/2 rescales of the tile update fire for complex shifts too."""
    H, sh = gen.block_scaled(48, 12, 3)
    wr = np.asarray(sh)[:4]
    wim = np.full(4, 1e-3)
    o = po.oracle_inverse_iteration_cplx(H, wr, wim, 12, 4, intscale=1, max_restarts=1)
    st = o["stats"]
    assert st["part1_rescales"] > 0 and st["part2_rescales"] > 0 and st["consistency_rescales"] > 0
    assert np.isfinite(o["vr"]).all() and o["status"].all()
