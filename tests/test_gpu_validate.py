"""Device residuals (hsr_residuals_device) against a numpy restatement of the
same formula, on ordinary, overflow-scaled and degenerate inputs, and on the
solver's own output."""
import numpy as np
import pytest

from hsrq3in_gb300 import generators as G

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _np_residuals(H, wr, X):
    """||H x - wr x|| / (||H||_F ||x||) over the Hessenberg part, in float64
    (inputs of ordinary magnitude only)."""
    Hh = np.triu(H, -1)
    R = Hh @ X - X * wr[None, :]
    return np.linalg.norm(R, axis=0) / (np.linalg.norm(Hh) * np.linalg.norm(X, axis=0))


def _to_dev(torch, H, wr, X):
    n = H.shape[0]
    ld = n + (n & 1)
    dH = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    dH[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T))
    dX = torch.zeros((X.shape[1], ld + 2), dtype=torch.float64, device="cuda")   # odd pitch on purpose
    dX[:, :n] = torch.from_numpy(np.ascontiguousarray(X.T))
    return dH, torch.from_numpy(np.ascontiguousarray(wr)).cuda(), dX


def _dev_residuals(H, wr, X):
    import torch
    import hsrq3in_gb300 as hsr
    dH, dwr, dX = _to_dev(torch, H, wr, X)
    res = hsr.residuals_device(dH, dwr, dX)
    torch.cuda.synchronize()
    return res.cpu().numpy()


@pytest.mark.parametrize("n,ncols,seed", [(1, 1, 1), (5, 3, 2), (64, 32, 3), (301, 45, 4), (777, 70, 5)])
def test_matches_numpy(gpu_lib, n, ncols, seed):
    rng = np.random.default_rng(seed)
    H = np.triu(rng.standard_normal((n, n)), -1) + np.tril(rng.standard_normal((n, n)), -2)  # garbage below
    X = rng.standard_normal((n, ncols))
    wr = rng.uniform(-2, 2, ncols)
    dev = _dev_residuals(H, wr, X)
    ref = _np_residuals(H, wr, X)
    np.testing.assert_allclose(dev, ref, rtol=1e-12)


def test_scale_invariant_extremes(gpu_lib):
    # H ~ 1e300 and columns of x from 1e-300 to 1e300: no overflow, same ratio.
    rng = np.random.default_rng(7)
    n, ncols = 200, 6
    H = np.triu(rng.standard_normal((n, n)), -1)
    X = rng.standard_normal((n, ncols))
    wr = rng.uniform(-2, 2, ncols)
    ref = _np_residuals(H, wr, X)
    colscale = np.array([1e-300, 1e-150, 1.0, 1e150, 1e300, 2.0 ** -1070])
    dev = _dev_residuals(H * 1e300, wr * 1e300, X * colscale[None, :])
    np.testing.assert_allclose(dev[:5], ref[:5], rtol=1e-12)
    assert np.isfinite(dev[5])          # subnormal column: finite, accuracy not claimed


def test_degenerate_columns(gpu_lib):
    rng = np.random.default_rng(8)
    n = 50
    H = np.triu(rng.standard_normal((n, n)), -1)
    X = rng.standard_normal((n, 3))
    X[:, 1] = 0.0
    X[7, 2] = np.nan
    dev = _dev_residuals(H, np.array([0.1, 0.2, 0.3]), X)
    assert np.isfinite(dev[0])
    assert np.isinf(dev[1]) and dev[1] > 0
    assert np.isnan(dev[2])


@pytest.mark.parametrize("n,tlsz", [(500, 64), (1000, 200)])
def test_solver_output_meets_bound(gpu_lib, n, tlsz):
    import hsrq3in_gb300 as hsr
    H, lam = G.real_spectrum(n, 11)
    wr = G.perturbed_shifts(lam, 12)
    out = hsr.inverse_iteration(H, wr, tlsz, 64)
    dev = _dev_residuals(H, out["wr"], out["vr"])
    assert np.all(dev <= 10 * n * EPS), dev.max()
