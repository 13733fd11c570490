"""Hessenberg reduction on the device (hsr_hessenberg_device) against LAPACK
dgehrd through scipy, the orthogonal factor it implies, extreme scalings, and
the dense-input pipeline: reduce, solve on H, back-transform."""
import numpy as np
import pytest

from hsrq3in_gb300 import generators as G

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _reduce(A):
    import torch
    import hsrq3in_gb300 as hsr
    n = A.shape[0]
    ld = n + 3                                                  # odd pitch on purpose
    dA = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    dA[:, :n] = torch.from_numpy(np.ascontiguousarray(A.T))
    tau = hsr.hessenberg_device(dA)
    torch.cuda.synchronize()
    return dA, tau, dA[:, :n].cpu().numpy().T.copy(order="F"), tau.cpu().numpy()


def _form_q(dA, tau, n):
    import torch
    import hsrq3in_gb300 as hsr
    dQ = torch.eye(n, dtype=torch.float64, device="cuda")     # rows = columns of I
    hsr.hessenberg_apply_q_device(dA, tau, dQ)
    torch.cuda.synchronize()
    return dQ.cpu().numpy().T


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (3, 3), (4, 4), (17, 5), (100, 6), (300, 7), (700, 8)])
def test_matches_lapack_dgehrd(gpu_lib, n, seed):
    from scipy.linalg import lapack
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    _, _, out, tau = _reduce(A)
    hq, tau_ref, info = lapack.dgehrd(np.asfortranarray(A))
    assert info == 0
    scale = np.linalg.norm(A)
    np.testing.assert_allclose(np.triu(out, -1), np.triu(hq, -1), rtol=0, atol=1e3 * n * EPS * scale)
    np.testing.assert_allclose(tau[:n - 1], tau_ref[:n - 1], rtol=0, atol=1e3 * n * EPS)
    np.testing.assert_allclose(np.tril(out, -2), np.tril(hq, -2), rtol=0, atol=1e3 * n * EPS)


@pytest.mark.parametrize("n", [50, 400])
def test_q_orthogonal_similarity(gpu_lib, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    dA, tau, out, _ = _reduce(A)
    H = np.triu(out, -1)
    Q = _form_q(dA, tau, n)
    assert np.linalg.norm(Q.T @ Q - np.eye(n)) <= 50 * n * EPS
    assert np.linalg.norm(A @ Q - Q @ H) / np.linalg.norm(A) <= 50 * n * EPS


@pytest.mark.parametrize("scale", [1e300, 1e-300])
def test_extreme_scale(gpu_lib, scale):
    from scipy.linalg import lapack
    rng = np.random.default_rng(9)
    n = 120
    A = rng.standard_normal((n, n))
    _, _, out, _ = _reduce(A * scale)
    assert np.all(np.isfinite(out))
    hq, _, _ = lapack.dgehrd(np.asfortranarray(A))
    np.testing.assert_allclose(np.triu(out, -1) / scale, np.triu(hq, -1), rtol=0,
                               atol=1e3 * n * EPS * np.linalg.norm(A))


def test_dense_pipeline(gpu_lib):
    """Dense A with a known real spectrum: reduce on the device, solve on H,
    back-transform with Q; every eigenpair of A within the residual bound."""
    import torch
    import hsrq3in_gb300 as hsr
    n = 600
    H0, lam = G.real_spectrum(n, 21)
    rng = np.random.default_rng(22)
    Z, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = Z @ H0 @ Z.T
    dA, tau, out, _ = _reduce(A)
    H = np.triu(out, -1)
    wr = G.perturbed_shifts(lam, 23)
    sol = hsr.inverse_iteration(np.asfortranarray(H), wr, 64, 64)
    dX = torch.from_numpy(np.ascontiguousarray(sol["vr"].T)).cuda()
    hsr.hessenberg_apply_q_device(dA, tau, dX)
    torch.cuda.synchronize()
    X = dX.cpu().numpy().T
    R = A @ X - X * sol["wr"][None, :]
    res = np.linalg.norm(R, axis=0) / (np.linalg.norm(A) * np.linalg.norm(X, axis=0))
    assert np.all(res <= 100 * n * EPS), res.max()
