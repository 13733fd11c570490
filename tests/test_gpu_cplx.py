"""Complex-conjugate shifts on the device, through the C ABI, against the
oracle's complex path (oracle/hsro_cplx.c), which executes the kernels'
arithmetic in the kernels' order: vectors, perturbation flags, reconciled
scaling factors and convergence must agree bit for bit.  The oracle's complex
path is itself checked against LAPACK dgeev and the reference's robust
complex kernels (tests/test_oracle_cplx.py).
"""
import numpy as np
import pytest

from hsrq3in_gb300 import generators as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _device(H, mu, tlsz, rhs_tlsz=16, **kw):
    import hsrq3in_gb300 as hsr
    return hsr.inverse_iteration_cplx(H, mu, tlsz, rhs_tlsz, **kw)


def _oracle(H, mu, tlsz, intscale=1, max_restarts=-1):
    return O.oracle_inverse_iteration_cplx(H, mu.real, mu.imag, tlsz, 16, intscale=intscale,
                                           max_restarts=max_restarts, variant="fma")


def _same(dev, orc):
    assert np.array_equal(dev["vr"], orc["vr"], equal_nan=True), \
        np.nanmax(np.abs(dev["vr"] - orc["vr"]))
    assert np.array_equal(dev["perturbed"], orc["perturbed"])
    assert np.array_equal(dev["scale"], orc["colscale"], equal_nan=True)
    assert np.array_equal(dev["status"], orc["status"])


@pytest.mark.parametrize("n,tlsz,seed,upper", [
    (2, 4, 1, 1.0), (8, 8, 2, 1.0), (60, 64, 3, 1.0),        # one tile
    (64, 16, 4, 1.0), (101, 12, 5, 1.0), (203, 40, 6, 1.0),  # ragged first tile
    (256, 64, 7, 1 / 256), (333, 20, 8, 1 / 333),            # well-conditioned
    (900, 440, 9, 1.0),                                       # v/y in global scratch
])
def test_cplx_bitwise_vs_oracle(gpu_lib, n, tlsz, seed, upper):
    H, pairs, _ = G.complex_spectrum(n, seed, upper_scale=upper)
    dev = _device(H, pairs, tlsz)
    orc = _oracle(H, pairs, tlsz)
    _same(dev, orc)
    assert dev["status"].all()
    assert O.residuals(H, pairs, dev["X"]).max() <= 10 * n * EPS


def test_cplx_n1000_residual_and_lapack(gpu_lib):
    """n = 1000 with 500 conjugate pairs, tlsz = 200: every vector within the
    residual bound; on the well-conditioned spectrum the vectors agree with
    LAPACK dgeev's to 1e-10 rad."""
    n = 1000
    H, pairs, _ = G.complex_spectrum(n, 41)
    dev = _device(H, pairs, 200, 64)
    assert dev["rc"] == 0
    assert np.all(np.isfinite(dev["vr"]))
    assert O.residuals(H, pairs, dev["X"]).max() <= 10 * n * EPS
    _same(dev, _oracle(H, pairs, 200))
    Hw, pw, _ = G.complex_spectrum(400, 42, upper_scale=1 / 400)
    dw = _device(Hw, pw, 40)
    assert O.phase_angles(dw["X"], O.eig_vectors_for(Hw, pw)).max() <= 1e-10


@pytest.mark.parametrize("wi", [1e-300, 1e-100])
@pytest.mark.parametrize("scaling,intscale", [("pow2", 1), ("double", 0)])
def test_cplx_protection_reduced(gpu_lib, wi, scaling, intscale):
    """Zero diagonal, tiny complex shifts: the robust complex division and the
    diagonal-solve rescales fire; bit-exact in both scaling representations
    (NaN positions included for the reference's double factors)."""
    H, _ = G.reduced_triangular(96, 5)
    mu = np.array([0.0, 0.0, 0.0]) + 1j * np.array([wi, 2 * wi, 0.5 * wi])
    dev = _device(H, mu, 24, 4, scaling=scaling, max_restarts=1)
    orc = _oracle(H, mu, 24, intscale=intscale, max_restarts=1)
    assert orc["stats"]["div_rescales"] > 0
    _same(dev, orc)
    if scaling == "pow2":
        assert np.all(np.isfinite(dev["vr"])) and dev["status"].all()


def test_cplx_protection_tile_update(gpu_lib):
    """Block-scaled input: Part 0/1/2 rescales of the tile update fire, which
    runs the full complex Part 1 and the protected (rescaled Ytilde2) path of
    the complex GEMM epilogue."""
    H, sh = G.block_scaled(96, 16, 3)
    mu = np.asarray(sh)[:4] + 1e-3j
    dev = _device(H, mu, 16, 4, max_restarts=1)
    orc = _oracle(H, mu, 16, max_restarts=1)
    st = orc["stats"]
    assert st["part1_rescales"] > 0 and st["part2_rescales"] > 0 and st["consistency_rescales"] > 0
    _same(dev, orc)
    assert np.all(np.isfinite(dev["vr"]))


def test_cplx_restarts_in_place(gpu_lib):
    """Every other shift 1e-9 away from its well-conditioned eigenvalue: those
    pairs do not pass ||y|| > 0.1/sqrt(n), the restart rounds run on them
    (after the stable partition that moves converged pairs first), and every
    pair is back at its position on return."""
    n = 48
    H, pairs, _ = G.complex_spectrum(n, 12, upper_scale=1 / n)
    mu = pairs.copy()
    mu[::2] *= 1 + 1e-9
    dev = _device(H, mu, 16, max_restarts=3)
    orc = _oracle(H, mu, 16, max_restarts=3)
    assert orc["stats"]["restarts"] > 0
    assert orc["status"][1::2].all() and not orc["status"][::2].any()
    _same(dev, orc)


def test_cplx_device_entry(gpu_lib):
    """hsr_inverse_iteration_cplx_device on device-resident tensors gives the
    host call's result bit for bit, with per-pair status and scale."""
    import torch
    import hsrq3in_gb300 as hsr
    n, tlsz = 150, 24
    H, pairs, _ = G.complex_spectrum(n, 17)
    host = _device(H, pairs, tlsz)
    dev = torch.device("cuda:0")
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)       # rows = columns of H
    dwr = torch.from_numpy(pairs.real.copy()).to(dev)
    dwi = torch.from_numpy(pairs.imag.copy()).to(dev)
    dvr = torch.zeros((2 * pairs.size, n), dtype=torch.float64, device=dev)
    d_status = torch.zeros(pairs.size, dtype=torch.int32, device=dev)
    d_scale = torch.zeros(pairs.size, dtype=torch.float64, device=dev)
    rc = hsr.inverse_iteration_cplx_device(dH, dwr, dwi, dvr, tlsz, d_status=d_status, d_scale=d_scale)
    torch.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(dvr.cpu().numpy().T, host["vr"])
    assert np.array_equal(d_status.cpu().numpy(), host["status"])
    assert np.array_equal(d_scale.cpu().numpy(), host["scale"])


def test_mixed_real_and_pairs(gpu_lib):
    """hsr_inverse_iteration_mixed on a spectrum with real eigenvalues and
    conjugate pairs interleaved (the LAPACK dhsein layout) equals the real and
    the complex entry points called separately, column for column, bit for
    bit; every eigenpair meets the residual bound."""
    import hsrq3in_gb300 as hsr
    n, tlsz = 160, 32
    H, pairs, lam_r = G.complex_spectrum(n, 31, n_real=40)
    rng = np.random.default_rng(5)
    items = [("r", x) for x in lam_r[:12]] + [("c", z) for z in pairs[:14]]
    rng.shuffle(items)
    wr, wi = [], []
    for kind, v in items:
        if kind == "r":
            wr.append(v)
            wi.append(0.0)
        else:
            wr += [v.real, v.real]
            wi += [v.imag, -v.imag]
    wr, wi = np.array(wr), np.array(wi)
    out = hsr.inverse_iteration_mixed(H, wr, wi, tlsz, 16)
    assert out["rc"] == 0 and out["status"].all()
    rpos = np.where(wi == 0.0)[0]
    cpos = np.where(wi > 0.0)[0]
    sep_r = hsr.inverse_iteration(H, wr[rpos], tlsz, 16)
    sep_c = hsr.inverse_iteration_cplx(H, wr[cpos] + 1j * wi[cpos], tlsz, 16)
    assert np.array_equal(out["vr"][:, rpos], sep_r["vr"])
    assert np.array_equal(out["vr"][:, cpos], sep_c["vr"][:, 0::2])
    assert np.array_equal(out["vr"][:, cpos + 1], sep_c["vr"][:, 1::2])
    X = out["vr"].astype(complex)
    X[:, cpos] = out["vr"][:, cpos] + 1j * out["vr"][:, cpos + 1]
    X[:, cpos + 1] = np.conj(X[:, cpos])
    mu = out["wr"] + 1j * out["wi"]
    assert O.residuals(H, mu, X).max() <= 10 * n * EPS


def test_cplx_passes_by_hbm_budget(gpu_lib):
    """Complex shifts in passes of 32 pairs (a 400 KB workspace budget) give
    the one-pass result bit for bit."""
    n, tlsz = 300, 40
    H, pairs, _ = G.complex_spectrum(n, 43)
    one = _device(H, pairs[:90], tlsz)
    split = _device(H, pairs[:90], tlsz, hbm_budget_bytes=4e5)
    _same(dict(split, colscale=split["scale"]), dict(one, colscale=one["scale"]))
