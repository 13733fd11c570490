"""Device parity: the CUDA library (through its C ABI) against the CPU oracle.

The oracle's "fma" variant executes the kernels' arithmetic in the kernels'
order, so the device result must be bit-identical to it.  The oracle's "ref"
variant is bit-identical to the reference itself (tests/test_oracle.py);
between the two only rounding differs, which the residual bound and the
well-conditioned angle tests cover.
"""
import numpy as np
import pytest

from hsrq3in_gb300 import generators as G
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _device(H, wr, tlsz, rhs_tlsz=16, **kw):
    import hsrq3in_gb300 as hsr
    return hsr.inverse_iteration(H, wr, tlsz, rhs_tlsz, **kw)


@pytest.mark.parametrize("n,tlsz,seed", [
    (1, 4, 1), (2, 4, 2), (7, 8, 3), (60, 64, 4),          # one tile
    (64, 16, 5), (100, 40, 6), (203, 40, 7), (256, 64, 8),  # several tiles, ragged first tile
    (333, 12, 9),
    (900, 440, 10),                                         # v/y in global scratch (tile too big for smem)
])
def test_bitwise_vs_oracle(gpu_lib, n, tlsz, seed):
    H, lam = G.real_spectrum(n, seed)
    wr = G.perturbed_shifts(lam, seed + 100)
    dev = _device(H, wr, tlsz)
    orc = O.oracle_inverse_iteration(H, wr, tlsz, 16, intscale=1, variant="fma")
    assert np.array_equal(dev["wr"], orc["wr"])
    assert np.array_equal(dev["vr"], orc["vr"]), np.max(np.abs(dev["vr"] - orc["vr"]))
    assert np.array_equal(dev["perturbed"], orc["perturbed"])
    assert np.array_equal(dev["scale"], orc["colscale"])
    assert np.array_equal(dev["status"], orc["status"])


def test_residual_config1(gpu_lib):
    """n=1000, all 1000 shifts (the small plain configuration)."""
    n = 1000
    H, lam = G.real_spectrum(n, 1234)
    wr = G.perturbed_shifts(lam, 7)
    dev = _device(H, wr, 200, 64)
    assert dev["rc"] == 0
    assert np.all(np.isfinite(dev["vr"]))
    res = O.residuals(H, dev["wr"], dev["vr"])
    assert res.max() <= 10 * n * EPS, res.max()
    orc = O.oracle_inverse_iteration(H, wr, 200, 64, intscale=1, variant="fma")
    assert np.array_equal(dev["vr"], orc["vr"])


@pytest.mark.parametrize("scaling,intscale", [("pow2", 1), ("double", 0)])
def test_stress_finite_and_bitwise(gpu_lib, scaling, intscale):
    n = 300
    H, lam = G.stress(n, 5)
    dev = _device(H, lam, 40, scaling=scaling)
    orc = O.oracle_inverse_iteration(H, lam, 40, 16, intscale=intscale, variant="fma")
    assert np.all(np.isfinite(dev["vr"]))
    assert np.array_equal(dev["vr"], orc["vr"])
    assert O.residuals(H, dev["wr"], dev["vr"]).max() <= 10 * n * EPS


def test_stress_config_n5000(gpu_lib):
    """The robustness-stress configuration at its full order (n = 5000,
    clustered spectrum of width 1e-13, columns scaled by up to 1e150, shifts
    equal to the eigenvalues), on 128 of its shifts: finite, within the
    residual bound, and bit-identical to the oracle in vectors, perturbation
    flags, reconciled scales and convergence."""
    n = 5000
    H, lam = G.stress(n, 3)
    wr = lam[np.linspace(0, n - 1, 128).astype(int)]
    dev = _device(H, wr, 200)
    orc = O.oracle_inverse_iteration(H, wr, 200, 16, intscale=1, variant="fma")
    assert np.all(np.isfinite(dev["vr"]))
    assert np.array_equal(dev["wr"], orc["wr"])
    assert np.array_equal(dev["vr"], orc["vr"])
    assert np.array_equal(dev["perturbed"], orc["perturbed"])
    assert np.array_equal(dev["scale"], orc["colscale"])
    assert np.array_equal(dev["status"], orc["status"])
    assert O.residuals(H, dev["wr"], dev["vr"]).max() <= 10 * n * EPS


@pytest.mark.parametrize("kind", ["reduced", "reduced_sub", "block_scaled"])
def test_protection_branches_pow2(gpu_lib, kind):
    """Nearly reduced and block-scaled inputs fire the division, diagonal,
    consistency, Part-1 and Part-2 rescales.  With power-of-two factors the
    result stays finite; it must equal the oracle bit for bit, which also
    covers the protected (rescaled Ytilde2) path of the GEMM epilogue."""
    if kind == "reduced":
        H, wr = G.reduced_triangular(120, 5)
        tlsz = 40
    elif kind == "reduced_sub":
        H, wr = G.reduced_triangular(120, 6, sub=1e-300)
        tlsz = 40
    else:
        H, wr = G.block_scaled(96, 16, 3)
        tlsz = 16
    dev = _device(H, wr, tlsz, rhs_tlsz=4)
    orc = O.oracle_inverse_iteration(H, wr, tlsz, 4, intscale=1, variant="fma")
    st = orc["stats"]
    fired = st["div_rescales"] + st["solve_rescales"] + st["part1_rescales"] + st["part2_rescales"]
    assert fired > 0
    if kind == "block_scaled":
        assert st["part1_rescales"] > 0 and st["part2_rescales"] > 0 and st["consistency_rescales"] > 0
    assert np.all(np.isfinite(dev["vr"]))
    assert np.array_equal(dev["wr"], orc["wr"])
    assert np.array_equal(dev["vr"], orc["vr"])
    assert np.array_equal(dev["scale"], orc["colscale"])
    assert np.array_equal(dev["status"], orc["status"])


def test_double_scaling_matches_reference_semantics(gpu_lib):
    """With the reference's double factors the same reduced input underflows
    its scale factors to 0 and yields NaN, as the reference does; the device
    reproduces the oracle exactly (NaN positions included)."""
    H, wr = G.reduced_triangular(40, 7)
    dev = _device(H, wr, 12, rhs_tlsz=4, scaling="double", max_restarts=2)
    orc = O.oracle_inverse_iteration(H, wr, 12, 4, intscale=0, variant="fma")
    assert not np.all(np.isfinite(orc["vr"]))
    assert np.isnan(dev["vr"]).sum() > 0


def test_restart_path_matches_oracle(gpu_lib):
    """Well-conditioned H with 1e-12 shift noise: one solve does not pass
    ||y|| > 0.1/sqrt(n), so the restart rounds run (and reorder wr)."""
    n = 48
    H, lam = G.well_conditioned(n, 3)
    wr = G.perturbed_shifts(lam, 4)
    dev = _device(H, wr, 16)
    orc = O.oracle_inverse_iteration(H, wr, 16, 16, intscale=1, variant="fma")
    assert orc["stats"]["restarts"] > 0
    assert np.array_equal(dev["wr"], orc["wr"])          # same reordering
    assert np.array_equal(dev["status"], orc["status"])
    assert np.array_equal(dev["vr"], orc["vr"])


def test_user_rhs(gpu_lib):
    n = 150
    H, lam = G.real_spectrum(n, 21)
    wr = G.perturbed_shifts(lam, 22)
    rhs = G.uniform_rhs(n, n, 23)
    dev = _device(H, wr, 20, rhs=rhs)
    orc = O.oracle_solve_rhs(H, wr, rhs, 20, 16, intscale=1, variant="fma")
    assert np.array_equal(dev["vr"], orc["vr"])


def test_passes_by_hbm_budget(gpu_lib):
    """A workspace budget that holds only 32 columns splits the shifts into
    passes; every column is the same bit for bit as in one pass."""
    n, tlsz = 300, 40
    H, lam = G.real_spectrum(n, 41)
    wr = G.perturbed_shifts(lam, 42)[:100]
    one = _device(H, wr, tlsz)
    split = _device(H, wr, tlsz, hbm_budget_bytes=4e5)
    assert np.array_equal(one["vr"], split["vr"])
    assert np.array_equal(one["scale"], split["scale"])
    assert np.array_equal(one["status"], split["status"])


def test_concurrent_host_threads(gpu_lib):
    """Calls from different host threads use separate workspaces and streams:
    two threads solving different problems with different tile sizes (and so
    different shared-memory footprints) concurrently get the results of the
    same calls made one after the other."""
    import threading
    jobs = []
    for n, tlsz, seed in ((300, 40, 51), (257, 88, 52), (410, 200, 53)):
        H, lam = G.real_spectrum(n, seed)
        jobs.append((H, G.perturbed_shifts(lam, seed + 1)[:120], tlsz))
    serial = [_device(H, wr, t) for H, wr, t in jobs]
    out = [None] * len(jobs)

    def work(k):
        H, wr, t = jobs[k]
        for _ in range(3):
            out[k] = _device(H, wr, t)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(jobs))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for a, b in zip(serial, out):
        assert np.array_equal(a["vr"], b["vr"]) and np.array_equal(a["wr"], b["wr"])


def test_bounded_wait_reports_and_context_survives(gpu_lib):
    """Failure detection without a fault: a device wait that can never
    complete gives up after its poll limit, the call reports HSR_ERR_DEVICE,
    and the context stays usable -- the next solve is bit-exact to the oracle."""
    from hsrq3in_gb300 import _lib
    assert gpu_lib.hsr_selftest_bounded_wait(None) == _lib.HSR_ERR_DEVICE
    n, tlsz = 64, 16
    H, lam = G.real_spectrum(n, 61)
    wr = G.perturbed_shifts(lam, 62)
    dev = _device(H, wr, tlsz)
    orc = O.oracle_inverse_iteration(H, wr, tlsz, 16, intscale=1, variant="fma")
    assert dev["rc"] == 0 and np.array_equal(dev["vr"], orc["vr"])


@pytest.mark.parametrize("extra_h,extra_v", [(1, 3), (3, 0), (0, 5)])
def test_leading_dimensions_through_c_abi(gpu_lib, extra_h, extra_v):
    """The drop-in call with ldH = n + extra_h (odd pitches are re-padded for
    TMA) and ldvr = n + extra_v: the result equals the compact call bit for
    bit and the caller's padding rows of vr are left untouched; the same for
    the complex-shift entry."""
    import ctypes as C
    from hsrq3in_gb300 import _lib
    n, tlsz, m = 97, 24, 20
    H, lam = G.real_spectrum(n, 71)
    wr = np.ascontiguousarray(G.perturbed_shifts(lam, 72)[:m])
    ldh, ldv = n + extra_h, n + extra_v
    Hp = np.full((ldh, n), 7.0, order="F")
    Hp[:n, :] = H
    ref = _device(H, wr, tlsz)
    vr = np.full((ldv, m), -3.25, order="F")
    w = wr.copy()
    gpu_lib.tiled_inverse_iteration(n, Hp.ctypes.data, ldh, m, w.ctypes.data, tlsz, 16, vr.ctypes.data, ldv)
    assert gpu_lib.hsr_last_status() == 0
    assert np.array_equal(vr[:n], ref["vr"]) and np.array_equal(w, ref["wr"])
    assert np.all(vr[n:] == -3.25)
    Hc, pairs, _ = G.complex_spectrum(n, 73)
    Hcp = np.full((ldh, n), 7.0, order="F")
    Hcp[:n, :] = Hc
    cref = hsr_cplx(Hc, pairs[:10], tlsz)
    vc = np.full((ldv, 20), -3.25, order="F")
    a, b = np.ascontiguousarray(pairs[:10].real), np.ascontiguousarray(pairs[:10].imag)
    opt = _lib.Options(0, 0, -1, 0.0)
    rc = gpu_lib.hsr_inverse_iteration_cplx_ex(n, Hcp.ctypes.data, ldh, 10, a.ctypes.data, b.ctypes.data, tlsz, 16,
                                               vc.ctypes.data, ldv, C.byref(opt), None)
    assert rc == 0
    assert np.array_equal(vc[:n], cref["vr"]) and np.all(vc[n:] == -3.25)


@pytest.mark.parametrize("extra_h,extra_v", [(0, 0), (1, 3), (2, 2)])
def test_pinned_host_buffers_through_c_abi(gpu_lib, extra_h, extra_v):
    """With page-locked host buffers the drop-in calls move H in and X out by
    SM copies through the mapped pointers (paired-double and single-double
    forms, depending on the pitches); the result equals the pageable call bit
    for bit and the caller's padding rows of vr stay untouched."""
    import ctypes as C
    import torch
    from hsrq3in_gb300 import _lib
    n, tlsz, m = 98, 24, 20
    H, lam = G.real_spectrum(n, 81)
    wr = np.ascontiguousarray(G.perturbed_shifts(lam, 82)[:m])
    ldh, ldv = n + extra_h, n + extra_v
    ref = _device(H, wr, tlsz)
    Hp = torch.full((n, ldh), 7.0, dtype=torch.float64).pin_memory()
    Hp.numpy()[:, :n] = H.T
    vr = torch.full((m, ldv), -3.25, dtype=torch.float64).pin_memory()
    w = torch.from_numpy(wr.copy()).pin_memory()
    assert Hp.is_pinned() and vr.is_pinned()
    gpu_lib.tiled_inverse_iteration(n, Hp.data_ptr(), ldh, m, w.data_ptr(), tlsz, 16, vr.data_ptr(), ldv)
    assert gpu_lib.hsr_last_status() == 0
    got = vr.numpy()
    assert np.array_equal(got[:, :n].T, ref["vr"]) and np.array_equal(w.numpy(), ref["wr"])
    assert np.all(got[:, n:] == -3.25)
    Hc, pairs, _ = G.complex_spectrum(n, 83)
    Hcp = torch.full((n, ldh), 7.0, dtype=torch.float64).pin_memory()
    Hcp.numpy()[:, :n] = Hc.T
    cref = hsr_cplx(Hc, pairs[:10], tlsz)
    vc = torch.full((20, ldv), -3.25, dtype=torch.float64).pin_memory()
    a, b = np.ascontiguousarray(pairs[:10].real), np.ascontiguousarray(pairs[:10].imag)
    opt = _lib.Options(0, 0, -1, 0.0)
    rc = gpu_lib.hsr_inverse_iteration_cplx_ex(n, Hcp.data_ptr(), ldh, 10, a.ctypes.data, b.ctypes.data, tlsz, 16,
                                               vc.data_ptr(), ldv, C.byref(opt), None)
    assert rc == 0
    gc = vc.numpy()
    assert np.array_equal(gc[:, :n].T, cref["vr"]) and np.all(gc[:, n:] == -3.25)


def hsr_cplx(H, mu, tlsz):
    import hsrq3in_gb300 as hsr
    return hsr.inverse_iteration_cplx(H, mu, tlsz, 16)


@pytest.mark.parametrize("fused", ["1", "0"])
@pytest.mark.parametrize("sc", ["8", "16", "32"])
@pytest.mark.parametrize("n,tlsz,nrhs,seed", [
    (300, 64, 300, 31),      # several tiles, all shifts
    (203, 40, 77, 32),       # ragged first tile, ragged shift count
    (520, 160, 1000, 33),    # the benchmark tile size, more shifts than rows (repeated)
])
def test_diag_forms_bitwise(gpu_lib, monkeypatch, sc, n, tlsz, nrhs, seed, fused):
    """The diagonal kernel's three forms -- 8, 16 or 32 shifts per CTA, chosen
    by shift count -- with the top GEMM fused into the narrow forms or run as
    its own launch, give the oracle's result bit for bit."""
    monkeypatch.setenv("HSR_DIAG_SHIFTS_PER_CTA", sc)
    monkeypatch.setenv("HSR_FUSED_TOP", fused)
    H, lam = G.real_spectrum(n, seed)
    wr = G.perturbed_shifts(np.resize(lam, nrhs), seed + 1)
    dev = _device(H, wr, tlsz)
    orc = O.oracle_inverse_iteration(H, wr, tlsz, 16, intscale=1, variant="fma")
    assert np.array_equal(dev["wr"], orc["wr"])
    assert np.array_equal(dev["vr"], orc["vr"])
    assert np.array_equal(dev["perturbed"], orc["perturbed"])
    assert np.array_equal(dev["scale"], orc["colscale"])


def test_plain_autotune_and_tlsz_zero(gpu_lib):
    """hsr_autotune_plain records the fastest candidate for the order, and
    tlsz = 0 then solves with it: the same result bit for bit as passing that
    tile size."""
    import torch
    import hsrq3in_gb300 as hsr
    from hsrq3in_gb300 import _lib
    n = 260
    H, lam = G.real_spectrum(n, 41)
    wr = G.perturbed_shifts(lam, 42)
    dev = torch.device("cuda", 0)
    ld = n + (n & 1)
    dH = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dH[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr = torch.from_numpy(wr.copy()).to(dev)
    dX = torch.empty((n, ld), dtype=torch.float64, device=dev)
    best, ms, sc, sc_ms, fused, fz_ms = hsr.autotune_plain(dH, dwr, dX, candidates=(32, 64, 96), detail=True)
    assert best in (32, 64, 96) and all(0 < t < 1e299 for t in ms)
    assert sc in (8, 16, 32) and all(0 < t < 1e299 for t in sc_ms)
    if sc < 32:
        assert all(0 < t < 1e299 for t in fz_ms) and fused == (fz_ms[1] <= fz_ms[0])
    else:
        assert fz_ms == [-1.0, -1.0] and not fused
    assert np.array_equal(dwr.cpu().numpy(), wr)                 # restored
    assert _lib.load().hsr_autotune_plain_tlsz(n) == best
    a = hsr.inverse_iteration(H, wr, 0, 16)
    b = hsr.inverse_iteration(H, wr, best, 16)
    assert np.array_equal(a["vr"], b["vr"]) and np.array_equal(a["wr"], b["wr"])


def test_integer_pipe_division(gpu_lib):
    """The integer-pipe division the Givens rotation uses for its two
    quotients returns the FP64 division's results bit for bit on about 1.6e8
    seeded operand sets (random and edge-case significands, the whole normal
    exponent range), most of them on the integer path."""
    import ctypes as C
    lib = gpu_lib
    counts = (C.c_longlong * 4)()
    assert lib.hsr_selftest_arith(1024, 0x5eed1234, counts) == 0
    assert counts[3] >= 1024 * 256 * 4 * 100
    assert counts[2] > 0.8 * counts[3]
    assert (counts[0], counts[1]) == (0, 0)


def test_device_call_after_host_call_with_fewer_shifts(gpu_lib):
    """A device-resident call that passes no scale buffer writes no scales.
    An earlier host call on the same thread leaves the workspace's scale
    buffer sized for its own 8 shifts; the device call's 1000 columns must
    not be written there (that would run past the buffer into other device
    allocations), so every column is finite, converged and equal to the
    oracle bit for bit."""
    import torch
    import hsrq3in_gb300 as hsr
    H0, lam0 = G.real_spectrum(40, 61)
    hsr.inverse_iteration(H0, G.perturbed_shifts(lam0, 62)[:8], 8, 4)
    n = 1000
    H, lam = G.real_spectrum(n, 63)
    wr = G.perturbed_shifts(lam, 64)
    dev = torch.device("cuda", 0)
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr = torch.from_numpy(wr.copy()).to(dev)
    dX = torch.empty((n, n), dtype=torch.float64, device=dev)
    d_status = torch.zeros(n, dtype=torch.int32, device=dev)
    assert hsr.inverse_iteration_device(dH, dwr, dX, 200, d_status=d_status) == 0
    X = dX.cpu().numpy().T
    assert np.all(np.isfinite(X)) and int(d_status.sum().item()) == n
    cols = np.array([0, 333, 999])
    orc = O.oracle_inverse_iteration(H, wr[cols], 200, 1, intscale=1, variant="fma")
    assert np.array_equal(X[:, cols], orc["vr"])
