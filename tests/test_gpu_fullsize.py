"""The plain large configuration at its full size: n = 10000, all 10000
eigenvalues (relative 1e-12 noise) as shifts, device-resident, at the
benchmark's tile size 160 and at 200.

Size-independent properties over every column -- finite, converged, unit
2-norm, device residual ||Hx - lambda x|| / (||H||_F ||x||) <= 10 n eps --
and, because each column's arithmetic does not depend on the other columns
of the solve, bit-for-bit agreement with the oracle on 6 columns sampled from
the full solve.  The input comes from the benchmark's generator and cache.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


@pytest.mark.parametrize("tlsz", [160, 200])
def test_plain_large_full_size(gpu_lib, tlsz):
    import torch
    import bench
    import hsrq3in_gb300 as hsr
    n = 10000
    H, wr = bench.workload(n, 1234)
    dev = torch.device("cuda:0")
    ld = n + (n & 1)
    dH = torch.zeros((n, ld), dtype=torch.float64, device=dev)
    dH[:, :n] = torch.from_numpy(np.ascontiguousarray(H.T)).to(dev)
    dwr = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    dX = torch.empty((n, ld), dtype=torch.float64, device=dev)
    d_status = torch.zeros(n, dtype=torch.int32, device=dev)
    rc = hsr.inverse_iteration_device(dH, dwr, dX, tlsz, d_status=d_status)
    torch.cuda.synchronize()
    assert rc == 0
    assert bool(torch.isfinite(dX[:, :n]).all().item())
    assert int(d_status.sum().item()) == n
    norms = torch.linalg.norm(dX[:, :n], dim=1).cpu().numpy()
    assert np.all(np.abs(norms - 1.0) <= 1e-13)
    res = hsr.residuals_device(dH, dwr, dX).cpu().numpy()
    assert res.max() <= 10 * n * EPS, res.max()
    # No column needed a restart, so the shifts kept their order.
    assert np.array_equal(dwr.cpu().numpy(), wr)
    cols = np.array([0, 1777, 4242, 6001, 8888, n - 1])
    orc = O.oracle_inverse_iteration(H, wr[cols], tlsz, 1, intscale=1, variant="fma")
    got = dX[torch.from_numpy(cols).to(dev), :n].cpu().numpy().T
    assert np.array_equal(got, orc["vr"])
