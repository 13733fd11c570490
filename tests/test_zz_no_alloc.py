"""The no-allocation entry point against the allocating one.

hsr_inverse_iteration_noalloc exists for callers that may not call cudaMalloc
while they run (device memory owned by a caching allocator or a fixed pool,
or a plug-in host that forbids its plug-ins to allocate): it takes every
buffer beyond its inputs and outputs from one fixed __device__ array.  This
file runs last (pytest collects it last) so that a failure here cannot hide
the other tests; it passes on its own in a fresh process as well as after
them.  Results must be bit-identical to hsr_inverse_iteration_device, the
same tolerance the other device tests use, on two calls in a row (the shared
array keeps the previous call's contents).
"""
import ctypes as C

import numpy as np
import pytest

from hsrq3in_gb300 import generators as G

pytestmark = pytest.mark.gpu


def _colmajor(torch, A, ld, dev):
    """Device copy of A (n x m, Fortran order) as a (m, ld) tensor: column j
    of A is row j of the tensor, so the leading dimension is ld."""
    n, m = A.shape
    t = torch.zeros((m, ld), dtype=torch.float64, device=dev)
    t[:, :n] = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
    return t


@pytest.mark.parametrize("n,tlsz,nrhs,seed,ld", [
    (200, 40, 150, 31, 200),   # several tiles, even leading dimension
    (97, 24, 97, 32, 97),      # odd leading dimension: H is staged in the array
    (64, 64, 40, 33, 66),      # one tile
    (256, 32, 256, 34, 256),   # the stated maximum size
])
def test_noalloc_matches_device_entry(gpu_lib, n, tlsz, nrhs, seed, ld):
    import torch
    from hsrq3in_gb300 import _lib
    lib = gpu_lib
    dev = torch.device("cuda", 0)
    H, lam = G.real_spectrum(n, seed)
    wr0 = G.perturbed_shifts(lam, seed + 1)[:nrhs]
    dH = _colmajor(torch, H, ld, dev)
    stream = torch.cuda.current_stream(dev)

    # Allocating device entry point.
    dwr = torch.from_numpy(wr0.copy()).to(dev)
    dX = torch.full((nrhs, ld), float("nan"), dtype=torch.float64, device=dev)
    opt = _lib.Options(0, 0, -1, 0.0)
    rc = lib.hsr_inverse_iteration_device(n, dH.data_ptr(), ld, nrhs, dwr.data_ptr(), tlsz,
                                          dX.data_ptr(), ld, C.byref(opt),
                                          C.c_void_p(stream.cuda_stream), None, None)
    assert rc in (0, 1)
    torch.cuda.synchronize()
    ref_X = dX[:, :n].cpu().numpy()
    ref_wr = dwr.cpu().numpy()

    for call in range(2):
        dwr2 = torch.from_numpy(wr0.copy()).to(dev)
        dX2 = torch.full((nrhs, ld), float("nan"), dtype=torch.float64, device=dev)
        status = np.zeros(nrhs, dtype=np.int32)
        rc2 = lib.hsr_inverse_iteration_noalloc(n, dH.data_ptr(), ld, nrhs, dwr2.data_ptr(), tlsz,
                                                dX2.data_ptr(), ld, 0, C.c_void_p(stream.cuda_stream),
                                                status.ctypes.data)
        torch.cuda.synchronize()
        assert rc2 == rc, (call, rc2, rc)
        assert np.array_equal(dwr2.cpu().numpy(), ref_wr), call
        assert np.array_equal(dX2[:, :n].cpu().numpy(), ref_X), call
        assert status.sum() == nrhs if rc == 0 else status.sum() < nrhs


def test_noalloc_rejects_oversize(gpu_lib):
    """Sizes beyond the stated maximum are rejected before any GPU work."""
    from hsrq3in_gb300 import _lib
    lib = gpu_lib
    big = _lib.NOALLOC_MAX_N + 4
    rc = lib.hsr_inverse_iteration_noalloc(big, C.c_void_p(16), big, 8, C.c_void_p(16), 4,
                                           C.c_void_p(16), big, 0, None, None)
    assert rc == _lib.HSR_ERR_ARG
    rc = lib.hsr_inverse_iteration_noalloc(16, C.c_void_p(16), 16, _lib.NOALLOC_MAX_NRHS + 1,
                                           C.c_void_p(16), 4, C.c_void_p(16), 16, 0, None, None)
    assert rc == _lib.HSR_ERR_ARG
