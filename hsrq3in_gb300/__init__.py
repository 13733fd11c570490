"""hsrq3in_gb300 -- robust level-3 inverse iteration on GB300 (sm_103a).

The product is the C-ABI shared library ``libhsrq3in_gb300.so`` declared in
``include/hsrq3in_gb300.h``; this package builds it (``build.py``), binds it
(``_lib.py``), wraps it for numpy and torch callers (``api.py``), and ships
the seeded workload generators (``generators.py``).
"""
from .api import (BatchPlan, HsrError, Server, autotune_batch, autotune_plain, fp64_peak,  # noqa: F401
                  hessenberg_apply_q_device, hessenberg_device,
                  inverse_iteration, inverse_iteration_cplx, inverse_iteration_cplx_device, inverse_iteration_mixed,
                  inverse_iteration_device, last_launch_count,
                  residuals_device, tiled_inverse_iteration)
from ._lib import lib_path, load  # noqa: F401

__all__ = ["BatchPlan", "Server", "autotune_batch", "autotune_plain", "HsrError", "fp64_peak", "inverse_iteration", "inverse_iteration_cplx",
           "inverse_iteration_cplx_device", "inverse_iteration_mixed", "inverse_iteration_device",
           "last_launch_count", "residuals_device", "hessenberg_device", "hessenberg_apply_q_device", "tiled_inverse_iteration", "lib_path", "load"]
