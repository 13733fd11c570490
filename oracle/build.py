"""Build recipes for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

``build_oracle()`` compiles the plain-C restatement ``oracle/hsro.c`` into
``oracle/_build/``:

* ``libhsro_ref.so``  -- reference arithmetic, ``-ffp-contract=off``; the
  parity checker and the CPU port timed by ``bench.py``.
* ``libhsro_fma.so``  -- the CUDA kernels' expression shapes (``-DHSRO_FMA``).
* ``libhsro_ref_fast.so`` -- the reference arithmetic at ``-O3`` with fused
  multiply-add contraction allowed, as the reference's own build does; timed
  as the CPU baseline.

``build_reference()`` compiles the *unmodified* reference sources where they
lie (``$HSRQ3IN_REFERENCE``, default ``/root/reference``, read-only) into
``oracle/_ref/`` -- only when they
are present, which is the case in the development container and never on a
GPU host.  The reference needs BLAS/LAPACK (``dgemm_``, ``dlange_``,
``dlartg_``); it is linked against the OpenBLAS that ships inside scipy,
whose symbols carry a ``scipy_`` prefix, so the reference's calls are renamed
with ``-D<name>_=scipy_<name>_``.  ``oracle/ref_shim.c`` is linked with
``-Wl,--wrap`` around the robust kernels to record protection decisions.
Two variants are built: default double scaling and ``-DINTSCALING``.
"""
from __future__ import annotations

import glob
import os
import platform
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
# Where the reference sources lie: $HSRQ3IN_REFERENCE, else the read-only
# checkout of the development container.
REFERENCE_SRC = os.environ.get("HSRQ3IN_REFERENCE", "/root/reference")

REF_SOURCES = [
    "inverse_iteration.c", "partition.c", "reduce.c", "robust.c",
    "shifted_Hessenberg_solve.c", "solve-task.c", "update-task.c", "utils.c",
    "validation.c",
]
BLAS_RENAMES = ["dgemm_", "dlange_", "dlartg_", "dgehrd_", "dnrm2_", "dgemv_",
                "dlaln2_", "dhseqr_"]
WRAPPED = ["solve_1x1_real_system", "protect_double_update", "protect_update",
           "protect_multi_rhs_update_real"]


def find_openblas() -> str | None:
    """Path of scipy's bundled OpenBLAS (exports scipy_dgemm_ etc.), if any."""
    try:
        import scipy  # noqa: F401
    except Exception:
        return None
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    for pat in ("scipy.libs/libscipy_openblas*.so*", "scipy_openblas*/lib/libscipy_openblas*.so*"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force: bool = False) -> dict[str, str]:
    """Compile the three oracle variants; returns {variant: path}."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "hsro.c")
    hdr = os.path.join(HERE, "hsro.h")
    inc = os.path.join(HERE, "hsro_cplx.c")     # included by hsro.c
    blas = find_openblas()
    link: list[str] = []
    defs: list[str] = []
    if blas:
        defs += ["-DHSRO_DGEMM=scipy_dgemm_",
                 "-DHSRO_BLAS_THREADS=scipy_openblas_set_num_threads"]
        link += [blas, "-Wl,-rpath," + os.path.dirname(blas)]
    variants = {
        "ref": ["-O2", "-ffp-contract=off"],
        "fma": ["-O2", "-ffp-contract=off", "-DHSRO_FMA"],
        "ref_fast": ["-O3", "-ffp-contract=fast", "-funroll-loops"],
    }
    out: dict[str, str] = {}
    for name, flags in variants.items():
        so = os.path.join(BUILD_DIR, "libhsro_%s.so" % name)
        if force or _stale(so, [src, hdr, inc, __file__]):
            cmd = (["gcc", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", "-Wall",
                    "-Wno-unused-function"] + flags + defs + [src, "-o", so] + link + ["-lm"])
            _run(cmd)
        out[name] = so
    return out


def build_reference(force: bool = False) -> dict[str, str]:
    """Compile the unmodified reference into oracle/_ref (when present)."""
    if not os.path.isdir(REFERENCE_SRC):
        return {}
    blas = find_openblas()
    if blas is None:
        raise RuntimeError("scipy's OpenBLAS not found; the reference needs BLAS/LAPACK")
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.c")
    srcs = [os.path.join(REFERENCE_SRC, f) for f in REF_SOURCES]
    out: dict[str, str] = {}
    inc_extra: list[str] = []
    if platform.machine() not in ("x86_64", "AMD64", "i686"):
        # mm_malloc.h is an x86 header; provide a posix_memalign shim.
        shim_inc = os.path.join(REF_DIR, "include")
        os.makedirs(shim_inc, exist_ok=True)
        with open(os.path.join(shim_inc, "mm_malloc.h"), "w") as f:
            f.write("#pragma once\n#include <stdlib.h>\n"
                    "static inline void *_mm_malloc(size_t n, size_t a)"
                    "{ void *p = 0; if (posix_memalign(&p, a < sizeof(void*) ? sizeof(void*) : a, n)) return 0; return p; }\n"
                    "static inline void _mm_free(void *p) { free(p); }\n")
        inc_extra = ["-I" + shim_inc]
    for variant, vdefs in (("", []), ("_int", ["-DINTSCALING"])):
        so = os.path.join(REF_DIR, "libhsrq3in_ref%s.so" % variant)
        if not force and not _stale(so, srcs + [shim, __file__]):
            out["ref" + variant] = so
            continue
        objdir = os.path.join(REF_DIR, "obj%s" % variant)
        os.makedirs(objdir, exist_ok=True)
        cflags = (["gcc", "-std=gnu99", "-O2", "-fopenmp", "-fPIC", "-ffp-contract=off",
                   "-DNDEBUG", "-DALIGNMENT=64", "-w"] + vdefs + inc_extra
                  + ["-D%s=scipy_%s" % (r, r) for r in BLAS_RENAMES])
        objs = []
        for s in srcs:
            o = os.path.join(objdir, os.path.basename(s)[:-2] + ".o")
            _run(cflags + ["-c", s, "-o", o])
            objs.append(o)
        o = os.path.join(objdir, "ref_shim.o")
        _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-c", shim, "-o", o]
             + (["-DSHIM_INTSCALING"] if vdefs else []))
        objs.append(o)
        wraps = ["-Wl,--wrap=" + w for w in WRAPPED]
        _run(["gcc", "-shared", "-fopenmp", "-o", so] + objs + wraps
             + [blas, "-Wl,-rpath," + os.path.dirname(blas), "-lm"])
        out["ref" + variant] = so
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_reference(force))
