"""The C ABI library: it loads and exports every function the header
declares; argument checking needs no GPU.  No compute calls here."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hsrq3in_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = "\n".join(ln for ln in src.splitlines() if not ln.lstrip().startswith("#"))
    return sorted(set(re.findall(r"\b(\w+)\s*\([^;{]*\)\s*;", src)) - {"sizeof"})


@pytest.fixture(scope="module")
def lib():
    from hsrq3in_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_drop_in_signature():
    src = open(HEADER).read()
    assert re.search(r"void\s+tiled_inverse_iteration\s*\(\s*int n,\s*const double \*H,\s*int ldH,\s*int nrhs,"
                     r"\s*double \*wr,\s*int tlsz,\s*int rhs_tlsz,\s*double \*vr,\s*int ldvr\)", src)


def test_library_exports_every_declared_symbol(lib):
    from hsrq3in_gb300 import _lib
    names = declared_functions()
    assert "tiled_inverse_iteration" in names
    for nm in names:
        assert hasattr(lib, nm), nm
    assert set(names) == set(_lib.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True, text=True).stdout
    for nm in names:
        assert re.search(r"\bT %s\b" % nm, out), nm


def test_sm103a_code_only(lib):
    """The library carries sm_103a code (cuobjdump lists the ELF targets; no
    disassembly is read)."""
    from hsrq3in_gb300 import _lib
    r = subprocess.run(["cuobjdump", "--list-elf", _lib.lib_path()], capture_output=True, text=True)
    assert "sm_103a" in r.stdout
    assert "sm_100" not in r.stdout.replace("sm_103a", "")


def test_argument_errors_without_gpu(lib):
    from hsrq3in_gb300 import _lib
    wr = (C.c_double * 4)()
    vr = (C.c_double * 16)()
    H = (C.c_double * 16)()
    cases = [(0, 4, 4, 4), (4, 3, 4, 4), (4, 4, 6, 4), (4, 4, 4, 3)]   # n, ldH, tlsz, ldvr
    for n, ldH, tlsz, ldvr in cases:
        lib.tiled_inverse_iteration(n, C.cast(H, C.c_void_p), ldH, 4, C.cast(wr, C.c_void_p), tlsz, 4,
                                    C.cast(vr, C.c_void_p), ldvr)
        assert lib.hsr_last_status() == _lib.HSR_ERR_ARG
    assert lib.hsr_status_string(_lib.HSR_ERR_ARG) == b"invalid argument"
    opt = _lib.Options(0, 0, -1, 0.0)
    assert lib.hsr_inverse_iteration_ex(4, C.cast(H, C.c_void_p), 4, 4, C.cast(wr, C.c_void_p), 4, 0,
                                        C.cast(vr, C.c_void_p), 4, C.byref(opt), None) == _lib.HSR_ERR_ARG


def test_complex_argument_errors_without_gpu(lib):
    """The complex-shift entry points reject bad arguments before any CUDA
    call: n, ldH, tlsz (a positive multiple of 4), ldvr, missing shifts, and
    caller right-hand sides (not supported for complex shifts)."""
    from hsrq3in_gb300 import _lib
    wr = (C.c_double * 4)()
    wi = (C.c_double * 4)()
    vr = (C.c_double * 32)()
    H = (C.c_double * 16)()
    opt = _lib.Options(0, 0, -1, 0.0)
    cases = [(0, 4, 4, 4), (4, 3, 4, 4), (4, 4, 6, 4), (4, 4, 4, 3)]   # n, ldH, tlsz, ldvr
    for n, ldH, tlsz, ldvr in cases:
        rc = lib.hsr_inverse_iteration_cplx_ex(n, C.cast(H, C.c_void_p), ldH, 2, C.cast(wr, C.c_void_p),
                                               C.cast(wi, C.c_void_p), tlsz, 4, C.cast(vr, C.c_void_p), ldvr,
                                               C.byref(opt), None)
        assert rc == _lib.HSR_ERR_ARG and lib.hsr_last_status() == _lib.HSR_ERR_ARG
    assert lib.hsr_inverse_iteration_cplx_ex(4, C.cast(H, C.c_void_p), 4, 2, C.cast(wr, C.c_void_p), None, 4, 4,
                                             C.cast(vr, C.c_void_p), 4, C.byref(opt), None) == _lib.HSR_ERR_ARG
    rhs = _lib.Options(0, 1, -1, 0.0)
    assert lib.hsr_inverse_iteration_cplx_ex(4, C.cast(H, C.c_void_p), 4, 2, C.cast(wr, C.c_void_p),
                                             C.cast(wi, C.c_void_p), 4, 4, C.cast(vr, C.c_void_p), 4,
                                             C.byref(rhs), None) == _lib.HSR_ERR_ARG
    assert lib.hsr_inverse_iteration_cplx_device(4, C.cast(H, C.c_void_p), 4, 2, C.cast(wr, C.c_void_p),
                                                 C.cast(wi, C.c_void_p), 6, C.cast(vr, C.c_void_p), 4,
                                                 C.byref(opt), None, None, None) == _lib.HSR_ERR_ARG


def test_mixed_layout_errors_without_gpu(lib):
    """Malformed conjugate pairs are rejected before any CUDA call."""
    from hsrq3in_gb300 import _lib
    H = (C.c_double * 16)()
    vr = (C.c_double * 16)()
    opt = _lib.Options(0, 0, -1, 0.0)
    for wr_, wi_ in ([0.1, 0.1], [0.5, 0.5]), ([0.1, 0.1], [-0.5, 0.5]), ([0.1, 0.2], [0.5, -0.5]), \
            ([0.0, 0.1], [0.0, 0.5]):
        wr = (C.c_double * 2)(*wr_)
        wi = (C.c_double * 2)(*wi_)
        rc = lib.hsr_inverse_iteration_mixed(4, C.cast(H, C.c_void_p), 4, 2, C.cast(wr, C.c_void_p),
                                             C.cast(wi, C.c_void_p), 4, 4, C.cast(vr, C.c_void_p), 4,
                                             C.byref(opt), None)
        assert rc == _lib.HSR_ERR_ARG, (wr_, wi_)


def test_version_string(lib):
    assert b"sm_103a" in lib.hsr_version()


def test_header_compiles_as_c_and_links(lib, tmp_path):
    """A C99 caller: the header beside the reference's own declaration of the
    entry point (inverse_iteration.h:19-22, restrict-qualified pointers)
    compiles with -Wall -Wextra -pedantic -Werror, so the two declarations
    are compatible; the address of every declared function resolves against
    the library at link time; the program then runs a call that needs no GPU."""
    from hsrq3in_gb300 import _lib
    names = declared_functions()
    prog = tmp_path / "caller.c"
    prog.write_text("\n".join([
        "#include <stdio.h>",
        "#include \"hsrq3in_gb300.h\"",
        "void tiled_inverse_iteration(int n, const double *restrict H, int ldH, int nrhs,",
        "                             double *restrict wr, int tlsz, int rhs_tlsz,",
        "                             double *restrict vr, int ldvr);",
        "typedef void (*any_fn)(void);",
        "int main(void) {",
        "    any_fn fns[] = {" + ", ".join("(any_fn)%s" % nm for nm in names) + "};",
        "    int resolved = 0;",
        "    for (size_t i = 0; i < sizeof fns / sizeof fns[0]; ++i) resolved += fns[i] != 0;",
        "    printf(\"%d %s\\n\", resolved, hsr_version());",
        "    return 0;",
        "}", ""]))
    libdir = os.path.dirname(_lib.lib_path())
    exe = tmp_path / "caller"
    cc = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                         "-I", os.path.join(ROOT, "include"), str(prog), "-L", libdir, "-lhsrq3in_gb300",
                         "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stderr
    count, version = run.stdout.split(" ", 1)
    assert int(count) == len(names)
    assert version.strip() == lib.hsr_version().decode()

