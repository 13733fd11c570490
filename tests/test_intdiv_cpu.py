"""The integer-pipe division the Givens rotation uses (hsr_device.cuh:
ip_recip, ip_quot, ip_div_ok) compiled for the host and compared bit for bit
with the host's IEEE double division on 2e7 seeded operand sets.  IEEE
division is correctly rounded, so the device's FP64 division gives the same
bits; the GPU self-test (test_integer_pipe_division) checks the device build
of the same code against the device's division."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_pipe_division_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "intdiv_check")
    src = os.path.join(HERE, "native", "intdiv_check.cu")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-o", exe, src],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe, "20000000"], check=False, capture_output=True, text=True, timeout=600)
    fast, bad = (int(v) for v in out.stdout.strip().split()[-2:])
    assert out.returncode == 0 and bad == 0, out.stdout
    assert fast > 0.9 * 20000000
