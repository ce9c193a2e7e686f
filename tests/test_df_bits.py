"""The bit-level double <-> double-float conversions that the double-float
kernels use at their storage boundary (mini_mdft_gb300/csrc/common.cuh),
checked on the host: df_bits_check.cu includes the same header, and its
functions are __host__ __device__, so the host build runs the device code
path.  f2d_bits must equal the hardware float->double conversion bit for
bit; df_from_double_bits must hold x to 2^-47 in the double-float range and
map the rest to truncated floats, +-inf or NaN; df_to_double must round
hi + lo to the nearest double."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "mini_mdft_gb300", "csrc")


def test_df_conversions_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "df_bits_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", CSRC, "-x", "cu",
                    os.path.join(HERE, "df_bits_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok"), out.stdout
