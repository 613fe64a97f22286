"""The integer double -> (hi, lo) float split of the double-float operator
(df_split in csrc/kernels.cuh) equals the FP64-conversion split bit for bit
on the device: tests/split_check.cu, compiled here with nvcc for sm_103a,
runs both on 16 M doubles covering every exponent field (zero, subnormal,
normal, beyond float range) with forced ties and carries."""
import os
import subprocess

import pytest

from sparlab_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))

pytestmark = pytest.mark.gpu


def test_split_matches_fp64_conversion(tmp_path):
    exe = str(tmp_path / "split_check")
    subprocess.check_call([B.nvcc()] + B.ARCH + ["-O3", "-std=c++17", "--expt-relaxed-constexpr",
                                                  "-I", B.CSRC, "-I", os.path.join(os.path.dirname(HERE), "include"),
                                                  os.path.join(HERE, "split_check.cu"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 of" in r.stdout
