"""The mixed path's integer-pipe FP64 <-> FP32 conversions equal the hardware
conversions bit for bit over the normal FP32 range, and its float-float
toolkit (position splits, differences, products, sums, accumulation) stays
within 2^-44 of FP64 references."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


def test_narrow_and_widen_match_hardware(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "convert_check"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                           "--expt-relaxed-constexpr", "-o", str(exe), str(HERE / "helpers" / "convert_check.cu")])
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "narrow mismatches 0 widen mismatches 0" in res.stdout
    assert "split mismatches 0 diff mismatches 0 ffop mismatches 0 acc mismatches 0" in res.stdout
