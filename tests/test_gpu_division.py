"""The setup pass's shared-reciprocal division (div_by in rast_kernels.cu: Markstein's correction
step after a correctly rounded reciprocal) against __fdiv_rn, on a strided sample of all
significand pairs: every b significand with every 1024th a significand (2^36 pairs). The full
check, tests/cuda/div_by_check.cu with stride 1 (all 2^46 pairs, about 40 s), found no difference
either."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_div_by_matches_fdiv_rn(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "div_by_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                    os.path.join(HERE, "cuda", "div_by_check.cu")], check=True, capture_output=True)
    r = subprocess.run([exe, "1024"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["status"] == "no error", out
    assert out["pairs"] == 1 << 36
    assert out["mismatches"] == 0, out
    assert r.returncode == 0
