"""The setup pass's shared-reciprocal division (rast::div_by and rast::div_by_recip in
rast_exact.cuh: Markstein's correction step after a correctly rounded reciprocal) against
__fdiv_rn. The check program calls the header's functions themselves, on a strided sample of all
significand pairs (every b significand with every 1024th a significand: 2^36 pairs), on every pair
of 64 special values around the range guard (2^-60, 2^60 and their neighbours, zeros, infinities,
NaN, subnormals) and on 2^24 random pairs with exponents in [-70, 70]. With stride 1 the program
checks all 2^46 significand pairs (about 40 s); that run found no difference either."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rasteriser_gb300", "csrc")


def test_div_by_matches_fdiv_rn(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "div_by_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-prec-div=true",
                    "-ftz=false", "-I" + CSRC, "-o", exe, os.path.join(HERE, "cuda", "div_by_check.cu")],
                   check=True, capture_output=True)
    r = subprocess.run([exe, "1024"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["status"] == "no error", out
    assert out["pairs"] == 1 << 36
    assert out["mismatches"] == 0, out
    assert out["edge_pairs"] == 64 * 64 and out["edge_mismatches"] == 0, out
    assert out["random_pairs"] == 1 << 24 and out["random_mismatches"] == 0, out
    assert r.returncode == 0
