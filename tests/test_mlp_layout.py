"""Host-side layout of the learned shader's networks (rasteriser_gb300/csrc/rast_mlp.h), on the CPU:
image offsets and sizes, the parameters kept fixed, and the tensor-core operand layout of the
weights (every element at its own slot) for both the compact and the wide network."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


def test_mlp_layouts(tmp_path):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("no CUDA headers or g++")
    exe = str(tmp_path / "mlp_layout_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "rasteriser_gb300", "csrc"), "-I" + inc,
                    os.path.join(ROOT, "tests", "cpp", "mlp_layout_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
