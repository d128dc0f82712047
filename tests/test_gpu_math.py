"""The step kernels' math helpers against CUDA's own functions on the GPU.

The kernels replace the library rcbrt of the hourglass coefficient
(src/domain.jl:1605) with inv_cbrt, form several reciprocals of one element
from one division (recip3) and take square roots as x * rsqrt(x). Bars, in
units in the last place of the CUDA result over 2^20 log-uniform inputs:
inv_cbrt within 2 ulps of rcbrt (on 1e-36..1e30, both of its branches),
recip3 within 4 ulps of each division, x * rsqrt(x) within 2 ulps of sqrt.
"""
import json
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_math_helpers_match_cuda(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "gpu_math_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", os.path.join(ROOT, "lulesh.jl_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "gpu_math_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    assert r["n"] == 1 << 20
    assert r["inv_cbrt_ulps"] <= 2.0, r
    assert r["recip3_ulps"] <= 4.0, r
    assert r["sqrt_ulps"] <= 2.0, r
