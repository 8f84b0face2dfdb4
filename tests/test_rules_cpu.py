"""The division-free decision helpers of the CUDA rules (gbp_rules.cuh) decide exactly like the divisions they
replace: a host build of the header is checked on millions of random and boundary-adversarial inputs."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_quotient_helpers_match_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "rules_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-x", "cu", os.path.join(HERE, "native", "rules_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert out.stdout.startswith("ok")
