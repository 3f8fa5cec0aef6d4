"""The integer exact-subtraction helpers of the bond kernels
(pd_gpu1_gb300/csrc/exact_sub.h), compiled for the host and checked against
the hardware double subtraction on two million operand pairs."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_exact_subtraction_matches_hardware(tmp_path):
    exe = tmp_path / "exact_sub_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "pd_gpu1_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "exact_sub_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
