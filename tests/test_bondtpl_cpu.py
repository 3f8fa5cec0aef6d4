"""The per-bond arithmetic of the compact-record force paths
(pd_gpu1_gb300/csrc/bondtpl.h), compiled for the host and checked against
quadruple precision: the 2-D bond on three million lattice bonds (extension
and force within 2e-13 of the strain scale, hardware-like reciprocal seeds),
its break decision against the double test on two million extensions around
the threshold, the 3-D stretch (extension, 1/L and direction) on the
bonds of a 3-D lattice, and the ADR damping term (within 8 units of 2^-53 of
the exact value of the reference's formula)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_bond_arithmetic_against_quad_precision(tmp_path):
    exe = tmp_path / "bondtpl_check"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "pd_gpu1_gb300", "csrc"), os.path.join(ROOT, "tests", "cpp",
                                                                              "bondtpl_check.cpp"),
                        "-o", str(exe), "-lquadmath"], capture_output=True, text=True)
    if r.returncode != 0 and "quadmath" in (r.stderr + r.stdout):
        pytest.skip("no libquadmath on this host")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "break decisions: 2000000 checked, 0 differ" in out.stdout
    assert "3-D stretch: worst extension" in out.stdout
    assert "damping terms: " in out.stdout
