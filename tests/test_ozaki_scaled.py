"""Host check of the exact integer-to-double conversion used by the epilogues
of the tensor-core products (taurus_vap_gb300/csrc/ozaki_scaled.h)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, os.pardir, "taurus_vap_gb300", "csrc")


def test_scaled_matches_fp64_formula(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "ozaki_scaled_check.cpp"), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "bad 0" in out.stdout
