"""The integer adder of the FP64 sweeps (csrc/prx_softadd.h, compiled here
for the host) against the CPU's IEEE 754 double addition on some 76 million
seeded operand pairs and sequential row sums (tests/cpp/test_softadd.cpp)."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, ROOT


def test_integer_adder_matches_ieee_addition(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = str(tmp_path / "test_softadd")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "test_softadd.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "1"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
