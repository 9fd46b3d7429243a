"""The C++ drop-in header compiles against the C ABI and, called like the
reference's main.cu calls inc/pagerankCuda.hxx, matches the oracle."""
import os
import subprocess

import pytest

from conftest import PKG, ROOT


def _compile(out):
    import pagerank_gb300
    lib = pagerank_gb300.library_path()
    if not os.path.exists(lib):
        pagerank_gb300.load()
    from oracle import pyoracle
    pyoracle.build()
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_adapter.cpp"), "-o", out,
           "-L", libdir, "-lpagerank_gb300", f"-Wl,-rpath,{libdir}",
           "-L", os.path.join(ROOT, "oracle"), "-loracle", f"-Wl,-rpath,{os.path.join(ROOT, 'oracle')}",
           "-fopenmp"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_adapter_compiles(tmp_path):
    _compile(str(tmp_path / "test_adapter"))


@pytest.mark.gpu
def test_adapter_matches_oracle(tmp_path):
    exe = str(tmp_path / "test_adapter")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "MISMATCH" not in r.stdout
