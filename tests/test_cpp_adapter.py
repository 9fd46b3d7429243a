"""The C++ drop-in header compiles against the C ABI and, called like the
reference's main.cu calls inc/pagerankCuda.hxx, matches the oracle; and a
main.cu-shaped unit built against the reference's own headers (DiGraph,
batch, transpose, OpenMP PageRank, the reference's PagerankOptions /
PagerankResult) compiles and links with it."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, REFERENCE_DIR, ROOT


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


def _compile_with_reference(out):
    """nvcc build of tests/cpp/test_adapter_reference.cu against the
    reference's inc/ headers (skipped where they are absent)."""
    inc = os.path.join(REFERENCE_DIR, "inc") if REFERENCE_DIR else None
    if not inc or not os.path.isfile(os.path.join(inc, "pagerank.hxx")):
        pytest.skip("the reference's headers are not present")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    import pagerank_gb300
    lib = pagerank_gb300.library_path()
    if not os.path.exists(lib):
        pagerank_gb300.load()
    libdir = os.path.dirname(lib)
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fopenmp",
           "-I", inc, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_adapter_reference.cu"), "-o", out,
           "-L", libdir, "-lpagerank_gb300", f"-Xlinker=-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_adapter_with_reference_types_compiles(tmp_path):
    _compile_with_reference(str(tmp_path / "test_adapter_reference"))


@pytest.mark.gpu
def test_adapter_with_reference_types_runs(tmp_path):
    exe = str(tmp_path / "test_adapter_reference")
    _compile_with_reference(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
