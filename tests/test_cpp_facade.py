"""The C++ facade (include/fideslib_gb300.hpp): compiles on any host; its example runs on the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")


def gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_facade_header_compiles():
    r = subprocess.run([gxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_example_runs(engine_lib, tmp_path):
    from fideslib_gb300 import build as B
    lib_dir = os.path.dirname(B.lib_path())
    exe = str(tmp_path / "facade_check")
    r = subprocess.run([gxx(), "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-L", lib_dir,
                        "-lfideslib_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "facade ok" in run.stdout
