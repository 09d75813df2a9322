"""The reference's C++ call pattern, compiled unchanged against the
include/yell_gb300 facade, run on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_facade_example_runs(cuda, tmp_path):
    exe = tmp_path / "facade_example"
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f"-I{ROOT}/include/yell_gb300",
           f"{ROOT}/tests/cpp/facade_example.cpp", f"-L{ROOT}/yell_gb300", "-lyell_gb300",
           f"-Wl,-rpath,{ROOT}/yell_gb300", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def test_cpp_facade_samplers_and_lifting(cuda, tmp_path):
    exe = tmp_path / "facade_samplers"
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f"-I{ROOT}/include/yell_gb300",
           f"{ROOT}/tests/cpp/facade_samplers.cpp", f"-L{ROOT}/yell_gb300", "-lyell_gb300",
           f"-Wl,-rpath,{ROOT}/yell_gb300", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


def test_cpp_facade_32bit_mode(cuda, tmp_path):
    """The same reference call pattern built in the reference's 32-bit moduli mode."""
    exe = tmp_path / "facade_example32"
    cmd = ["g++", "-std=c++17", "-O2", "-DYELL_USE_32BITS_MODULI", f"-I{ROOT}/include",
           f"-I{ROOT}/include/yell_gb300", f"{ROOT}/tests/cpp/facade_example32.cpp",
           f"-L{ROOT}/yell_gb300", "-lyell_gb300", f"-Wl,-rpath,{ROOT}/yell_gb300", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr
