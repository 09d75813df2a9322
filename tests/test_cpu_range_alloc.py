"""Host-only unit test of the server's HBM range allocator (C++)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_range_allocator(tmp_path):
    exe = tmp_path / "range_alloc_test"
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT}/yell_gb300/csrc",
                        f"{ROOT}/tests/cpp/range_alloc_test.cpp", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout
