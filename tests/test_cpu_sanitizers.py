"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer.

compute-sanitizer is closed on the GPU pool, so the host side is checked
here instead: the CPU oracle (every entry point, edge sizes and values,
invalid arguments) and the serving loop's range allocator, each built with
-fsanitize=address,undefined and no recovery, so any finding fails the run."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]


def _build(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in r.stderr or "ubsan" in r.stderr):
        pytest.skip("sanitizer runtime not available: " + r.stderr.strip().splitlines()[-1])
    assert r.returncode == 0, r.stderr


def _run(exe):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


def test_oracle_under_sanitizers(tmp_path):
    exe = tmp_path / "oracle_sanitize"
    src = [f"{ROOT}/tests/cpp/oracle_sanitize.c"] + [f"{ROOT}/oracle/{f}" for f in
                                                     ("yell_oracle.c", "samplers_oracle.c", "yell_oracle32.c")]
    _build(["gcc", *SAN, "-pthread", *src, "-lm", "-o", str(exe)])
    _run(exe)


def test_range_allocator_under_sanitizers(tmp_path):
    exe = tmp_path / "range_alloc_sanitize"
    _build(["g++", "-std=c++17", *SAN, f"-I{ROOT}/yell_gb300/csrc", f"{ROOT}/tests/cpp/range_alloc_test.cpp",
            "-o", str(exe)])
    _run(exe)
