"""The C ABI without a GPU: exports, host-side tables, argument checks."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "yell_ref_vectors.npz")


def test_library_exports_every_header_symbol(ylib):
    syms = _capi.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(ylib, s)]
    assert missing == []
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(syms) <= exported


def test_signature_table_covers_header():
    assert set(_capi.header_symbols()) <= set(_capi.SIGNATURES)


def test_abi_and_ranges(ylib):
    assert ylib.yell_abi_version() == 1
    assert y.max_moduli() == 1000
    assert (y.min_log_degree(), y.max_log_degree()) == (3, 20)
    assert ylib.yell_prime(1000) == 0


def test_prime_table_equals_reference(ylib):
    g = np.load(GOLDEN)
    for cm in range(1000):
        assert ylib.yell_prime(cm) == int(g["P"][cm])
        assert ylib.yell_prime_pn(cm) == int(g["Pn"][cm])
        assert ylib.yell_primitive_root(cm) == int(g["roots"][cm])


def test_host_tables_equal_reference(ylib, orc):
    g = np.load(GOLDEN)
    t, sc = y.ntt_tables(4, 0)
    assert np.array_equal(t, g["tables_4_0"]) and np.array_equal(sc, g["tables_4_0_scalars"])
    for log_n, cm in ((10, 3), (13, 999)):
        t, sc = y.ntt_tables(log_n, cm)
        to, so = orc.tables(log_n, cm)
        assert np.array_equal(t, to) and np.array_equal(sc, so)


def test_argument_errors_without_touching_cuda(ylib):
    buf = np.zeros(16, np.uint64)
    addr = buf.ctypes.data
    assert ylib.yell_ntt_forward(addr, 2, 0) == _capi.YELL_ERR_UNSUPPORTED_DEGREE
    assert ylib.yell_ntt_forward(addr, 21, 0) == _capi.YELL_ERR_UNSUPPORTED_DEGREE
    assert ylib.yell_ntt_backward(addr, 4, 1000) == _capi.YELL_ERR_INVALID_MODULUS
    assert ylib.yell_ntt_forward(None, 4, 0) == _capi.YELL_ERR_INVALID_ARGUMENT
    assert ylib.yell_dev_ntt(addr + 8, 1, 1, 4, 0, 0, None) == _capi.YELL_ERR_INVALID_ARGUMENT
    assert b"aligned" in ylib.yell_last_error()
    assert ylib.yell_dev_ntt(addr, 1, 1, 4, 0, 7, None) == _capi.YELL_ERR_INVALID_ARGUMENT
    assert ylib.yell_dev_polymul(addr, addr, addr, 1, 1, 4, 0, None, 0, None) == \
        _capi.YELL_ERR_INVALID_ARGUMENT
    assert ylib.yell_dev_elementwise(9, addr, addr, addr, 1, 1, 4, 0, None) == \
        _capi.YELL_ERR_INVALID_ARGUMENT
    assert ylib.yell_status_string(2) == b"unsupported degree"


def test_limb_count_overflow_rejected(ylib):
    """pairs * L (or count * L) beyond what one launch covers, in particular
    any product >= 2^32, is refused before any CUDA call; no entry point may
    wrap the product and run a truncated batch."""
    fake = [0x10000, 0x20000, 0x30000]  # aligned, never dereferenced: the check comes first
    big = 1 << 31
    E = _capi.YELL_ERR_INVALID_ARGUMENT
    assert ylib.yell_dev_polymul(*fake, big, 2, 16, 0, None, 0, None) == E
    assert b"limbs" in ylib.yell_last_error()
    assert ylib.yell_dev_polymul(*fake, (1 << 32) - 1, 1000, 10, 0, None, 0, None) == E
    assert ylib.yell_dev_polymul_noalloc(*fake, big, 2, 16, 0, None) == E
    assert ylib.yell_dev_ntt(fake[0], big, 4, 12, 0, 0, None) == E
    assert ylib.yell_dev_elementwise(0, *fake, big, 2, 12, 0, None) == E
    assert ylib.yell_dev_sample_uniform(fake[0], big, 2, 12, 0, 1, None) == E
    assert ylib.yell_dev_crt_lift(fake[0], fake[1], big, 2, 12, 0, None) == E
    # 2^20: one call takes at most (2^31 - 1) >> 8 limbs (4096-word tiles in a grid)
    assert ylib.yell_dev_polymul(*fake, 1 << 23, 1, 20, 0, None, 0, None) == E
    assert y.polymul_scratch_words(big, 2, 16) == 0
    assert y.polymul_scratch_words(1 << 23, 1, 20) == 0
    assert y.polymul_scratch_words((1 << 23) - 1, 1, 20) == ((1 << 23) - 1) << 20


def test_polymul_scratch_sizes(ylib):
    assert y.polymul_scratch_words(16, 32, 12) == 0
    assert y.polymul_scratch_words(16, 32, 13) == 16 * 32 << 13  # two-pass variants at 2^13
    assert y.polymul_scratch_words(16, 32, 16) == 16 * 32 << 16
    assert y.polymul_scratch_words(1, 1, 21) == 0


def test_no_kernel_ran_on_cpu(ylib):
    assert y.kernel_launches() == 0


def test_library_fails_loudly_without_build():
    code = ("import yell_gb300._capi as c; c._lib=None\n"
            "try:\n    c.load('/nonexistent/libyell_gb300.so')\nexcept RuntimeError as e:\n"
            "    print('raised', 'missing' in str(e))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT)
    assert "raised True" in r.stdout


def test_prime_table_regenerates():
    """gen_prime_table.py reproduces the committed prime_table.inc."""
    sys.path.insert(0, os.path.join(ROOT, "yell_gb300", "csrc"))
    import gen_prime_table as g

    primes, pn, roots = g.generate(64)
    committed = open(os.path.join(ROOT, "yell_gb300", "csrc", "prime_table.inc")).read()
    lines = g.render(primes, pn, roots).splitlines()[2:]
    assert all(line in committed for line in lines)


def test_cpp_facade_compiles(tmp_path):
    exe = tmp_path / "facade_example"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", f"-I{ROOT}/include/yell_gb300",
           f"{ROOT}/tests/cpp/facade_example.cpp", f"-L{ROOT}/yell_gb300", "-lyell_gb300",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_facade_math_helpers(tmp_path):
    """yell/utils/math.hpp (host helpers): compiled and run on the CPU."""
    exe = tmp_path / "facade_math"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", f"-I{ROOT}/include/yell_gb300",
           f"{ROOT}/tests/cpp/facade_math.cpp", f"-L{ROOT}/yell_gb300", "-lyell_gb300",
           f"-Wl,-rpath,{ROOT}/yell_gb300", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr
