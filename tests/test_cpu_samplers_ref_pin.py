"""The sampler and CRT-lifting oracles pinned to the reference's own code.

tests/golden/yell_ref_samplers.npz holds what the reference's own
poly<N>::set(uniform / ZO_dist / hwt_dist)
(include/yell/details/poly.hpp:195-330), FastGaussianNoise
(include/yell/prng/FastGaussianNoise.hpp) and gmp::poly2mpz
(include/yell/gmp.hpp:42-70, lib/gmp.cpp:6-51) produced on the counter stream
the device samplers read (tests/golden/make_golden_samplers.py).  Here:
* uniform, ZO and HWT from oracle/samplers_oracle.c equal the reference's
  output word for word;
* the Gaussian sampler's cumulative table (the oracle's and the library's
  host computation, yell_gaussian_table) equals the 64 most significant bits
  of every barrier of the reference's MPFR-built table, so the two samplers
  draw each value with probabilities within 2^-63 of each other; and the
  reference sampler's own draws follow that table (chi-square);
* oracle/crt.py returns the reference's poly2mpz integers, edge residues
  included.
Where the reference build is present the same comparisons also run live at
more sizes."""
import math
import os

import numpy as np
import pytest

import oracle
import yell_gb300 as y
from oracle.crt import poly2bigint

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "yell_ref_samplers.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


def _cases(g, kind):
    i = 0
    while f"{kind}_{i}" in g:
        yield g[f"{kind}_{i}"], [int(v) for v in g[f"{kind}_{i}_args"]]
        i += 1


def test_uniform_equals_reference(g, orc):
    n = 0
    for want, (count, L, log_n, seed) in _cases(g, "uniform"):
        assert np.array_equal(orc.sample_uniform(count, L, log_n, seed=seed), want)
        n += 1
    assert n == 3


def test_zo_equals_reference(g, orc):
    n = 0
    for want, (count, L, log_n, rho, seed) in _cases(g, "zo"):
        assert np.array_equal(orc.sample_zo(count, L, log_n, rho=rho, seed=seed), want), (log_n, rho)
        n += 1
    assert n == 5


def test_hwt_equals_reference(g, orc):
    n = 0
    for want, (count, L, log_n, h, seed) in _cases(g, "hwt"):
        got = orc.sample_hwt(count, L, log_n, h, seed=seed)
        assert np.array_equal(got, want), (log_n, h)
        assert all(int((want[j, 0] != 0).sum()) == h for j in range(count))
        n += 1
    assert n == 9


def _tail(info):
    return (int(info[0]) - 1) // 2


@pytest.mark.parametrize("i", [0, 1, 2])
def test_gaussian_table_equals_reference_barriers(g, orc, ylib, i):
    sigma, security, samples = g[f"gauss_{i}_args"]
    top = g[f"gauss_{i}_top64"]
    tail = _tail(g[f"gauss_{i}_info"])
    assert len(top) == 2 * tail + 1
    port = orc.gaussian_cdt(float(sigma), tail)
    lib = y.gaussian_table(float(sigma), tail)
    assert np.array_equal(port, lib)  # the oracle restates the library's table rule
    assert np.array_equal(lib, top), "table differs from the reference's barriers"


@pytest.mark.parametrize("i", [0, 2])
def test_reference_gaussian_draws_follow_the_table(g, i):
    """The reference's own draws on the counter stream against the pmf of the
    shared table: chi-square over the values with expected count >= 5."""
    draws = g[f"gauss_{i}_draws"]
    top = g[f"gauss_{i}_top64"].astype(object)
    tail = _tail(g[f"gauss_{i}_info"])
    prev, pmf = 0, []
    for t in top:
        pmf.append((int(t) - prev) / 2**64)
        prev = int(t)
    n = len(draws)
    assert np.abs(draws).max() <= tail
    counts = np.bincount(draws + tail, minlength=2 * tail + 1)
    e = np.array(pmf) * n
    keep = e >= 5
    chi2 = float((((counts[keep] - e[keep]) ** 2) / e[keep]).sum())
    dof = int(keep.sum()) - 1
    assert chi2 < dof + 6 * math.sqrt(2 * dof), (chi2, dof)


@pytest.mark.parametrize("L", [1, 2, 5, 32])
def test_crt_equals_reference_poly2mpz(g, orc, L):
    limbs = g[f"crt_{L}_limbs"]
    words = g[f"crt_{L}_words"]
    primes = [orc.prime(j) for j in range(L)]
    want = [int.from_bytes(words[i].astype("<u8").tobytes(), "little") for i in range(words.shape[0])]
    assert list(poly2bigint(limbs, primes)) == want
    assert want[0] == 0 and want[2] == 12345


@pytest.mark.skipif(not oracle.ref_samplers_available(), reason="reference sampler build absent")
@pytest.mark.parametrize("log_n", [3, 5, 11, 13, 16])
def test_live_against_reference_build(orc, log_n):
    ref = oracle.RefSamplers()
    n = 1 << log_n
    assert np.array_equal(ref.sample_uniform(2, 3, log_n, 101), orc.sample_uniform(2, 3, log_n, seed=101))
    for rho in (0, 0x7F, 0xFE):
        assert np.array_equal(ref.sample_zo(2, 2, log_n, rho, 102), orc.sample_zo(2, 2, log_n, rho=rho, seed=102))
    for h in sorted({1, min(64, n), n // 2, n}):
        assert np.array_equal(ref.sample_hwt(2, 2, log_n, h, 103), orc.sample_hwt(2, 2, log_n, h, seed=103)), h
