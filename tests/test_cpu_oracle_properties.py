"""Property checks of the oracle (the C restatement of the reference, and of
its 32-bit moduli build) on randomly drawn degrees, moduli and words, beside
the fixed golden vectors:
word-for-word equality with the reference's own compiled sources where that
build is present (NTTs, element-wise ops, the uniform / ZO / HWT samplers),
the negacyclic convolution theorem against the schoolbook product, linearity
of the forward transform, and forward -> backward as the identity.  CPU only;
hypothesis drives the draws."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

import oracle  # noqa: E402
from yell_gb300.inputs import splitmix64  # noqa: E402

SETTINGS = settings(max_examples=40, deadline=None, derandomize=True)


def _words(seed, n, bound):
    x = splitmix64(seed, n) % np.uint64(bound)
    # edge words at fixed places: 0 and the largest word allowed
    x[0] = 0
    x[-1] = bound - 1
    return x


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build not present")
@SETTINGS
@given(log_n=st.integers(3, 13), cm=st.integers(0, 999), seed=st.integers(0, 2**32))
def test_port_equals_reference_build(orc, log_n, cm, seed):
    ref = oracle.Oracle("ref")
    p = orc.prime(cm)
    n = 1 << log_n
    x4 = _words(seed, n, 4 * p)
    assert np.array_equal(orc.forward_lazy(x4, log_n, cm), ref.forward_lazy(x4, log_n, cm))
    assert np.array_equal(orc.forward(x4, log_n, cm), ref.forward(x4, log_n, cm))
    x2 = _words(seed + 1, n, 2 * p)
    assert np.array_equal(orc.backward(x2, log_n, cm), ref.backward(x2, log_n, cm))
    a, b = _words(seed + 2, n, p), _words(seed + 3, n, p)
    assert np.array_equal(orc.mulmod(a, b, cm), ref.mulmod(a, b, cm))
    assert np.array_equal(orc.addmod(a, b, cm), ref.addmod(a, b, cm))
    assert np.array_equal(orc.submod(a, b, cm), ref.submod(a, b, cm))
    a4, b4 = _words(seed + 4, n, 4 * p), _words(seed + 5, n, 4 * p)
    assert np.array_equal(orc.muladd(a, a4, b4, cm), ref.muladd(a, a4, b4, cm))


@SETTINGS
@given(log_n=st.integers(3, 9), cm=st.integers(0, 999), seed=st.integers(0, 2**32))
def test_polymul_is_the_negacyclic_product(orc, log_n, cm, seed):
    p = orc.prime(cm)
    n = 1 << log_n
    a, b = _words(seed, n, p), _words(seed + 7, n, p)
    got = orc.polymul(a[None], b[None], log_n, cm)[0]
    assert np.array_equal(got, orc.schoolbook(a, b, log_n, cm))


@SETTINGS
@given(log_n=st.integers(3, 12), cm=st.integers(0, 999), seed=st.integers(0, 2**32))
def test_forward_is_linear_and_backward_inverts_it(orc, log_n, cm, seed):
    p = orc.prime(cm)
    n = 1 << log_n
    a, b = _words(seed, n, p), _words(seed + 11, n, p)
    fa, fb = orc.forward(a, log_n, cm), orc.forward(b, log_n, cm)
    assert np.array_equal(orc.forward(orc.addmod(a, b, cm), log_n, cm), orc.addmod(fa, fb, cm))
    assert np.array_equal(orc.backward(fa, log_n, cm), a)
    assert int(fa.max()) < p


def _words32(seed, n, bound):
    x = (splitmix64(seed, n) % np.uint64(bound)).astype(np.uint32)
    x[0] = 0
    x[-1] = bound - 1
    return x


@pytest.mark.skipif(not oracle.ref32_available(), reason="reference 32-bit build not present")
@SETTINGS
@given(log_n=st.integers(3, 15), cm=st.integers(0, 290), seed=st.integers(0, 2**32))
def test_port32_equals_reference_build(log_n, cm, seed):
    """The 32-bit moduli restatement against the reference's own sources built
    with -DYELL_USE_32BITS_MODULI: NTTs and element-wise ops word for word."""
    port, ref = oracle.Oracle32("port"), oracle.Oracle32("ref")
    p = port.prime(cm)
    n = 1 << log_n
    x4 = _words32(seed, n, 4 * p)
    assert np.array_equal(port.forward_lazy(x4, log_n, cm), ref.forward_lazy(x4, log_n, cm))
    assert np.array_equal(port.forward(x4, log_n, cm), ref.forward(x4, log_n, cm))
    x2 = _words32(seed + 1, n, 2 * p)
    assert np.array_equal(port.backward(x2, log_n, cm), ref.backward(x2, log_n, cm))
    a, b = _words32(seed + 2, n, p), _words32(seed + 3, n, p)
    for op in ("mulmod", "addmod", "submod"):
        assert np.array_equal(getattr(port, op)(a, b, cm), getattr(ref, op)(a, b, cm)), op
    a4, b4 = _words32(seed + 4, n, 4 * p), _words32(seed + 5, n, 4 * p)
    assert np.array_equal(port.muladd(a, a4, b4, cm), ref.muladd(a, a4, b4, cm))


@pytest.mark.skipif(not oracle.ref_samplers_available(), reason="reference sampler build absent")
@SETTINGS
@given(log_n=st.integers(3, 12), count=st.integers(1, 3), L=st.integers(1, 3),
       rho=st.integers(0, 255), hfrac=st.floats(0.0, 1.0), seed=st.integers(0, 2**40))
def test_samplers_equal_reference_on_drawn_shapes(orc, log_n, count, L, rho, hfrac, seed):
    """uniform, ZO(rho) and HWT(h) of the sampler oracle against the
    reference's own poly<N>::set(...) on the same counter stream, at drawn
    shapes, rho, Hamming weights (1 .. N) and seeds."""
    ref = oracle.RefSamplers()
    n = 1 << log_n
    h = max(1, min(n, int(round(hfrac * n))))
    assert np.array_equal(ref.sample_uniform(count, L, log_n, seed), orc.sample_uniform(count, L, log_n, seed=seed))
    assert np.array_equal(ref.sample_zo(count, L, log_n, rho, seed + 1),
                          orc.sample_zo(count, L, log_n, rho=rho, seed=seed + 1))
    assert np.array_equal(ref.sample_hwt(count, L, log_n, h, seed + 2),
                          orc.sample_hwt(count, L, log_n, h, seed=seed + 2))


@pytest.mark.skipif(not oracle.ref_samplers_available(), reason="reference sampler build absent")
@SETTINGS
@given(L=st.integers(1, 40), seed=st.integers(0, 2**40))
def test_crt_equals_reference_poly2mpz_on_drawn_residues(orc, L, seed):
    """oracle/crt.py against the reference's gmp::poly2mpz on residues of L
    moduli drawn from the counter stream, with 0, p - 1 and a small integer's
    residues planted."""
    from oracle.crt import CrtTable, poly2bigint, to_words

    log_n = 4
    n = 1 << log_n
    primes = [orc.prime(j) for j in range(L)]
    limbs = np.stack([splitmix64(seed + j, n) % np.uint64(p) for j, p in enumerate(primes)])
    limbs[:, 0] = 0
    limbs[:, 1] = [p - 1 for p in primes]  # Q - 1
    limbs[:, 2] = [12345 % p for p in primes]
    W = CrtTable(primes).words()
    want = oracle.RefSamplers().poly2mpz(limbs, log_n, W)
    got = poly2bigint(limbs, primes)
    assert np.array_equal(to_words(got, W), want)
    assert got[0] == 0 and got[2] == 12345
