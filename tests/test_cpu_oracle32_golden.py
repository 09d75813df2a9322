"""32-bit moduli mode: the oracle's restatement (yell_oracle32.c) and the
library's host-side prime and twiddle tables against fixtures produced by the
reference's own sources compiled with -DYELL_USE_32BITS_MODULI
(tests/golden/make_golden32.py)."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from yell_gb300.inputs import splitmix64

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "yell_ref32_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def o32():
    return oracle.Oracle32("port")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def test_prime_table(o32, gold):
    for cm in range(291):
        assert o32.prime(cm) == int(gold["P"][cm])
        assert o32.pn(cm) == int(gold["Pn"][cm])
        assert o32.primitive_root(cm) == int(gold["roots"][cm])


def test_library_prime_table_and_tables(gold):
    """Host-side tables of the CUDA library (no device work)."""
    from yell_gb300 import moduli32 as m32

    assert m32.max_moduli() == 291 and m32.max_log_degree() == 15
    for cm in range(291):
        assert m32.prime(cm) == int(gold["P"][cm])
        assert m32.prime_pn(cm) == int(gold["Pn"][cm])
        assert m32.primitive_root(cm) == int(gold["roots"][cm])
    t, sc = m32.ntt_tables(4, 0)
    assert np.array_equal(t, gold["tables_4_0"]) and np.array_equal(sc, gold["tables_4_0_scalars"])
    for line in gold["digests"]:
        op, log_n, cm, *_rest, dig = str(line).split()
        if op == "tables":
            t, sc = m32.ntt_tables(int(log_n), int(cm))
            assert _digest(np.concatenate([t.ravel(), sc])) == dig


@pytest.mark.parametrize("log_n", [3, 4, 5, 8, 11])
@pytest.mark.parametrize("cm", [0, 290])
def test_small_ntt_vectors(o32, gold, log_n, cm):
    k = f"ntt_{log_n}_{cm}"
    assert np.array_equal(o32.forward_lazy(gold[k + "_x4"], log_n, cm), gold[k + "_fwd_lazy"])
    assert np.array_equal(o32.forward(gold[k + "_x4"], log_n, cm), gold[k + "_fwd"])
    assert np.array_equal(o32.backward(gold[k + "_x2"], log_n, cm), gold[k + "_bwd"])


def test_large_digests(o32, gold):
    for line in gold["digests"]:
        op, log_n, cm, seed, mult, dig = str(line).split()
        log_n, cm, seed, mult = int(log_n), int(cm), int(seed), int(mult)
        if op == "tables":
            t, sc = o32.tables(log_n, cm)
            got = _digest(np.concatenate([t.ravel(), sc]))
        else:
            p = o32.prime(cm)
            x = (splitmix64(seed, 1 << log_n) % np.uint64(mult * p)).astype(np.uint32)
            got = _digest(getattr(o32, op)(x, log_n, cm))
        assert got == dig, line


@pytest.mark.parametrize("cm", [0, 290])
def test_elementwise_and_barrett(o32, gold, cm):
    x, y, z, x4 = (gold[f"ew_{cm}_{k}"] for k in ("x", "y", "z", "x4"))
    assert np.array_equal(o32.mulmod(x, y, cm), gold[f"ew_{cm}_mulmod"])
    assert np.array_equal(o32.addmod(x, y, cm), gold[f"ew_{cm}_addmod"])
    assert np.array_equal(o32.submod(x, y, cm), gold[f"ew_{cm}_submod"])
    assert np.array_equal(o32.muladd(z, x4, x4, cm), gold[f"ew_{cm}_muladd"])
    p = o32.prime(cm)
    got = [o32.barrett(int(v) % (16 * p * p), cm) for v in gold[f"barrett_{cm}_x"]]
    assert np.array_equal(np.array(got, dtype=np.uint32), gold[f"barrett_{cm}"])


def test_polymul_vector(o32, gold):
    assert np.array_equal(o32.polymul(gold["pm_a"], gold["pm_b"], 12), gold["pm_c"])
    # the product is the negacyclic convolution of the residues
    n, p = 4096, o32.prime(0)
    a, b = gold["pm_a"][0][:n].astype(object), gold["pm_b"][0][:n].astype(object)
    c = gold["pm_c"][0]
    for k in (0, 1, 2047, 4095):
        s = sum(int(a[i]) * int(b[k - i]) for i in range(k + 1)) - sum(int(a[i]) * int(b[n + k - i]) for i in range(k + 1, n))
        assert s % p == int(c[k])


@pytest.mark.skipif(not oracle.ref32_available(), reason="reference 32-bit build not present")
def test_port_matches_reference_build(o32):
    ref = oracle.Oracle32("ref")
    for log_n in range(2, 16):
        for cm in (0, 57, 290):
            p = o32.prime(cm)
            x = (splitmix64(log_n * 1000 + cm, 1 << log_n) % np.uint64(4 * p)).astype(np.uint32)
            for op in ("forward", "forward_lazy"):
                assert np.array_equal(getattr(o32, op)(x, log_n, cm), getattr(ref, op)(x, log_n, cm))
            x2 = (x % np.uint32(2 * p)).astype(np.uint32)
            assert np.array_equal(o32.backward(x2, log_n, cm), ref.backward(x2, log_n, cm))
