"""The oracle (C restatement of the reference) against fixtures produced by the
reference's own compiled sources (tests/golden/make_golden.py)."""
import hashlib
import os

import numpy as np
import pytest

from yell_gb300.inputs import splitmix64

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "yell_ref_vectors.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def test_prime_table(orc, gold):
    for cm in list(range(64)) + [500, 998, 999]:
        assert orc.prime(cm) == int(gold["P"][cm])
        assert orc.pn(cm) == int(gold["Pn"][cm])
        assert orc.primitive_root(cm) == int(gold["roots"][cm])


def test_config1_vectors(orc, gold):
    a, b = gold["cfg1_a"], gold["cfg1_b"]
    p0 = int(gold["P"][0])
    assert np.array_equal(a, splitmix64(1, 1024) % np.uint64(p0))
    assert np.array_equal(orc.forward(a, 10, 0), gold["cfg1_fwd_a"])
    assert np.array_equal(orc.forward(b, 10, 0), gold["cfg1_fwd_b"])
    assert np.array_equal(orc.forward_lazy(a, 10, 0), gold["cfg1_fwd_lazy_a"])
    assert np.array_equal(orc.mulmod(gold["cfg1_fwd_a"], gold["cfg1_fwd_b"], 0), gold["cfg1_prod"])
    assert np.array_equal(orc.backward(gold["cfg1_prod"], 10, 0), gold["cfg1_c"])
    # and the reference's polymul is the negacyclic product
    assert np.array_equal(orc.schoolbook(a, b, 10, 0), gold["cfg1_c"])


@pytest.mark.parametrize("log_n", [3, 4, 5, 8, 11])
@pytest.mark.parametrize("cm", [0, 999])
def test_small_ntt_vectors(orc, gold, log_n, cm):
    k = f"ntt_{log_n}_{cm}"
    assert np.array_equal(orc.forward_lazy(gold[k + "_x4"], log_n, cm), gold[k + "_fwd_lazy"])
    assert np.array_equal(orc.forward(gold[k + "_x4"], log_n, cm), gold[k + "_fwd"])
    assert np.array_equal(orc.backward(gold[k + "_x2"], log_n, cm), gold[k + "_bwd"])


def test_large_ntt_digests(orc, gold):
    for line in gold["digests"]:
        op, log_n, cm, seed, mult, dig = str(line).split()
        log_n, cm, seed, mult = int(log_n), int(cm), int(seed), int(mult)
        if op == "tables":
            t, sc = orc.tables(log_n, cm)
            got = _digest(np.concatenate([t.ravel(), sc]))
        else:
            p = orc.prime(cm)
            x = splitmix64(seed, 1 << log_n) % np.uint64(mult * p)
            got = _digest(getattr(orc, op)(x, log_n, cm))
        assert got == dig, line


def test_tables_small(orc, gold):
    t, sc = orc.tables(4, 0)
    assert np.array_equal(t, gold["tables_4_0"])
    assert np.array_equal(sc, gold["tables_4_0_scalars"])


@pytest.mark.parametrize("cm", [0, 999])
def test_elementwise_vectors(orc, gold, cm):
    x, y, z = gold[f"ew_{cm}_x"], gold[f"ew_{cm}_y"], gold[f"ew_{cm}_z"]
    assert np.array_equal(orc.mulmod(x, y, cm), gold[f"ew_{cm}_mulmod"])
    assert np.array_equal(orc.addmod(x, y, cm), gold[f"ew_{cm}_addmod"])
    assert np.array_equal(orc.submod(x, y, cm), gold[f"ew_{cm}_submod"])
    assert np.array_equal(orc.muladd(z, x, y, cm), gold[f"ew_{cm}_muladd"])
    yy = int(y[0]) % int(gold["P"][cm])
    assert np.array_equal(orc.mulmod_shoup(x, yy, cm), gold[f"ew_{cm}_mulmod_shoup"])


def test_reference_quirk_at_degree_4(orc):
    """The reference's inverse at N = 4 is not an inverse (its second GS loop
    already is the last layer, lib/ntt.cpp:174-187, and backward applies it
    again); the oracle reproduces that, which is why the library rejects 4."""
    p = orc.prime(0)
    x = splitmix64(9, 4) % np.uint64(p)
    assert not np.array_equal(orc.backward(orc.forward(x, 2, 0), 2, 0), x)
    y = splitmix64(9, 8) % np.uint64(p)
    assert np.array_equal(orc.backward(orc.forward(y, 3, 0), 3, 0), y)


def test_schoolbook_is_independent(orc):
    """Schoolbook negacyclic product: X * X^(N-1) = X^N = -1."""
    n = 1 << 6
    p = orc.prime(3)
    a = np.zeros(n, np.uint64)
    b = np.zeros(n, np.uint64)
    a[1] = 1
    b[n - 1] = 1
    c = orc.schoolbook(a, b, 6, 3)
    want = np.zeros(n, np.uint64)
    want[0] = p - 1
    assert np.array_equal(c, want)


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference build not present")
def test_port_matches_reference_build(orc):
    import oracle

    ref = oracle.Oracle("ref")
    for log_n in (6, 12, 14, 16):
        for cm in (0, 17):
            p = orc.prime(cm)
            x = splitmix64(log_n * 31 + cm, 1 << log_n) % np.uint64(4 * p)
            assert np.array_equal(orc.forward_lazy(x, log_n, cm), ref.forward_lazy(x, log_n, cm))
            assert np.array_equal(orc.forward(x, log_n, cm), ref.forward(x, log_n, cm))
            y = x % np.uint64(2 * p)
            assert np.array_equal(orc.backward(y, log_n, cm), ref.backward(y, log_n, cm))


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference build not present")
def test_free_functions_match_reference_build(orc):
    """negacylic_forward_lazy / backward_lazy with caller tables: the port
    against the reference's own compiled functions."""
    import oracle

    ref = oracle.Oracle("ref")
    for log_n in (2, 3, 5, 8, 12, 15):
        for cm in (0, 999):
            p = orc.prime(cm)
            t, _ = orc.tables(log_n, cm)
            n = 1 << log_n
            x4 = splitmix64(60 + log_n + cm, n) % np.uint64(4 * p)
            x2 = splitmix64(70 + log_n + cm, n) % np.uint64(2 * p)
            assert np.array_equal(orc.negacyclic_lazy(x4, t[0], t[1], p), ref.negacyclic_lazy(x4, t[0], t[1], p))
            assert np.array_equal(orc.negacyclic_lazy(x2, t[2], t[3], p, True),
                                  ref.negacyclic_lazy(x2, t[2], t[3], p, True))
