"""GPU RNS -> big-integer lifting (gmp::poly2mpz, include/yell/gmp.hpp:42-70)
against the big-integer oracle, word for word, plus CRT properties at full
size and the cases that take the kernel's quotient-correction path."""
import numpy as np
import pytest

import yell_gb300 as y
from oracle.crt import CrtTable, poly2bigint, to_words
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).reshape(-1).copy()).cuda()


def _lift(torch, polys, count, L, log_n, cm0=0):
    W = y.crt_words(L, cm0)
    out = torch.zeros(count * (W << log_n), dtype=torch.int64, device="cuda")
    y.dev_crt_lift(out, _dev(torch, polys), count, L, log_n, cm0)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint64).reshape(count, 1 << log_n, W)


@pytest.mark.parametrize("L,log_n,cm0,count", [(1, 3, 0, 1), (2, 4, 0, 2), (3, 10, 0, 1), (8, 12, 0, 1),
                                               (32, 8, 0, 2), (5, 9, 123, 1), (64, 5, 900, 1)])
def test_lift_matches_oracle(cuda, orc, L, log_n, cm0, count):
    ps = [orc.prime(cm0 + j) for j in range(L)]
    polys = uniform_polys(L * 31 + log_n, count, L, log_n, ps)
    got = _lift(cuda, polys, count, L, log_n, cm0)
    W = CrtTable(ps).words()
    for i in range(count):
        want = to_words(poly2bigint(polys[i], ps), W)
        assert np.array_equal(got[i], want), (L, log_n, i)


def test_lift_edge_values(cuda, orc):
    """Zero, small integers (the quotient estimate falls one short for these,
    so the correction path runs), Q - 1 and Q - k, at L = 7 and L = 40."""
    for L in (7, 40):
        ps = [orc.prime(j) for j in range(L)]
        t = CrtTable(ps)
        xs = [0, 1, 2, 3, 1 << 64, 1 << 100] + list(range(5, 59)) + [t.Q - 1, t.Q - 2, t.Q - 12345, t.Q // 2]
        xs += [0] * (64 - len(xs))
        polys = np.array([[x % p for x in xs] for p in ps], dtype=np.uint64)[None]
        got = _lift(cuda, polys, 1, L, 6)
        assert y.words_to_ints(got) == xs


def test_lift_full_size_properties(cuda, orc):
    """N = 2^16, L = 32, 4 polys: every coefficient below Q and, on a sample,
    congruent to its residues (the CRT fixes the value uniquely)."""
    count, L, log_n = 4, 32, 16
    ps = [orc.prime(j) for j in range(L)]
    polys = uniform_polys(5, count, L, log_n, ps)
    got = _lift(cuda, polys, count, L, log_n)
    Q = CrtTable(ps).Q
    rng = np.random.default_rng(0)
    for i in rng.integers(0, count << log_n, 400):
        poly, c = divmod(int(i), 1 << log_n)
        x = y.words_to_ints(got[poly, c][None])[0]
        assert x < Q
        assert all(x % ps[j] == int(polys[poly, j, c]) for j in range(L))


def test_host_poly_to_bigint(cuda, orc):
    L, log_n = 4, 11
    ps = [orc.prime(j) for j in range(L)]
    limbs = [np.ascontiguousarray(l) for l in uniform_polys(77, 1, L, log_n, ps)[0]]
    got = y.poly_to_bigint(limbs)
    assert y.words_to_ints(got) == poly2bigint(np.stack(limbs), ps)


def test_lift_after_polymul(cuda, orc):
    """Lifting a GPU polymul of small-integer polys gives the integer negacyclic
    product (coefficients mapped to [0, Q))."""
    L, log_n = 4, 9
    n = 1 << log_n
    ps = [orc.prime(j) for j in range(L)]
    rng = np.random.default_rng(3)
    ia = rng.integers(-1000, 1000, n)
    ib = rng.integers(-1000, 1000, n)
    a = np.array([[int(v) % p for v in ia] for p in ps], dtype=np.uint64)[None]
    b = np.array([[int(v) % p for v in ib] for p in ps], dtype=np.uint64)[None]
    da, db = _dev(cuda, a), _dev(cuda, b)
    dc = cuda.zeros_like(da)
    y.dev_polymul(dc, da, db, 1, L, log_n)
    cuda.cuda.synchronize()
    got = _lift(cuda, dc.cpu().numpy().view(np.uint64).reshape(1, L, n), 1, L, log_n)
    Q = CrtTable(ps).Q
    want = [0] * n
    for i in range(n):
        for j in range(n):
            k = i + j
            v = int(ia[i]) * int(ib[j])
            if k >= n:
                want[k - n] -= v
            else:
                want[k] += v
    assert y.words_to_ints(got[0]) == [w % Q for w in want]


def test_crt_errors(cuda):
    t = cuda.zeros(64, dtype=cuda.int64, device="cuda")
    with pytest.raises(y.YellError):
        y.dev_crt_lift(t, t, 1, 401, 3)
    with pytest.raises(y.YellError):
        y.dev_crt_lift(t, t, 1, 2, 2)
    with pytest.raises(y.YellError):
        y.dev_crt_lift(t, t, 1, 2, 3, cm0=999)
