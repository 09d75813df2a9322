"""Every launch variant of every degree (the autotuner's search space) gives
the same words as the oracle, and the autotuner selects one of them."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import splitmix64, uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


@pytest.mark.parametrize("log_n", list(range(3, 21)))
def test_all_variants_match_oracle(cuda, orc, log_n):
    torch = cuda
    names = y.variants(log_n)
    assert names
    L, cm0, pairs = 2, 4, 2
    ps = y.primes(L, cm0)
    x = uniform_polys(1300 + log_n, 1, L, log_n, ps)[0]
    x4 = (splitmix64(1400 + log_n, L << log_n).reshape(L, -1) % (4 * ps.reshape(L, 1)))
    a = uniform_polys(1500 + log_n, pairs, L, log_n, ps)
    b = uniform_polys(1600 + log_n, pairs, L, log_n, ps)
    want_f = [orc.forward(x4[l], log_n, cm0 + l) for l in range(L)]
    want_l = [orc.forward_lazy(x4[l], log_n, cm0 + l) for l in range(L)]
    want_b = [orc.backward(x[l] % ps[l], log_n, cm0 + l) for l in range(L)]
    want_p = [orc.polymul(a[i], b[i], log_n, cm0) for i in range(pairs)]
    try:
        for v, name in enumerate(names):
            y.set_variant(log_n, v)
            assert y.get_variant(log_n) == v
            for direction, want, src in ((0, want_f, x4), (1, want_l, x4), (2, want_b, x)):
                t = _dev(torch, src)
                y.dev_ntt(t, 1, L, log_n, cm0, direction)
                torch.cuda.synchronize()
                got = t.cpu().numpy().view(np.uint64).reshape(L, -1)
                for l in range(L):
                    assert np.array_equal(got[l], want[l]), (name, direction, l)
            c = torch.empty(a.size, dtype=torch.int64, device="cuda")
            y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, cm0)
            torch.cuda.synchronize()
            got = c.cpu().numpy().view(np.uint64).reshape(a.shape)
            for i in range(pairs):
                assert np.array_equal(got[i], want_p[i]), (name, "polymul", i)
    finally:
        y.set_variant(log_n, 0)


def test_autotune_selects_a_variant_and_stays_exact(cuda, orc, tmp_path, monkeypatch):
    torch = cuda
    log_n, L, pairs = 16, 4, 2
    best, ms = y.autotune(log_n, L, pairs)
    assert 0 <= best < len(y.variants(log_n)) and ms > 0
    assert y.get_variant(log_n) == best
    ps = y.primes(L)
    a = uniform_polys(1700, pairs, L, log_n, ps)
    b = uniform_polys(1701, pairs, L, log_n, ps)
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, 0)
    torch.cuda.synchronize()
    got = c.cpu().numpy().view(np.uint64).reshape(a.shape)
    assert np.array_equal(got[1], orc.polymul(a[1], b[1], log_n, 0))
    y.set_variant(log_n, 0)


@pytest.mark.parametrize("log_n", [16])
def test_pipelined_variants_over_many_tiles(cuda, orc, log_n):
    """The pipelined polymul kernels are persistent: with 48 limbs (768 tiles
    of 4096 words, above the resident CTAs of every pass) each CTA runs
    several tiles, and every copy-ahead overlaps the previous tile."""
    torch = cuda
    names = y.variants(log_n)
    pipe = [v for v, n in enumerate(names) if "pipelined" in n]
    assert pipe, names
    L, cm0, pairs = 4, 2, 12
    ps = y.primes(L, cm0)
    a = uniform_polys(1800 + log_n, pairs, L, log_n, ps)
    b = uniform_polys(1900 + log_n, pairs, L, log_n, ps)
    want = [orc.polymul(a[i], b[i], log_n, cm0) for i in range(pairs)]
    try:
        for v in pipe:
            y.set_variant(log_n, v)
            c = torch.empty(a.size, dtype=torch.int64, device="cuda")
            y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, cm0)
            torch.cuda.synchronize()
            got = c.cpu().numpy().view(np.uint64).reshape(a.shape)
            for i in range(pairs):
                assert np.array_equal(got[i], want[i]), (names[v], i)
    finally:
        y.set_variant(log_n, 0)
