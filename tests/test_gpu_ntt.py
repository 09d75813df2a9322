"""GPU parity of the NTT entry points against the CPU oracle (word for word).

The oracle restates the reference's lib/ntt.cpp and details/ntt.hpp and is
itself pinned against the reference build and tests/golden fixtures.
Bit-exact equality is required for every output, including forward_lazy,
whose [0, 4p) words are a public result (include/yell/ntt.hpp:60-62).
"""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import splitmix64, uniform_polys

pytestmark = pytest.mark.gpu

ALL_LOG_N = list(range(3, 21))  # the reference's degrees 2^3 .. kMaxPolyDegree = 2^20


def _uniform(seed, log_n, cm, scale=1):
    p = y.prime(cm)
    raw = splitmix64(seed, 1 << log_n)
    return raw % np.uint64(p * scale) if p * scale < 2**64 else raw


@pytest.mark.parametrize("log_n", ALL_LOG_N)
@pytest.mark.parametrize("cm", [0, 1, 999])
def test_forward_per_limb(cuda, orc, log_n, cm):
    x = _uniform(100 + log_n, log_n, cm)
    assert np.array_equal(y.ntt_forward(x, log_n, cm), orc.forward(x, log_n, cm))


@pytest.mark.parametrize("log_n", ALL_LOG_N)
@pytest.mark.parametrize("cm", [0, 7])
def test_forward_lazy_words_match(cuda, orc, log_n, cm):
    # lazy inputs anywhere in [0, 4p), the CT butterfly's contract (lib/ntt.cpp:65-68)
    x = _uniform(200 + log_n, log_n, cm, scale=4)
    got = y.ntt_forward_lazy(x, log_n, cm)
    want = orc.forward_lazy(x, log_n, cm)
    assert np.array_equal(got, want)
    assert int(got.max()) < 4 * y.prime(cm)


@pytest.mark.parametrize("log_n", ALL_LOG_N)
@pytest.mark.parametrize("cm", [0, 31])
def test_backward_per_limb(cuda, orc, log_n, cm):
    # inverse inputs in [0, 2p) (lib/ntt.cpp:43-46)
    x = _uniform(300 + log_n, log_n, cm, scale=2)
    got = y.ntt_backward(x, log_n, cm)
    assert np.array_equal(got, orc.backward(x, log_n, cm))
    assert int(got.max()) < y.prime(cm)


@pytest.mark.parametrize("log_n", [3, 8, 13, 14, 16, 17, 18, 20])
def test_round_trip_identity(cuda, log_n):
    x = _uniform(400 + log_n, log_n, 3)
    f = y.ntt_forward(x, log_n, 3)
    assert np.array_equal(y.ntt_backward(f, log_n, 3), x)
    fl = y.ntt_forward_lazy(x, log_n, 3)
    assert np.array_equal(y.ntt_backward(fl % np.uint64(y.prime(3)), log_n, 3), x)


@pytest.mark.parametrize("log_n", [4, 10, 15])
def test_edge_values(cuda, orc, log_n):
    cm = 0
    p = y.prime(cm)
    n = 1 << log_n
    for x in (np.zeros(n, np.uint64), np.full(n, p - 1, np.uint64),
              np.full(n, 4 * p - 1, np.uint64)):
        assert np.array_equal(y.ntt_forward_lazy(x, log_n, cm), orc.forward_lazy(x, log_n, cm))
        assert np.array_equal(y.ntt_forward(x, log_n, cm), orc.forward(x, log_n, cm))
    for x in (np.zeros(n, np.uint64), np.full(n, 2 * p - 1, np.uint64)):
        assert np.array_equal(y.ntt_backward(x, log_n, cm), orc.backward(x, log_n, cm))


def test_unsupported_degree_is_an_error(cuda):
    for log_n in (0, 1, 2, 21):
        with pytest.raises(y.YellError) as ei:
            y.ntt_forward(np.zeros(1 << log_n, np.uint64), log_n, 0)
        assert ei.value.status == 2


@pytest.mark.parametrize("log_n,count,L", [(3, 5, 3), (10, 3, 4), (12, 2, 3), (13, 3, 2),
                                           (14, 2, 3), (16, 2, 2), (17, 1, 2), (19, 1, 2), (20, 2, 1)])
@pytest.mark.parametrize("direction", [0, 1, 2])
def test_device_batch(cuda, orc, log_n, count, L, direction):
    torch = cuda
    cm0 = 2
    ps = y.primes(L, cm0)
    x = uniform_polys(500 + log_n, count, L, log_n, ps)
    t = torch.from_numpy(x.view(np.int64).copy()).cuda()
    y.dev_ntt(t, count, L, log_n, cm0, direction)
    torch.cuda.synchronize()
    got = t.cpu().numpy().view(np.uint64).reshape(count, L, -1)
    f = {0: orc.forward, 1: orc.forward_lazy, 2: orc.backward}[direction]
    for i in range(count):
        for l in range(L):
            assert np.array_equal(got[i, l], f(x[i, l], log_n, cm0 + l)), (i, l)


@pytest.mark.parametrize("log_n", [10, 14])
def test_device_limb_pointer_list(cuda, orc, log_n):
    torch = cuda
    n = 1 << log_n
    cms = [5, 0, 999, 5]
    bufs = [torch.from_numpy(_uniform(600 + i, log_n, cm).view(np.int64).copy()).cuda()
            for i, cm in enumerate(cms)]
    want = [orc.forward(b.cpu().numpy().view(np.uint64), log_n, cm) for b, cm in zip(bufs, cms)]
    ptrs = torch.tensor([b.data_ptr() for b in bufs], dtype=torch.int64, device="cuda")
    cmt = torch.tensor(cms, dtype=torch.int32, device="cuda")
    y.dev_ntt_limbs(ptrs, cmt, log_n, 0)
    torch.cuda.synchronize()
    for b, w in zip(bufs, want):
        assert np.array_equal(b.cpu().numpy().view(np.uint64), w)
    assert n == bufs[0].numel()


def test_config2_forward_inverse_full_size(cuda, orc):
    """N=2^14, L=8 (P[0..7]), batch 64, one call each way over all 512 limbs
    (a column-pass and a row-pass launch): forward words equal the
    reference's, and the inverse returns the input exactly."""
    torch = cuda
    log_n, L, count = 14, 8, 64
    x = uniform_polys(2, count, L, log_n, y.primes(L))
    t = torch.from_numpy(x.view(np.int64).copy()).cuda()
    y.dev_ntt(t, count, L, log_n, 0, 0)
    torch.cuda.synchronize()
    f = t.cpu().numpy().view(np.uint64).reshape(count, L, -1)
    for i in range(count):
        for l in range(L):
            assert np.array_equal(f[i, l], orc.forward(x[i, l], log_n, l)), (i, l)
    y.dev_ntt(t, count, L, log_n, 0, 2)
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy().view(np.uint64).reshape(count, L, -1), x)
