"""GPU fused polymul against the oracle (reference-style forward, mulmod,
backward per limb) and the schoolbook negacyclic product in __int128."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300 import _capi
from yell_gb300.inputs import gaussian_polys, uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.uint64).reshape(shape)


def test_config1_plain_method(cuda, orc):
    """N=1024, L=1, q=P[0], one pair: bit-exact vs the reference-style path
    and the schoolbook product."""
    torch = cuda
    log_n = 10
    p = y.prime(0)
    a = uniform_polys(1, 1, 1, log_n, [p])
    b = uniform_polys(1, 1, 1, log_n, [p], offset=1 << log_n)
    c = torch.empty(1 << log_n, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), 1, 1, log_n, 0)
    torch.cuda.synchronize()
    got = _host(c, (1 << log_n,))
    assert np.array_equal(got, orc.schoolbook(a[0, 0], b[0, 0], log_n, 0))
    assert np.array_equal(got, orc.polymul(a[0], b[0], log_n, 0)[0])


@pytest.mark.parametrize("log_n", list(range(3, 21)))
def test_polymul_all_degrees(cuda, orc, log_n):
    torch = cuda
    pairs, L, cm0 = 2, 3, 1
    ps = y.primes(L, cm0)
    a = uniform_polys(10 + log_n, pairs, L, log_n, ps)
    b = uniform_polys(20 + log_n, pairs, L, log_n, ps)
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, cm0)
    torch.cuda.synchronize()
    got = _host(c, a.shape)
    for i in range(pairs):
        assert np.array_equal(got[i], orc.polymul(a[i], b[i], log_n, cm0)), i
    if log_n <= 11:
        assert np.array_equal(got[0, 0], orc.schoolbook(a[0, 0], b[0, 0], log_n, cm0))


def test_polymul_caller_scratch(cuda, orc):
    torch = cuda
    log_n, pairs, L = 15, 2, 2
    ps = y.primes(L)
    a = uniform_polys(31, pairs, L, log_n, ps)
    b = uniform_polys(32, pairs, L, log_n, ps)
    sw = y.polymul_scratch_words(pairs, L, log_n)
    assert sw == pairs * L << log_n
    scratch = torch.empty(sw, dtype=torch.int64, device="cuda")
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, 0, scratch=scratch)
    torch.cuda.synchronize()
    got = _host(c, a.shape)
    for i in range(pairs):
        assert np.array_equal(got[i], orc.polymul(a[i], b[i], log_n, 0))
    small = torch.empty(sw - 1, dtype=torch.int64, device="cuda")
    with pytest.raises(y.YellError):
        y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, 0, scratch=small)


def test_polymul_library_scratch_does_not_block(cuda, orc):
    """Without caller scratch the two-pass polymul takes its scratch
    stream-ordered from the library's pool: the call returns while the GPU is
    still busy with it (the stream has work left), and the result equals the
    caller-scratch path word for word."""
    torch = cuda
    log_n, pairs, L = 16, 8, 32
    ps = y.primes(L)
    a = uniform_polys(41, pairs, L, log_n, ps)
    b = uniform_polys(42, pairs, L, log_n, ps)
    da, db = _dev(torch, a), _dev(torch, b)
    want = torch.empty(a.size, dtype=torch.int64, device="cuda")
    scratch = torch.empty(y.polymul_scratch_words(pairs, L, log_n), dtype=torch.int64, device="cuda")
    stream = torch.cuda.Stream()
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    with torch.cuda.stream(stream):
        y.dev_polymul(want, da, db, pairs, L, log_n, 0, scratch=scratch, stream=stream.cuda_stream)
        y.dev_polymul(c, da, db, pairs, L, log_n, 0, stream=stream.cuda_stream)  # warm the pool
    stream.synchronize()
    allocs = y.allocations()
    with torch.cuda.stream(stream):
        for _ in range(4):  # several ms of work queued before the checked call
            y.dev_polymul(want, da, db, pairs, L, log_n, 0, scratch=scratch, stream=stream.cuda_stream)
        c.fill_(-1)
        y.dev_polymul(c, da, db, pairs, L, log_n, 0, stream=stream.cuda_stream)
        busy = not stream.query()
    stream.synchronize()
    assert busy, "yell_dev_polymul without scratch waited for the GPU"
    assert torch.equal(c, want)
    got = _host(c, a.shape)
    assert np.array_equal(got[0], orc.polymul(a[0], b[0], log_n, 0))


def test_config3_full_size(cuda, orc):
    """N=2^16, L=32 (P[0..31]), 16 pairs, A uniform, B centred discrete
    Gaussian (sigma 3.2, |e| <= 19) mapped per limb: every word of the fused
    GPU result equals the reference-style CPU result."""
    torch = cuda
    log_n, L, pairs = 16, 32, 16
    ps = y.primes(L)
    a = uniform_polys(3, pairs, L, log_n, ps)
    b = gaussian_polys(3, pairs, L, log_n, ps, offset=pairs * L << log_n)
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), pairs, L, log_n, 0)
    torch.cuda.synchronize()
    got = _host(c, a.shape)
    want, _ = orc.polymul_batch(a, b, pairs, L, log_n, threads=8)
    assert np.array_equal(got, want)


# chunking of pairs across the pipeline slots, with odd limb counts and a nonzero first modulus
@pytest.mark.parametrize("log_n,pairs,L,cm0", [(10, 3, 2, 0), (16, 3, 4, 0), (12, 2, 7, 5), (16, 5, 7, 11)])
def test_polymul_host_pipeline(cuda, orc, log_n, pairs, L, cm0):
    ps = y.primes(L, cm0)
    a = uniform_polys(40 + log_n, pairs, L, log_n, ps)
    b = uniform_polys(50 + log_n, pairs, L, log_n, ps)
    got = y.polymul_host(a, b, log_n, cm0=cm0)
    for i in range(pairs):
        assert np.array_equal(got[i], orc.polymul(a[i], b[i], log_n, cm0))


def test_polymul_host_pinned(cuda, orc):
    log_n, pairs, L = 14, 5, 3
    ps = y.primes(L)
    pa = y.PinnedBuffer((pairs, L, 1 << log_n))
    pb = y.PinnedBuffer((pairs, L, 1 << log_n))
    pc = y.PinnedBuffer((pairs, L, 1 << log_n))
    pa.array[:] = uniform_polys(61, pairs, L, log_n, ps)
    pb.array[:] = uniform_polys(62, pairs, L, log_n, ps)
    y.polymul_host(pa.array, pb.array, log_n, out=pc.array)
    for i in range(pairs):
        assert np.array_equal(pc.array[i], orc.polymul(pa.array[i], pb.array[i], log_n, 0))
    for buf in (pa, pb, pc):
        buf.free()


def test_polymul_every_modulus_in_one_call(cuda, orc):
    """All 1000 moduli of the table (params::kMaxNbModuli) as the limbs of one
    poly at N = 2^10; the last modulus index is 999."""
    torch = cuda
    log_n, L = 10, 1000
    ps = y.primes(L)
    a = uniform_polys(1000, 1, L, log_n, ps)
    b = uniform_polys(1001, 1, L, log_n, ps)
    c = torch.empty(a.size, dtype=torch.int64, device="cuda")
    y.dev_polymul(c, _dev(torch, a), _dev(torch, b), 1, L, log_n, 0)
    torch.cuda.synchronize()
    got = _host(c, a.shape)
    assert np.array_equal(got[0], orc.polymul(a[0], b[0], log_n, 0))


def test_modulus_range_boundaries(cuda, orc):
    torch = cuda
    log_n = 12
    # room for every limb the rejected calls name, so no call could write past it
    t = torch.zeros(1001 << log_n, dtype=torch.int64, device="cuda")
    y.dev_ntt(t[: 1 << log_n], 1, 1, log_n, 999, 0)  # the last modulus alone is fine
    for cm0, L in ((999, 2), (1000, 1), (0, 1001)):
        with pytest.raises(y.YellError) as ei:
            y.dev_ntt(t, 1, L, log_n, cm0, 0)
        assert ei.value.status == _capi.YELL_ERR_INVALID_MODULUS, (cm0, L)
