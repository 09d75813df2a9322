"""Two-pass kernels launched as programmatic dependents of the stream's
previous kernel: their CTAs may become resident while that kernel's last
CTAs run, and each waits for it (griddepcontrol.wait) before it reads or
writes global memory.  Checked word for word against the oracle where the
previous kernel is a foreign one that writes the polymul's operand just
before it, where polymuls and NTTs follow one another on one stream with
each consuming the last one's output, and on a caller's own stream."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.uint64).reshape(shape)


@pytest.mark.parametrize("log_n", [14, 16])
def test_operand_written_by_the_kernel_just_before(cuda, orc, log_n):
    """Each round: a torch kernel overwrites the operand with garbage, a second
    torch kernel writes the real operand, and the polymul follows at once on
    the same stream; its words must be those of the real operand."""
    torch = cuda
    pairs, L = 2, 4
    ps = y.primes(L)
    a = uniform_polys(41, pairs, L, log_n, ps)
    b = uniform_polys(42, pairs, L, log_n, ps)
    src, db = _dev(torch, a), _dev(torch, b)
    da = torch.empty_like(src)
    c = torch.empty_like(src)
    want = np.stack([orc.polymul(a[i], b[i], log_n, 0) for i in range(pairs)])
    for _ in range(4):
        da.fill_(-1)
        torch.add(src, 0, out=da)
        y.dev_polymul(c, da, db, pairs, L, log_n, 0)
        torch.cuda.synchronize()
        assert np.array_equal(_host(c, a.shape), want)


def test_chain_of_calls_on_one_stream(cuda, orc):
    """polymul -> polymul -> forward NTT -> backward NTT, back to back on a
    caller's stream, each reading what the one before wrote."""
    torch = cuda
    log_n, pairs, L = 16, 2, 3
    ps = y.primes(L)
    a = uniform_polys(51, pairs, L, log_n, ps)
    b = uniform_polys(52, pairs, L, log_n, ps)
    da, db = _dev(torch, a), _dev(torch, b)
    c1, c2 = torch.empty_like(da), torch.empty_like(da)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        y.dev_polymul(c1, da, db, pairs, L, log_n, 0, stream=s)
        y.dev_polymul(c2, c1, db, pairs, L, log_n, 0, stream=s)
        f = c2.clone()
        y.dev_ntt(f, pairs, L, log_n, 0, 0, stream=s)
        r = f.clone()
        y.dev_ntt(r, pairs, L, log_n, 0, 2, stream=s)
    s.synchronize()
    w1 = np.stack([orc.polymul(a[i], b[i], log_n, 0) for i in range(pairs)])
    w2 = np.stack([orc.polymul(w1[i], b[i], log_n, 0) for i in range(pairs)])
    assert np.array_equal(_host(c1, a.shape), w1)
    assert np.array_equal(_host(c2, a.shape), w2)
    got_f = _host(f, a.shape)
    for i in range(pairs):
        assert np.array_equal(got_f[i], orc.poly_forward(w2[i], log_n, 0)), i
    assert np.array_equal(_host(r, a.shape), w2)


def test_captured_into_a_caller_graph(cuda, orc):
    """A caller captures the polymul (caller scratch, tables built before) into
    its own CUDA graph: the dependent launches become programmatic edges of
    the graph, and replays on new operands give the oracle's words."""
    torch = cuda
    log_n, pairs, L = 16, 2, 2
    ps = y.primes(L)
    y.init_ntt_tables(log_n, L, 0)
    a = uniform_polys(61, pairs, L, log_n, ps)
    b = uniform_polys(62, pairs, L, log_n, ps)
    da, db = _dev(torch, a), _dev(torch, b)
    c = torch.empty_like(da)
    scratch = torch.empty(y.polymul_scratch_words(pairs, L, log_n), dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # one eager call first, as torch asks before a capture
        y.dev_polymul(c, da, db, pairs, L, log_n, 0, scratch=scratch, stream=s)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        y.dev_polymul(c, da, db, pairs, L, log_n, 0, scratch=scratch,
                      stream=torch.cuda.current_stream())
    for seed in (63, 64):
        a2 = uniform_polys(seed, pairs, L, log_n, ps)
        da.copy_(_dev(torch, a2))
        c.zero_()
        g.replay()
        torch.cuda.synchronize()
        want = np.stack([orc.polymul(a2[i], b[i], log_n, 0) for i in range(pairs)])
        assert np.array_equal(_host(c, a.shape), want), seed


@pytest.mark.parametrize("log_n,h", [(10, 64), (16, 192)])
def test_samplers_after_a_foreign_write(cuda, orc, log_n, h):
    """A torch kernel fills the output with all-ones words just before each
    sampler call on the same stream: the HWT sample (zero fill beside the
    draws, then the chosen words) and the ZO sample equal the oracle's."""
    torch = cuda
    count, L = 3, 2
    t = torch.empty((count * L) << log_n, dtype=torch.int64, device="cuda")
    for _ in range(2):
        t.fill_(-1)
        y.sample_hwt(t, count, L, log_n, h, cm0=1, seed=h + 7)
        torch.cuda.synchronize()
        got = _host(t, (count, L, 1 << log_n))
        assert np.array_equal(got, orc.sample_hwt(count, L, log_n, h, 1, h + 7))
        t.fill_(-1)
        y.sample_zo(t, count, L, log_n, 1, rho=0x7F, seed=h + 8)
        torch.cuda.synchronize()
        assert np.array_equal(_host(t, (count, L, 1 << log_n)), orc.sample_zo(count, L, log_n, 1, 0x7F, h + 8))
