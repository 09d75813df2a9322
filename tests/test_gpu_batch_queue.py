"""The uneven batch as ONE launch of the persistent work-queue kernel, and the
same work items as three phase launches: results against the oracle and
against the graph-bucketed batch, repeated launches (counters reset), and the
bounded dependency wait (a queue whose waits cannot be satisfied records
YELL_ERR_TIMEOUT instead of hanging)."""
import time

import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300._capi import YELL_ERR_TIMEOUT
from yell_gb300.inputs import uniform_polys
from yell_gb300.workloads import mix_operands, uneven_mix

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


def _run(torch, mix, ops, cm0s, fn):
    items, outs = [], []
    for (log_n, L), (a, b), cm0 in zip(mix, ops, cm0s):
        c = torch.empty(a.size, dtype=torch.int64, device="cuda")
        items.append((c, _dev(torch, a), _dev(torch, b), log_n, L, cm0))
        outs.append(c)
    fn(items)
    y.synchronize()
    return [o.cpu().numpy().view(np.uint64).reshape(ops[i][0].shape) for i, o in enumerate(outs)]


def test_every_degree_matches_oracle(cuda, orc):
    mix = [(d, 1 + d % 3) for d in range(3, 21)] + [(13, 4), (10, 2), (16, 1), (3, 5)]
    cm0s = [i % 5 for i in range(len(mix))]
    ops = []
    for i, ((log_n, L), cm0) in enumerate(zip(mix, cm0s)):
        ps = y.primes(L, cm0)
        ops.append((uniform_polys(1700 + i, 1, L, log_n, ps)[0], uniform_polys(1800 + i, 1, L, log_n, ps)[0]))
    got = _run(cuda, mix, ops, cm0s, y.dev_polymul_batch_queue)
    assert y.batch_queue_status() == 0
    for (log_n, L), (a, b), cm0, g in zip(mix, ops, cm0s, got):
        assert np.array_equal(g, orc.polymul(a, b, log_n, cm0)), (log_n, L, cm0)


def test_config4_queue_equals_graph_batch(cuda, orc):
    """512 polymuls (log2 N uniform in 10..16, L in 1..16, seed 4): the one-launch
    queue equals the graph-bucketed batch word for word, twice in a row."""
    mix = uneven_mix(4, 512)
    ops = mix_operands(mix, y.primes(16), 4)
    want = _run(cuda, mix, ops, [0] * len(mix), y.dev_polymul_batch)
    for rep in range(2):
        got = _run(cuda, mix, ops, [0] * len(mix), y.dev_polymul_batch_queue)
        assert y.batch_queue_status() == 0
        for i in range(len(mix)):
            assert np.array_equal(got[i], want[i]), (rep, i)
    for i in range(0, 512, 41):
        (log_n, L), (a, b) = mix[i], ops[i]
        assert np.array_equal(want[i], orc.polymul(a, b, log_n, 0)), i


def test_phased_every_degree_matches_oracle(cuda, orc):
    """The queue's items as three phase launches: every degree 2^3..2^20, mixed
    limb counts and moduli, word for word against the oracle."""
    mix = [(d, 1 + d % 3) for d in range(3, 21)] + [(13, 4), (10, 2), (16, 1), (3, 5)]
    cm0s = [(i + 2) % 5 for i in range(len(mix))]
    ops = []
    for i, ((log_n, L), cm0) in enumerate(zip(mix, cm0s)):
        ps = y.primes(L, cm0)
        ops.append((uniform_polys(3700 + i, 1, L, log_n, ps)[0], uniform_polys(3800 + i, 1, L, log_n, ps)[0]))
    got = _run(cuda, mix, ops, cm0s, y.dev_polymul_batch_phased)
    for (log_n, L), (a, b), cm0, g in zip(mix, ops, cm0s, got):
        assert np.array_equal(g, orc.polymul(a, b, log_n, cm0)), (log_n, L, cm0)


def test_config4_phased_equals_graph_batch(cuda):
    mix = uneven_mix(4, 512)
    ops = mix_operands(mix, y.primes(16), 4)
    want = _run(cuda, mix, ops, [0] * len(mix), y.dev_polymul_batch)
    for rep in range(2):
        got = _run(cuda, mix, ops, [0] * len(mix), y.dev_polymul_batch_phased)
        for i in range(len(mix)):
            assert np.array_equal(got[i], want[i]), (rep, i)


def test_bounded_wait_records_timeout(cuda, orc):
    t0 = time.perf_counter()
    st = y.batch_queue_wait_check(0.02)
    assert st == YELL_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 10
    assert y.batch_queue_status() == 0  # read and cleared
    # the queue still works afterwards
    mix = [(14, 2), (11, 1)]
    ops = []
    for i, (log_n, L) in enumerate(mix):
        ps = y.primes(L)
        ops.append((uniform_polys(2900 + i, 1, L, log_n, ps)[0], uniform_polys(2950 + i, 1, L, log_n, ps)[0]))
    got = _run(cuda, mix, ops, [0, 0], y.dev_polymul_batch_queue)
    assert y.batch_queue_status() == 0
    for (log_n, L), (a, b), g in zip(mix, ops, got):
        assert np.array_equal(g, orc.polymul(a, b, log_n, 0))


def test_queue_errors(cuda):
    t = cuda.zeros(1 << 10, dtype=cuda.int64, device="cuda")
    with pytest.raises(y.YellError):
        y.dev_polymul_batch_queue([(t, t, t, 10, 1, 0)])  # output aliases operands
    with pytest.raises(y.YellError):
        y.dev_polymul_batch_phased([(t, t, t, 10, 1, 0)])
    with pytest.raises(y.YellError):
        y.batch_queue_wait_check(0.0)
