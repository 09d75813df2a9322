"""Uneven batched polymul (one graph per batch shape) against the oracle and
against per-call GPU results."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import uniform_polys
from yell_gb300.workloads import mix_operands, uneven_mix

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


def _run_batch(torch, mix, ops, cm0s):
    items, outs = [], []
    for (log_n, L), (a, b), cm0 in zip(mix, ops, cm0s):
        c = torch.empty(a.size, dtype=torch.int64, device="cuda")
        items.append((c, _dev(torch, a), _dev(torch, b), log_n, L, cm0))
        outs.append(c)
    y.dev_polymul_batch(items)
    y.synchronize()
    return [o.cpu().numpy().view(np.uint64).reshape(ops[i][0].shape) for i, o in enumerate(outs)]


def test_small_uneven_batch_matches_oracle(cuda, orc):
    torch = cuda
    mix = [(3, 2), (10, 1), (13, 3), (14, 2), (17, 1), (10, 4), (16, 2), (3, 1), (12, 5), (15, 1)]
    cm0s = [i % 7 for i in range(len(mix))]
    ops = []
    for i, ((log_n, L), cm0) in enumerate(zip(mix, cm0s)):
        ps = y.primes(L, cm0)
        ops.append((uniform_polys(700 + i, 1, L, log_n, ps)[0], uniform_polys(800 + i, 1, L, log_n, ps)[0]))
    got = _run_batch(torch, mix, ops, cm0s)
    for (log_n, L), (a, b), cm0, g in zip(mix, ops, cm0s, got):
        assert np.array_equal(g, orc.polymul(a, b, log_n, cm0)), (log_n, L, cm0)


def test_graph_replay_with_new_data(cuda, orc):
    """Same batch shape twice (graph captured, then replayed) on different
    operands and buffers: both results are right."""
    torch = cuda
    mix = [(11, 2), (14, 3), (11, 1)]
    for rep in range(3):
        ops = []
        for i, (log_n, L) in enumerate(mix):
            ps = y.primes(L)
            ops.append((uniform_polys(900 + 10 * rep + i, 1, L, log_n, ps)[0],
                        uniform_polys(950 + 10 * rep + i, 1, L, log_n, ps)[0]))
        got = _run_batch(torch, mix, ops, [0] * len(mix))
        for (log_n, L), (a, b), g in zip(mix, ops, got):
            assert np.array_equal(g, orc.polymul(a, b, log_n, 0)), (rep, log_n, L)


def test_config4_uneven_512_matches_per_call(cuda, orc):
    """512 polymuls, log2 N uniform in 10..16, L uniform in 1..16 (seed 4):
    the batched graph equals 512 plain per-call launches word for word, and a
    sample of entries equals the oracle."""
    torch = cuda
    mix = uneven_mix(4, 512)
    ps = y.primes(16)
    ops = mix_operands(mix, ps, 4)
    got = _run_batch(torch, mix, ops, [0] * len(mix))
    for i, ((log_n, L), (a, b)) in enumerate(zip(mix, ops)):
        da, db = _dev(torch, a), _dev(torch, b)
        c = torch.empty(a.size, dtype=torch.int64, device="cuda")
        y.dev_polymul(c, da, db, 1, L, log_n, 0)
        torch.cuda.synchronize()
        assert np.array_equal(got[i], c.cpu().numpy().view(np.uint64).reshape(a.shape)), i
    for i in range(0, 512, 37):
        (log_n, L), (a, b) = mix[i], ops[i]
        assert np.array_equal(got[i], orc.polymul(a, b, log_n, 0)), i
