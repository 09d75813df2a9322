"""Serving loop: continuous batching, HBM-budget admission, failure handling.

A request's result is the same alone and in a concurrent mix of other
requests (and equals the oracle); failures are per-request status codes made
on the host (budget overflow, invalid sizes, cancellation, a wait that runs
out, an injected allocation refusal) - no GPU fault is involved."""
import threading

import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300 import _capi
from yell_gb300.inputs import uniform_polys
from yell_gb300.serve import Server
from yell_gb300.workloads import uneven_mix

pytestmark = pytest.mark.gpu


def _operands(seed, log_n, L, cm0=0):
    ps = y.primes(L, cm0)
    return uniform_polys(seed, 1, L, log_n, ps)[0], uniform_polys(seed + 1, 1, L, log_n, ps)[0]


def test_result_same_alone_and_in_mix(cuda, orc):
    with Server(hbm_budget_bytes=2 << 30, max_inflight=4) as srv:
        a, b = _operands(11, 14, 3)
        c_alone = np.zeros_like(a)
        rid = srv.submit(a, b, c_alone, 14, 3)
        assert srv.wait(rid)["status"] == 0
        assert np.array_equal(c_alone, orc.polymul(a, b, 14, 0))
        # the same request in the middle of a mix of 60 others of mixed size
        mix = uneven_mix(5, 60, lo=8, hi=15, max_L=4)
        jobs = []
        for i, (log_n, L) in enumerate(mix):
            x, z = _operands(100 + 2 * i, log_n, L)
            out = np.zeros_like(x)
            jobs.append((srv.submit(x, z, out, log_n, L), x, z, out, log_n))
            if i == 30:
                c_mix = np.zeros_like(a)
                rid_mix = srv.submit(a, b, c_mix, 14, 3)
        for rid_i, x, z, out, log_n in jobs:
            assert srv.wait(rid_i)["status"] == 0
        assert srv.wait(rid_mix)["status"] == 0
        assert np.array_equal(c_mix, c_alone)
        for rid_i, x, z, out, log_n in jobs[::7]:
            assert np.array_equal(out, orc.polymul(x, z, log_n, 0))
        st = srv.stats()
        assert st["completed"] == 62 and st["failed"] == 0
        assert st["batches"] >= 2  # requests were coalesced and overlapped, not one per batch


def test_budget_admission_and_overflow(cuda, orc):
    log_n, L = 14, 4
    words = L << log_n
    fp = 4 * words * 8  # a, b, c, scratch
    with Server(hbm_budget_bytes=2 * fp + 4096, max_inflight=4) as srv:
        ids = []
        for i in range(8):
            a, b = _operands(300 + 2 * i, log_n, L)
            c = np.zeros_like(a)
            ids.append((srv.submit(a, b, c, log_n, L), a, b, c))
        for rid, a, b, c in ids:
            assert srv.wait(rid)["status"] == 0
            assert np.array_equal(c, orc.polymul(a, b, log_n, 0))
        st = srv.stats()
        assert st["hbm_peak"] <= st["hbm_budget"]
        assert st["hbm_in_use"] == 0
        # a request that can never fit is refused at submit time
        a, b = _operands(400, 16, 8)
        with pytest.raises(y.YellError) as ei:
            srv.submit(a, b, np.zeros_like(a), 16, 8)
        assert ei.value.status == _capi.YELL_ERR_BUDGET


def test_invalid_sizes_rejected(cuda):
    with Server(hbm_budget_bytes=64 << 20) as srv:
        a = np.zeros(16, np.uint64)
        with pytest.raises(y.YellError) as ei:
            srv.submit(a, a, a.copy(), 2, 1)
        assert ei.value.status == _capi.YELL_ERR_UNSUPPORTED_DEGREE
        with pytest.raises(y.YellError) as ei:
            srv.submit(a, a, a.copy(), 4, 2, cm0=999)
        assert ei.value.status == _capi.YELL_ERR_INVALID_MODULUS


def test_cancel_and_bounded_wait(cuda, orc):
    with Server(hbm_budget_bytes=256 << 20) as srv:
        srv.pause(True)
        reqs = []
        for i in range(3):
            a, b = _operands(500 + 2 * i, 10, 2)
            c = np.zeros_like(a)
            reqs.append((srv.submit(a, b, c, 10, 2), a, b, c))
        with pytest.raises(y.YellError) as ei:
            srv.wait(reqs[0][0], timeout=0.05)
        assert ei.value.status == _capi.YELL_ERR_TIMEOUT
        srv.cancel(reqs[1][0])
        srv.pause(False)
        with pytest.raises(y.YellError) as ei:
            srv.wait(reqs[1][0])
        assert ei.value.status == _capi.YELL_ERR_CANCELLED
        for k in (0, 2):
            rid, a, b, c = reqs[k]
            assert srv.wait(rid)["status"] == 0
            assert np.array_equal(c, orc.polymul(a, b, 10, 0))
        assert srv.stats()["cancelled"] == 1


def test_injected_allocation_refusal(cuda, orc):
    with Server(hbm_budget_bytes=256 << 20, inject_alloc_failures=1) as srv:
        srv.pause(True)
        reqs = []
        for i in range(3):
            a, b = _operands(600 + 2 * i, 11, 2)
            c = np.zeros_like(a)
            reqs.append((srv.submit(a, b, c, 11, 2), a, b, c))
        srv.pause(False)
        with pytest.raises(y.YellError) as ei:
            srv.wait(reqs[0][0])
        assert ei.value.status == _capi.YELL_ERR_OUT_OF_MEMORY
        for rid, a, b, c in reqs[1:]:
            assert srv.wait(rid)["status"] == 0
            assert np.array_equal(c, orc.polymul(a, b, 11, 0))


def test_concurrent_submitters(cuda, orc):
    with Server(hbm_budget_bytes=1 << 30) as srv:
        results = {}

        def worker(t):
            out = []
            for i in range(10):
                log_n = 10 + (t + i) % 6
                a, b = _operands(700 + 100 * t + 2 * i, log_n, 2)
                c = np.zeros_like(a)
                out.append((srv.submit(a, b, c, log_n, 2), a, b, c, log_n))
            for rid, a, b, c, log_n in out:
                srv.wait(rid)
            results[t] = out

        th = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for t in range(4):
            for rid, a, b, c, log_n in results[t][::3]:
                assert np.array_equal(c, orc.polymul(a, b, log_n, 0))


def test_poisson_load_device_resident(cuda):
    torch = cuda
    mix = uneven_mix(4, 64)
    templates = []
    for i, (log_n, L) in enumerate(mix):
        a, b = _operands(800 + 2 * i, log_n, L)
        templates.append((torch.from_numpy(a.view(np.int64)).cuda(),
                          torch.from_numpy(b.view(np.int64)).cuda(), log_n, L, 0))
    with Server(hbm_budget_bytes=4 << 30) as srv:
        st = srv.load_test(templates, offered_rps=20000, duration_s=0.3, seed=5)
    assert st["completed"] == st["submitted"] > 1000
    assert st["failed"] == 0 and 0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]


def test_ntt_requests_in_a_mix(cuda, orc):
    """Forward and backward NTT requests (host and device, in place and not)
    served in the same batches as polymul requests; each equals the oracle."""
    torch = cuda
    with Server(hbm_budget_bytes=2 << 30, max_inflight=3) as srv:
        jobs = []
        for i, (log_n, L) in enumerate([(10, 2), (14, 1), (12, 3), (16, 2), (11, 1), (13, 2)]):
            a, b = _operands(3000 + 4 * i, log_n, L, i)
            # host forward
            f = np.zeros_like(a)
            jobs.append(("fwd", srv.submit(a, None, f, log_n, L, cm0=i, op="forward"), a, f, log_n, L, i))
            # host backward of the forward output's reference values
            fa = np.stack([orc.forward(a[l], log_n, i + l) for l in range(L)])
            bk = np.zeros_like(a)
            jobs.append(("bwd", srv.submit(fa, None, bk, log_n, L, cm0=i, op="backward"), fa, bk, log_n, L, i))
            # device forward in place
            d = torch.from_numpy(a.view(np.int64).copy()).cuda()
            jobs.append(("dfwd", srv.submit(d, None, d, log_n, L, cm0=i, device=True, op="forward"), a, d, log_n, L, i))
            # a polymul in the same batch
            c = np.zeros_like(a)
            jobs.append(("mul", srv.submit(a, b, c, log_n, L, cm0=i), (a, b), c, log_n, L, i))
        for kind, rid, x, out, log_n, L, cm0 in jobs:
            assert srv.wait(rid)["status"] == 0, kind
            if kind == "mul":
                want = orc.polymul(x[0], x[1], log_n, cm0)
            elif kind == "bwd":
                want = np.stack([orc.backward(x[l], log_n, cm0 + l) for l in range(L)])
            else:
                want = np.stack([orc.forward(x[l], log_n, cm0 + l) for l in range(L)])
            got = out if isinstance(out, np.ndarray) else out.cpu().numpy().view(np.uint64).reshape(want.shape)
            assert np.array_equal(got, want), (kind, log_n, L)
        with pytest.raises(y.YellError):
            a, _ = _operands(9, 10, 1)
            srv._submit_flags(a, None, np.zeros_like(a), 10, 1, 0, 4 | 8)
