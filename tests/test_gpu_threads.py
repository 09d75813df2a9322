"""Reentrancy: the reference's calls are safe from several host threads on
different buffers (its tables are built under a lock); so are the drop-ins
and device calls here.  Eight threads mix host NTTs, host polymuls, table
builds of new degrees and device polymuls on their own buffers."""
import threading

import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def test_concurrent_calls_from_host_threads(cuda, orc):
    torch = cuda
    errors = []

    def worker(k):
        try:
            log_n = 10 + k % 4
            L = 1 + k % 3
            ps = y.primes(L, k)
            a = uniform_polys(5000 + k, 1, L, log_n, ps)[0]
            b = uniform_polys(5100 + k, 1, L, log_n, ps)[0]
            for rep in range(5):
                f = y.ntt_forward(a[0], log_n, k)
                if not np.array_equal(f, orc.forward(a[0], log_n, k)):
                    errors.append(("forward", k, rep))
                c = y.polymul_host(a[None], b[None], log_n, cm0=k)
                if not np.array_equal(c[0], orc.polymul(a, b, log_n, k)):
                    errors.append(("polymul_host", k, rep))
                da = torch.from_numpy(a.view(np.int64).copy()).cuda()
                db = torch.from_numpy(b.view(np.int64).copy()).cuda()
                dc = torch.empty_like(da)
                s = torch.cuda.Stream()
                y.dev_polymul(dc, da, db, 1, L, log_n, k, stream=s)
                s.synchronize()
                if not np.array_equal(dc.cpu().numpy().view(np.uint64), c[0]):
                    errors.append(("dev_polymul", k, rep))
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(("exception", k, repr(e)))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads)
    assert errors == []
