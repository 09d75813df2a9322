"""yell_dev_polymul_noalloc: the fused polymul for callers that cannot
allocate device memory (HBM owned by a fixed budget or a pooled allocator,
or a latency-critical path that cannot let cudaMalloc/cudaFree synchronise
the device).  Its scratch is a fixed 16 MiB array inside the library,
brought up when the twiddle tables are first built on the device.

Checked through the C ABI against yell_dev_polymul (the allocating entry
point with caller scratch) on two calls in a row; results must be identical
word for word, and neither call may allocate: the library's own allocation
counter (yell_allocations) must not move across either call, and, as a loose
second check, the device's free memory must not shrink.  This file is
collected last so that a run stopping at the first failure has already run
every other test; it sets up its own state, so it also passes alone in a
fresh process."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300 import _capi
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


@pytest.mark.parametrize("log_n,pairs,L,cm0", [(16, 1, 32, 0), (14, 4, 8, 3), (12, 3, 5, 1)])
def test_noalloc_matches_allocating_polymul_twice(cuda, log_n, pairs, L, cm0):
    torch = cuda
    lib = y.load()
    y.init_ntt_tables(log_n, L, cm0)  # building tables allocates: done up front
    ps = y.primes(L, cm0)
    for call in range(2):
        a = uniform_polys(900 + 10 * call + log_n, pairs, L, log_n, ps)
        b = uniform_polys(950 + 10 * call + log_n, pairs, L, log_n, ps)
        da, db = _dev(torch, a), _dev(torch, b)
        want = torch.empty(a.size, dtype=torch.int64, device="cuda")
        sw = y.polymul_scratch_words(pairs, L, log_n)
        scratch = torch.empty(max(sw, 2), dtype=torch.int64, device="cuda")
        y.dev_polymul(want, da, db, pairs, L, log_n, cm0, scratch=scratch if sw else None)
        got = torch.full((a.size,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        allocs_before = y.allocations()
        st = lib.yell_dev_polymul_noalloc(got.data_ptr(), da.data_ptr(), db.data_ptr(), pairs, L,
                                          log_n, cm0, None)
        assert st == _capi.YELL_OK, lib.yell_last_error()
        assert y.allocations() == allocs_before, f"call {call} allocated"
        assert lib.yell_synchronize() == _capi.YELL_OK
        # loose: other processes share the device, but nothing of ours may take memory
        assert torch.cuda.mem_get_info()[0] >= free_before - (1 << 20), f"call {call} took device memory"
        assert torch.equal(got, want), f"call {call} differs from yell_dev_polymul"


def test_noalloc_rejects_oversize_and_missing_tables(cuda):
    torch = cuda
    lib = y.load()
    log_n = 16
    y.init_ntt_tables(log_n, 33)
    n = 33 << log_n  # 33 limbs of 2^16 need 33 * 2^16 > 2^21 scratch words
    buf = [torch.empty(n, dtype=torch.int64, device="cuda") for _ in range(3)]
    st = lib.yell_dev_polymul_noalloc(buf[0].data_ptr(), buf[1].data_ptr(), buf[2].data_ptr(), 1, 33,
                                      log_n, 0, None)
    assert st == _capi.YELL_ERR_INVALID_ARGUMENT
    assert b"fixed scratch" in lib.yell_last_error()
    # tables never built for these moduli at this degree
    st = lib.yell_dev_polymul_noalloc(buf[0].data_ptr(), buf[1].data_ptr(), buf[2].data_ptr(), 1, 2,
                                      15, 990, None)
    assert st == _capi.YELL_ERR_INVALID_ARGUMENT
    assert b"not resident" in lib.yell_last_error()


@pytest.mark.parametrize("variant", [1, 2])
def test_noalloc_two_pass_degree_13_beyond_fixed_scratch(cuda, variant):
    """2^13 with a two-pass variant selected: 160 pairs of L = 2 (320 limbs)
    need more scratch than the fixed array holds (256 limbs), so the call runs
    the scratch-free whole-limb polymul, and its words equal the two-pass
    result of yell_dev_polymul."""
    torch = cuda
    lib = y.load()
    log_n, pairs, L = 13, 160, 2
    assert y.polymul_scratch_words(pairs, L, log_n) > 1 << 21
    y.init_ntt_tables(log_n, L, 0)
    ps = y.primes(L, 0)
    a = uniform_polys(1300 + variant, pairs, L, log_n, ps)
    b = uniform_polys(1350 + variant, pairs, L, log_n, ps)
    da, db = _dev(torch, a), _dev(torch, b)
    before = y.get_variant(log_n)
    y.set_variant(log_n, variant)
    try:
        want = torch.empty(a.size, dtype=torch.int64, device="cuda")
        y.dev_polymul(want, da, db, pairs, L, log_n, 0)
        got = torch.full((a.size,), -1, dtype=torch.int64, device="cuda")
        st = lib.yell_dev_polymul_noalloc(got.data_ptr(), da.data_ptr(), db.data_ptr(), pairs, L,
                                          log_n, 0, None)
        assert st == _capi.YELL_OK, lib.yell_last_error()
        assert lib.yell_synchronize() == _capi.YELL_OK
    finally:
        y.set_variant(log_n, before)
    assert torch.equal(got, want)
