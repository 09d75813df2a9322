"""Host-pointer calls whose limbs move by kernels that load and store the
caller's pageable host memory in place (GB300 with Grace: NVLink-C2C and the
host's page tables), against the same calls through driver copies and the
oracle: NTT forward / lazy / backward and every element-wise op on the
reference's layout (one host allocation per limb), plus a limb that is not
16-byte aligned (it takes the copies)."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def _limbs(x):
    return [np.array(x[l], copy=True) for l in range(x.shape[0])]


@pytest.fixture
def both_paths(cuda):
    """Yields the two settings; restores direct access afterwards."""
    yield [True, False]
    y.set_host_access(True)


def test_direct_path_is_used_where_supported(cuda):
    y.set_host_access(True)
    if not y.host_access():
        pytest.skip("device does not reach pageable host memory through the host's page tables")
    y.set_host_access(False)
    assert not y.host_access()
    y.set_host_access(True)
    assert y.host_access()


@pytest.mark.parametrize("log_n, L", [(16, 32), (17, 3), (15, 2), (8, 300)])  # 300: two gather launches
def test_host_ntt_paths(cuda, orc, both_paths, log_n, L):
    ps = y.primes(L)
    x = uniform_polys(4100 + log_n, 1, L, log_n, ps)[0]
    x4 = x + ps.reshape(L, 1) * np.uint64(3)  # lazy inputs in [0, 4p)
    want_f = [orc.forward(x4[l], log_n, l) for l in range(L)]
    want_l = [orc.forward_lazy(x4[l], log_n, l) for l in range(L)]
    want_b = [orc.backward(x[l], log_n, l) for l in range(L)]
    for direct in both_paths:
        y.set_host_access(direct)
        for fn, src, want in ((y.poly_forward, x4, want_f), (y.poly_forward_lazy, x4, want_l),
                              (y.poly_backward, x, want_b)):
            limbs = _limbs(src)
            fn(limbs)
            for l in range(L):
                assert np.array_equal(limbs[l], want[l]), (direct, fn.__name__, l)


def test_host_elementwise_paths(cuda, orc, both_paths):
    log_n, L = 16, 4
    ps = y.primes(L)
    a = uniform_polys(4200, 1, L, log_n, ps)[0]
    b = uniform_polys(4201, 1, L, log_n, ps)[0]
    acc = uniform_polys(4202, 1, L, log_n, ps)[0]
    for direct in both_paths:
        y.set_host_access(direct)
        for name, ref in (("poly_mulmod", orc.mulmod), ("poly_addmod", orc.addmod), ("poly_submod", orc.submod)):
            dst = _limbs(np.zeros_like(a))
            getattr(y, name)(dst, _limbs(a), _limbs(b))
            for l in range(L):
                assert np.array_equal(dst[l], ref(a[l], b[l], l)), (direct, name, l)
        got = _limbs(acc)
        y.poly_add_product_of(got, _limbs(a), _limbs(b))
        for l in range(L):
            assert np.array_equal(got[l], orc.muladd(acc[l], a[l], b[l], l)), (direct, "muladd", l)
        got = _limbs(a)
        y.poly_negate(got)
        for l in range(L):
            assert np.array_equal(got[l], orc.negate(a[l], l)), (direct, "negate", l)


def test_misaligned_limb_takes_the_copies(cuda, orc):
    y.set_host_access(True)
    log_n, L = 16, 2
    ps = y.primes(L)
    x = uniform_polys(4300, 1, L, log_n, ps)[0]
    raw = np.zeros((1 << log_n) + 1, dtype=np.uint64)
    off = 1 if raw.ctypes.data % 16 == 0 else 0  # an address 8 bytes past a 16-byte boundary
    limb0 = raw[off:off + (1 << log_n)]
    assert limb0.ctypes.data % 16 == 8
    limb0[:] = x[0]
    limbs = [limb0, np.array(x[1], copy=True)]
    y.poly_forward(limbs)
    assert np.array_equal(limbs[0], orc.forward(x[0], log_n, 0))
    assert np.array_equal(limbs[1], orc.forward(x[1], log_n, 1))
