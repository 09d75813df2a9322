"""32-bit moduli mode on the GPU (the reference's -DYELL_USE_32BITS_MODULI
build) against the 32-bit oracle, word for word, at every degree."""
import numpy as np
import pytest

import oracle
from yell_gb300 import YellError
from yell_gb300 import moduli32 as m32
from yell_gb300._capi import YELL_OP_ADDMOD, YELL_OP_MULADD, YELL_OP_MULMOD, YELL_OP_NEGATE, YELL_OP_SUBMOD
from yell_gb300.inputs import splitmix64

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def o32():
    return oracle.Oracle32("port")


def _polys(seed, count, L, log_n, cm0, mult=1):
    n = 1 << log_n
    w = splitmix64(seed, count * L * n).reshape(count, L, n)
    ps = np.array([m32.prime(cm0 + l) for l in range(L)], dtype=np.uint64).reshape(1, L, 1)
    return (w % (ps * np.uint64(mult))).astype(np.uint32)


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32).reshape(-1).copy()).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.uint32).reshape(shape)


@pytest.mark.parametrize("log_n", list(range(3, 16)))
def test_device_ntt_all_degrees(cuda, o32, log_n):
    count, L, cm0 = 3, 2, 7
    n = 1 << log_n
    x4 = _polys(100 + log_n, count, L, log_n, cm0, 4)
    x2 = (x4 % np.array([2 * m32.prime(cm0 + l) for l in range(L)], dtype=np.uint32).reshape(1, L, 1)).astype(np.uint32)
    for direction, name, x in ((m32.YELL_FORWARD, "forward", x4), (m32.YELL_FORWARD_LAZY, "forward_lazy", x4),
                               (m32.YELL_BACKWARD, "backward", x2)):
        t = _dev(cuda, x)
        m32.dev_ntt(t, count, L, log_n, cm0, direction)
        cuda.cuda.synchronize()
        got = _host(t, (count, L, n))
        for i in range(count):
            for l in range(L):
                want = getattr(o32, name)(x[i, l], log_n, cm0 + l)
                assert np.array_equal(got[i, l], want), (name, log_n, i, l)


@pytest.mark.parametrize("log_n", [3, 6, 10, 11, 12, 14, 15])
def test_device_polymul(cuda, o32, log_n):
    pairs, L, cm0 = 2, 3, 288 if log_n == 3 else 0
    n = 1 << log_n
    a = _polys(200 + log_n, pairs, L, log_n, cm0)
    b = _polys(300 + log_n, pairs, L, log_n, cm0)
    c = cuda.zeros(pairs * L * n, dtype=cuda.int32, device="cuda")
    m32.dev_polymul(c, _dev(cuda, a), _dev(cuda, b), pairs, L, log_n, cm0)
    cuda.cuda.synchronize()
    assert m32.wait_status() == 0
    got = _host(c, (pairs, L, n))
    for i in range(pairs):
        assert np.array_equal(got[i], o32.polymul(a[i], b[i], log_n, cm0)), (log_n, i)


@pytest.mark.parametrize("log_n", [14, 15])
def test_polymul_offset_operands(cuda, o32, log_n):
    """Operands and output 16 bytes past an allocation's start: the bulk copies
    that stage the CTA-pair kernel's operands need 16-byte alignment only."""
    pairs, L = 2, 2
    n = 1 << log_n
    a, b = _polys(21, pairs, L, log_n, 0), _polys(22, pairs, L, log_n, 0)
    words = pairs * L * n

    def shifted(x):
        t = cuda.zeros(words + 4, dtype=cuda.int32, device="cuda")
        t[4:] = _dev(cuda, x)
        return t[4:]

    c = cuda.zeros(words + 4, dtype=cuda.int32, device="cuda")[4:]
    m32.dev_polymul(c, shifted(a), shifted(b), pairs, L, log_n, 0)
    assert m32.wait_status() == 0
    got = _host(c, (pairs, L, n))
    for i in range(pairs):
        assert np.array_equal(got[i], o32.polymul(a[i], b[i], log_n)), (log_n, i)


def test_polymul_many_limbs(cuda, o32):
    """A batch whose limb count is not a multiple of the limbs per CTA."""
    pairs, L, log_n = 5, 7, 9
    n = 1 << log_n
    a, b = _polys(7, pairs, L, log_n, 0), _polys(8, pairs, L, log_n, 0)
    c = cuda.zeros(pairs * L * n, dtype=cuda.int32, device="cuda")
    m32.dev_polymul(c, _dev(cuda, a), _dev(cuda, b), pairs, L, log_n)
    cuda.cuda.synchronize()
    got = _host(c, (pairs, L, n))
    for i in range(pairs):
        assert np.array_equal(got[i], o32.polymul(a[i], b[i], log_n))


@pytest.mark.parametrize("op", ["mulmod", "addmod", "submod", "muladd", "negate"])
def test_device_elementwise(cuda, o32, op):
    count, L, log_n, cm0 = 2, 3, 10, 100
    a, b, acc = (_polys(s, count, L, log_n, cm0) for s in (1, 2, 3))
    code = {"mulmod": YELL_OP_MULMOD, "addmod": YELL_OP_ADDMOD, "submod": YELL_OP_SUBMOD,
            "muladd": YELL_OP_MULADD, "negate": YELL_OP_NEGATE}[op]
    dst = _dev(cuda, acc)
    m32.dev_elementwise(code, dst, _dev(cuda, a), _dev(cuda, b), count, L, log_n, cm0)
    cuda.cuda.synchronize()
    got = _host(dst, a.shape)
    for i in range(count):
        for l in range(L):
            cm = cm0 + l
            if op == "muladd":
                want = o32.muladd(acc[i, l], a[i, l], b[i, l], cm)
            elif op == "negate":
                want = o32.negate(a[i, l], cm)
            else:
                want = getattr(o32, op)(a[i, l], b[i, l], cm)
            assert np.array_equal(got[i, l], want), (op, i, l)


@pytest.mark.parametrize("log_n", [3, 10, 15])
def test_host_dropins(cuda, o32, log_n):
    x = _polys(9, 1, 1, log_n, 5, 4)[0, 0]
    assert np.array_equal(m32.ntt_forward(x, log_n, 5), o32.forward(x, log_n, 5))
    assert np.array_equal(m32.ntt_forward_lazy(x, log_n, 5), o32.forward_lazy(x, log_n, 5))
    x2 = (x % np.uint32(2 * m32.prime(5))).astype(np.uint32)
    assert np.array_equal(m32.ntt_backward(x2, log_n, 5), o32.backward(x2, log_n, 5))


def test_full_size_roundtrip(cuda):
    """N = 2^15, L = 32, 16 pairs: forward then backward is the identity and
    the polymul by the constant 1 is the identity."""
    pairs, L, log_n = 16, 32, 15
    n = 1 << log_n
    a = _polys(11, pairs, L, log_n, 0)
    t = _dev(cuda, a)
    m32.dev_ntt(t, pairs, L, log_n, 0, m32.YELL_FORWARD)
    m32.dev_ntt(t, pairs, L, log_n, 0, m32.YELL_BACKWARD)
    cuda.cuda.synchronize()
    assert np.array_equal(_host(t, a.shape), a)
    one = np.zeros_like(a)
    one[:, :, 0] = 1
    c = cuda.zeros_like(t)
    m32.dev_polymul(c, _dev(cuda, a), _dev(cuda, one), pairs, L, log_n, 0)
    cuda.cuda.synchronize()
    assert m32.wait_status() == 0
    assert np.array_equal(_host(c, a.shape), a)


def test_wait_check(cuda, o32):
    """The staged 2^14 / 2^15 polymul's bounded copy wait: a wait that nothing
    completes runs out and reports YELL_ERR_TIMEOUT, no GPU fault; the status is
    read and cleared, and a polymul afterwards runs normally."""
    from yell_gb300._capi import YELL_ERR_TIMEOUT
    assert m32.wait_check(0.02) == YELL_ERR_TIMEOUT
    assert m32.wait_status() == 0
    with pytest.raises(YellError):
        m32.wait_check(0.0)
    pairs, L, log_n = 1, 2, 15
    a, b = _polys(31, pairs, L, log_n, 0), _polys(32, pairs, L, log_n, 0)
    c = cuda.zeros(pairs * L << log_n, dtype=cuda.int32, device="cuda")
    m32.dev_polymul(c, _dev(cuda, a), _dev(cuda, b), pairs, L, log_n, 0)
    assert m32.wait_status() == 0
    assert np.array_equal(_host(c, (pairs, L, 1 << log_n))[0], o32.polymul(a[0], b[0], log_n))


def test_errors(cuda):
    t = cuda.zeros(1 << 16, dtype=cuda.int32, device="cuda")
    with pytest.raises(YellError):
        m32.dev_ntt(t, 1, 1, 16, 0)  # above 2^15
    with pytest.raises(YellError):
        m32.dev_ntt(t, 1, 1, 2, 0)
    with pytest.raises(YellError):
        m32.dev_ntt(t, 1, 2, 10, 290)  # past the 291 moduli
    with pytest.raises(YellError):
        m32.dev_polymul(t, t, t, 1, 1, 10)
    with pytest.raises(YellError):
        m32.dev_ntt(t[1:], 1, 1, 10, 0)  # misaligned


def test_host_poly_dropins(cuda, o32):
    """yell32_poly_* (poly<N> members on host limbs, moduli 0 .. L-1)."""
    import ctypes

    from yell_gb300._capi import call

    L, log_n = 3, 11
    n = 1 << log_n
    a = [np.ascontiguousarray(x) for x in _polys(31, 1, L, log_n, 0)[0]]
    b = [np.ascontiguousarray(x) for x in _polys(32, 1, L, log_n, 0)[0]]

    def arr(ls):
        return (ctypes.c_void_p * len(ls))(*[x.ctypes.data for x in ls])

    f = [x.copy() for x in a]
    call("yell32_poly_forward", arr(f), L, log_n)
    for l in range(L):
        assert np.array_equal(f[l], o32.forward(a[l], log_n, l))
    d = [np.zeros(n, np.uint32) for _ in range(L)]
    call("yell32_poly_mulmod", arr(d), arr(f), arr(b), L, log_n)
    for l in range(L):
        assert np.array_equal(d[l], o32.mulmod(f[l], b[l], l))
    acc = [x.copy() for x in b]
    call("yell32_poly_add_product_of", arr(acc), arr(f), arr(a), L, log_n)
    for l in range(L):
        assert np.array_equal(acc[l], o32.muladd(b[l], f[l], a[l], l))
    call("yell32_poly_backward", arr(f), L, log_n)
    for l in range(L):
        assert np.array_equal(f[l], a[l])
    g = [x.copy() for x in a]
    call("yell32_poly_negate", arr(g), L, log_n)
    for l in range(L):
        assert np.array_equal(g[l], o32.negate(a[l], l))
