"""GPU element-wise ops (the reference's ops functors behind poly<N>'s
operators) against the oracle on full-range words: the formulas are the
reference's own, so results must match even outside [0, p)."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import splitmix64, uniform_polys

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64).copy()).cuda()


@pytest.mark.parametrize("op", ["mulmod", "addmod", "submod", "muladd", "negate"])
@pytest.mark.parametrize("full_range", [False, True])
def test_device_elementwise(cuda, orc, op, full_range):
    torch = cuda
    log_n, count, L, cm0 = 12, 3, 4, 5
    n = 1 << log_n
    ps = y.primes(L, cm0)
    if full_range:
        a = splitmix64(7, count * L * n).reshape(count, L, n)
        b = splitmix64(8, count * L * n).reshape(count, L, n)
        acc = splitmix64(9, count * L * n).reshape(count, L, n)
    else:
        a = uniform_polys(7, count, L, log_n, ps)
        b = uniform_polys(8, count, L, log_n, ps)
        acc = uniform_polys(9, count, L, log_n, ps)
    code = {"mulmod": 0, "addmod": 1, "submod": 2, "muladd": 3, "negate": 4}[op]
    dst = _dev(torch, acc)
    y.dev_elementwise(code, dst, _dev(torch, a), _dev(torch, b), count, L, log_n, cm0)
    torch.cuda.synchronize()
    got = dst.cpu().numpy().view(np.uint64).reshape(count, L, n)
    for i in range(count):
        for l in range(L):
            cm = cm0 + l
            if op == "muladd":
                want = orc.muladd(acc[i, l], a[i, l], b[i, l], cm)
            elif op == "negate":
                want = orc.negate(a[i, l], cm)
            else:
                want = getattr(orc, op)(a[i, l], b[i, l], cm)
            assert np.array_equal(got[i, l], want), (op, i, l)


def test_poly_operators_host(cuda, orc):
    """poly<N> operators * + - *= += -=, add_product_of and negate through the
    host-memory drop-ins (include/yell/poly.hpp:163-168)."""
    log_n, L = 11, 3
    ps = y.primes(L)
    a = y.Poly(log_n, L, uniform_polys(70, 1, L, log_n, ps)[0])
    b = y.Poly(log_n, L, uniform_polys(71, 1, L, log_n, ps)[0])
    for name, fn in (("mulmod", lambda u, v: u * v), ("addmod", lambda u, v: u + v),
                     ("submod", lambda u, v: u - v)):
        r = fn(a, b)
        for l in range(L):
            assert np.array_equal(r.limbs[l], getattr(orc, name)(a.limbs[l], b.limbs[l], l))
    c = a.copy()
    c *= b
    assert c == a * b
    c = a.copy()
    c += b
    assert c == a + b
    c = a.copy()
    c -= b
    assert c == a - b
    acc = a.copy()
    acc.add_product_of(a, b)
    for l in range(L):
        assert np.array_equal(acc.limbs[l], orc.muladd(a.limbs[l], a.limbs[l], b.limbs[l], l))
    n = a.copy().negate()
    for l in range(L):
        assert np.array_equal(n.limbs[l], orc.negate(a.limbs[l], l))


def test_rlwe_style_round_trip(cuda, orc):
    """The example.cpp call pattern on lazy forward outputs: forward_lazy,
    add_product_of, backward (include/yell/details/poly.hpp:118-186)."""
    log_n, L = 13, 4
    ps = y.primes(L)
    s = y.Poly(log_n, L, uniform_polys(80, 1, L, log_n, ps)[0]).forward()
    u = y.Poly(log_n, L, uniform_polys(81, 1, L, log_n, ps)[0])
    e = y.Poly(log_n, L, uniform_polys(82, 1, L, log_n, ps)[0])
    ref_s = [orc.forward(x, log_n, l) for l, x in enumerate(uniform_polys(80, 1, L, log_n, ps)[0])]
    e.forward_lazy()
    ref_e = [orc.forward_lazy(x, log_n, l) for l, x in enumerate(uniform_polys(82, 1, L, log_n, ps)[0])]
    for l in range(L):
        assert np.array_equal(e.limbs[l], ref_e[l])
    e.add_product_of(u, s)
    ref = [orc.muladd(ref_e[l], u.limbs[l], ref_s[l], l) for l in range(L)]
    for l in range(L):
        assert np.array_equal(e.limbs[l], ref[l])
    e.backward()
    for l in range(L):
        assert np.array_equal(e.limbs[l], orc.backward(ref[l], log_n, l))
