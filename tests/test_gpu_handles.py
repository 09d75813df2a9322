"""Device-resident poly handles (the device-side poly<N>,
include/yell/poly.hpp:43-168) and asynchronous batch tickets, against the
oracle."""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300.inputs import uniform_polys

pytestmark = pytest.mark.gpu


def _poly(seed, L, log_n, cm0=0):
    return uniform_polys(seed, 1, L, log_n, y.primes(L, cm0))[0]


def test_upload_download_roundtrip(cuda):
    a = _poly(1, 3, 10, 4)
    h = y.DevPoly(10, 3, 4, a)
    assert np.array_equal(h.download(), a)
    h.free()
    h.free()  # idempotent


@pytest.mark.parametrize("log_n", [3, 12, 16])
def test_handle_ntt(cuda, orc, log_n):
    L = 2
    a = _poly(2 + log_n, L, log_n, 1)
    h = y.DevPoly(log_n, L, 1, a).forward()
    want = np.stack([orc.forward(a[l], log_n, 1 + l) for l in range(L)])
    assert np.array_equal(h.download(), want)
    h.backward()
    assert np.array_equal(h.download(), a)
    h.upload(a).forward_lazy()
    want = np.stack([orc.forward_lazy(a[l], log_n, 1 + l) for l in range(L)])
    assert np.array_equal(h.download(), want)


def test_handle_operators(cuda, orc):
    """a.forward(); b.forward(); c = a * b; c += a; c.add_product_of(a, b);
    c.negate(); c.backward(): the reference's example.cpp chain."""
    L, log_n = 3, 11
    a, b = _poly(10, L, log_n), _poly(11, L, log_n)
    ha, hb = y.DevPoly(log_n, L, 0, a).forward(), y.DevPoly(log_n, L, 0, b).forward()
    hc = y.DevPoly(log_n, L)
    hc.op(y.YELL_OP_MULMOD, ha, hb).op(y.YELL_OP_ADDMOD, hc, ha).add_product_of(ha, hb)
    hc.op(y.YELL_OP_SUBMOD, hc, hb).negate().backward()
    for l in range(L):
        fa, fb = orc.forward(a[l], log_n, l), orc.forward(b[l], log_n, l)
        c = orc.mulmod(fa, fb, l)
        c = orc.addmod(c, fa, l)
        c = orc.muladd(c, fa, fb, l)
        c = orc.submod(c, fb, l)
        c = orc.negate(c, l)
        c = orc.backward(c, log_n, l)
        assert np.array_equal(hc.download()[l], c), l


@pytest.mark.parametrize("log_n", [10, 14, 16])
def test_handle_mul(cuda, orc, log_n):
    L = 4
    a, b = _poly(20, L, log_n), _poly(21, L, log_n)
    hc = y.DevPoly(log_n, L).mul(y.DevPoly(log_n, L, 0, a), y.DevPoly(log_n, L, 0, b))
    assert np.array_equal(hc.download(), orc.polymul(a, b, log_n))


def test_batch_ticket_uneven(cuda, orc):
    shapes = [(10, 1), (16, 3), (12, 2), (14, 5), (10, 4), (16, 1)]
    A, B, hs = [], [], []
    for i, (log_n, L) in enumerate(shapes):
        a, b = _poly(100 + i, L, log_n), _poly(200 + i, L, log_n)
        A.append(a)
        B.append(b)
        hs.append((y.DevPoly(log_n, L), y.DevPoly(log_n, L, 0, a), y.DevPoly(log_n, L, 0, b)))
    t = y.batch_submit([h[0] for h in hs], [h[1] for h in hs], [h[2] for h in hs])
    t.wait(60.0)
    for i, (log_n, L) in enumerate(shapes):
        assert np.array_equal(hs[i][0].download(), orc.polymul(A[i], B[i], log_n)), shapes[i]


def test_handle_errors(cuda):
    a = y.DevPoly(10, 2)
    b = y.DevPoly(11, 2)
    c = y.DevPoly(10, 3)
    with pytest.raises(y.YellError):
        a.mul(a, a)  # product over an operand
    with pytest.raises(y.YellError):
        y.DevPoly(10, 2).mul(a, b)  # degree mismatch
    with pytest.raises(y.YellError):
        c.op(y.YELL_OP_ADDMOD, a, a)  # limb count mismatch
    with pytest.raises(y.YellError):
        y.batch_submit([a], [a], [a])
    with pytest.raises(ValueError):
        a.upload([np.zeros(1024, dtype=np.uint64)])
    with pytest.raises(y.YellError):
        y.DevPoly(10, 0)
