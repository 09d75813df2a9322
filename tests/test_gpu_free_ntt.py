"""The reference's runtime-N free functions negacylic_forward_lazy /
negacylic_backward_lazy (include/yell/details/ntt.hpp:10-23) with caller
tables, on the GPU against the oracle's restatement of lib/ntt.cpp:89-210
(itself pinned to the reference's compiled functions)."""
import ctypes

import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300._capi import call
from yell_gb300.inputs import splitmix64

pytestmark = pytest.mark.gpu


def _run(name, x, w, ws, p):
    a = np.ascontiguousarray(x, dtype=np.uint64).copy()
    call(name, a.ctypes.data, a.size, np.ascontiguousarray(w).ctypes.data, np.ascontiguousarray(ws).ctypes.data, p)
    return a


@pytest.mark.parametrize("log_n", [2, 3, 4, 9, 13, 16, 18, 20])
def test_free_functions_with_the_reference_tables(cuda, orc, log_n):
    cm = 5
    p = orc.prime(cm)
    t, _ = orc.tables(log_n, cm)
    n = 1 << log_n
    x4 = splitmix64(40 + log_n, n) % np.uint64(4 * p)
    x2 = splitmix64(50 + log_n, n) % np.uint64(2 * p)
    assert np.array_equal(_run("yell_negacyclic_forward_lazy", x4, t[0], t[1], p),
                          orc.negacyclic_lazy(x4, t[0], t[1], p))
    assert np.array_equal(_run("yell_negacyclic_backward_lazy", x2, t[2], t[3], p),
                          orc.negacyclic_lazy(x2, t[2], t[3], p, inverse=True))


def test_free_functions_follow_caller_tables(cuda, orc):
    """Arbitrary twiddles (not powers of a root): the functions apply whatever
    table they are given, like the reference's."""
    log_n, cm = 11, 0
    n = 1 << log_n
    p = orc.prime(cm)
    w = splitmix64(7, n) % np.uint64(p)
    ws = np.array([orc.shoupify(int(v), cm) for v in w], dtype=np.uint64)
    x = splitmix64(8, n) % np.uint64(2 * p)
    assert np.array_equal(_run("yell_negacyclic_forward_lazy", x, w, ws, p), orc.negacyclic_lazy(x, w, ws, p))
    assert np.array_equal(_run("yell_negacyclic_backward_lazy", x, w, ws, p),
                          orc.negacyclic_lazy(x, w, ws, p, inverse=True))


def test_free_function_errors(cuda):
    x = np.zeros(12, dtype=np.uint64)
    with pytest.raises(y.YellError):
        call("yell_negacyclic_forward_lazy", x.ctypes.data, 12, x.ctypes.data, x.ctypes.data, 97)
    with pytest.raises(y.YellError):
        call("yell_negacyclic_forward_lazy", x.ctypes.data, 8, x.ctypes.data, x.ctypes.data, 1 << 63)
