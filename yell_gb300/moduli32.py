"""32-bit moduli mode (the reference built with -DYELL_USE_32BITS_MODULI,
include/yell/params_32.hpp): 291 30-bit primes, uint32 words, N = 2^3..2^15.

Host calls take numpy uint32 arrays; device calls take torch CUDA int32
tensors (the words are used as raw uint32).  Every call runs the CUDA
library.
"""
from __future__ import annotations

import numpy as np

from ._capi import YELL_BACKWARD, YELL_FORWARD, YELL_FORWARD_LAZY, call, load


def max_moduli() -> int:
    return int(load().yell32_max_moduli())


def max_log_degree() -> int:
    return int(load().yell32_max_log_degree())


def prime(cm: int) -> int:
    return int(load().yell32_prime(cm))


def primes(L: int, cm0: int = 0) -> np.ndarray:
    return np.array([prime(cm0 + i) for i in range(L)], dtype=np.uint32)


def prime_pn(cm: int) -> int:
    return int(load().yell32_prime_pn(cm))


def primitive_root(cm: int) -> int:
    return int(load().yell32_primitive_root(cm))


def init_ntt_tables(log_n: int, L: int, cm0: int = 0) -> None:
    call("yell32_init_ntt_tables", log_n, cm0, L)


def ntt_tables(log_n: int, cm: int):
    n = 1 << log_n
    out = np.zeros(4 * n, dtype=np.uint32)
    sc = np.zeros(4, dtype=np.uint32)
    call("yell32_ntt_tables", log_n, cm, out.ctypes.data, sc.ctypes.data)
    return out.reshape(4, n), sc


def _host(name, x, log_n, cm):
    a = np.ascontiguousarray(x, dtype=np.uint32).copy()
    if a.size != 1 << log_n:
        raise ValueError("limb size does not match log_n")
    call(name, a.ctypes.data, log_n, cm)
    return a


def ntt_forward(x, log_n: int, cm: int) -> np.ndarray:
    return _host("yell32_ntt_forward", x, log_n, cm)


def ntt_forward_lazy(x, log_n: int, cm: int) -> np.ndarray:
    return _host("yell32_ntt_forward_lazy", x, log_n, cm)


def ntt_backward(x, log_n: int, cm: int) -> np.ndarray:
    return _host("yell32_ntt_backward", x, log_n, cm)


def _dptr(t) -> int:
    if not t.is_cuda or t.element_size() != 4 or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor of 32-bit words")
    return t.data_ptr()


def _stream(stream):
    if stream is None:
        return None
    return getattr(stream, "cuda_stream", stream)


def dev_ntt(t, count: int, L: int, log_n: int, cm0: int = 0, direction: int = YELL_FORWARD,
            stream=None) -> None:
    call("yell32_dev_ntt", _dptr(t), count, L, log_n, cm0, direction, _stream(stream))


def dev_polymul(c, a, b, pairs: int, L: int, log_n: int, cm0: int = 0, stream=None) -> None:
    call("yell32_dev_polymul", _dptr(c), _dptr(a), _dptr(b), pairs, L, log_n, cm0, _stream(stream))


def wait_status() -> int:
    """Waits for the device's queued work and returns (and clears) the status the
    2^14 / 2^15 polymul kernels record when a wait for their operand copies runs out."""
    import ctypes
    st = ctypes.c_uint32(0)
    call("yell32_wait_status", ctypes.byref(st))
    return st.value


def wait_check(timeout_s: float) -> int:
    """Runs the check of the bounded copy wait: a wait that nothing completes runs
    out after timeout_s and the returned status is YELL_ERR_TIMEOUT."""
    import ctypes
    st = ctypes.c_uint32(0)
    call("yell32_wait_check", int(timeout_s * 1e9), ctypes.byref(st))
    return st.value


def dev_elementwise(op: int, dst, a, b, count: int, L: int, log_n: int, cm0: int = 0,
                    stream=None) -> None:
    call("yell32_dev_elementwise", op, _dptr(dst), _dptr(a), _dptr(b) if b is not None else None,
         count, L, log_n, cm0, _stream(stream))


def calibrate_butterflies() -> tuple[float, float]:
    """Register-only rate of the 32-bit butterflies on this GPU: (CT per s, GS per s)."""
    import ctypes

    ct, gs = ctypes.c_double(), ctypes.c_double()
    call("yell32_calibrate_butterflies", ctypes.addressof(ct), ctypes.addressof(gs))
    return ct.value, gs.value


__all__ = ["calibrate_butterflies", "max_moduli", "max_log_degree", "prime", "primes", "prime_pn", "primitive_root",
           "init_ntt_tables", "ntt_tables", "ntt_forward", "ntt_forward_lazy", "ntt_backward",
           "dev_ntt", "dev_polymul", "dev_elementwise", "YELL_FORWARD", "YELL_FORWARD_LAZY",
           "YELL_BACKWARD"]
