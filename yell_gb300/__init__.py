"""yell_gb300: GB300 (sm_103a) implementation of YELL's RNS polynomial hot path.

Python mirror of the reference's call surface (fionser/YELL
``yell::ntt<N>``, ``yell::poly<N>``, ``yell::ops``) over the C ABI in
``include/yell_gb300.h``.  Host-memory calls take numpy uint64 arrays;
device-resident calls take torch CUDA tensors (any 64-bit integer dtype; the
words are used as raw uint64).  Every call runs the CUDA library; there is no
CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi, moduli32
from ._capi import (YELL_BACKWARD, YELL_FORWARD, YELL_FORWARD_LAZY, YELL_OP_ADDMOD,
                    YELL_OP_MULADD, YELL_OP_MULMOD, YELL_OP_NEGATE, YELL_OP_SUBMOD, YellError,
                    call, load)

__all__ = [
    "YellError", "load", "prime", "primes", "max_moduli", "min_log_degree", "max_log_degree",
    "init_ntt_tables", "ntt_tables", "ntt_forward", "ntt_forward_lazy", "ntt_backward",
    "poly_forward", "poly_forward_lazy", "poly_backward", "poly_mulmod", "poly_addmod",
    "poly_submod", "poly_add_product_of", "poly_negate", "polymul_host", "set_host_access", "host_access",
    "dev_ntt",
    "dev_ntt_limbs", "dev_elementwise", "dev_polymul", "polymul_scratch_words", "kernel_launches", "allocations",
    "Poly", "PinnedBuffer", "sample_uniform", "sample_zo", "sample_hwt", "sample_gaussian",
    "crt_words", "dev_crt_lift", "poly_to_bigint", "words_to_ints", "DevPoly", "BatchTicket",
    "batch_submit", "dev_polymul_batch_queue", "dev_polymul_batch_phased", "batch_queue_status", "batch_queue_wait_check",
]


def _u64(a) -> np.ndarray:
    a = np.ascontiguousarray(a)
    if a.dtype != np.uint64:
        a = a.astype(np.uint64)
    return a


def _addr(a: np.ndarray) -> int:
    return a.ctypes.data


def _ptr_array(arrs) -> ctypes.Array:
    arr = (ctypes.c_void_p * len(arrs))()
    for i, a in enumerate(arrs):
        arr[i] = a.ctypes.data
    return arr


# --- params ---------------------------------------------------------------
def max_moduli() -> int:
    return int(load().yell_max_moduli())


def min_log_degree() -> int:
    return int(load().yell_min_log_degree())


def max_log_degree() -> int:
    return int(load().yell_max_log_degree())


def prime(cm: int) -> int:
    return int(load().yell_prime(cm))


def primes(L: int, cm0: int = 0) -> np.ndarray:
    return np.array([prime(cm0 + i) for i in range(L)], dtype=np.uint64)


def kernel_launches() -> int:
    return int(load().yell_kernel_launches())


def allocations() -> int:
    """Device, pinned-host and pool allocations the library made so far."""
    return int(load().yell_allocations())


# --- tables -----------------------------------------------------------------
def init_ntt_tables(log_n: int, L: int, cm0: int = 0) -> None:
    call("yell_init_ntt_tables_range", log_n, cm0, L)


def ntt_tables(log_n: int, cm: int):
    """Host copy of the reference's tables: (4, N) array and 4 scalars."""
    n = 1 << log_n
    out = np.zeros(4 * n, dtype=np.uint64)
    sc = np.zeros(4, dtype=np.uint64)
    call("yell_ntt_tables", log_n, cm, _addr(out), _addr(sc))
    return out.reshape(4, n), sc


# --- drop-ins: yell::ntt<N>::forward/forward_lazy/backward on host memory --
def _ntt1(name, x, log_n, cm):
    y = _u64(x).copy()
    if y.size != 1 << log_n:
        raise ValueError(f"limb has {y.size} words, expected {1 << log_n}")
    call(name, _addr(y), log_n, cm)
    return y


def ntt_forward(x, log_n: int, cm: int) -> np.ndarray:
    return _ntt1("yell_ntt_forward", x, log_n, cm)


def ntt_forward_lazy(x, log_n: int, cm: int) -> np.ndarray:
    return _ntt1("yell_ntt_forward_lazy", x, log_n, cm)


def ntt_backward(x, log_n: int, cm: int) -> np.ndarray:
    return _ntt1("yell_ntt_backward", x, log_n, cm)


# --- drop-ins: poly<N> members on a list of limb arrays (in place) ---------
def _limbs(limbs):
    out = []
    for a in limbs:
        if not (isinstance(a, np.ndarray) and a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]):
            raise TypeError("limbs must be C-contiguous uint64 numpy arrays")
        out.append(a)
    return out


def _log_n_of(limbs) -> int:
    n = limbs[0].size
    return n.bit_length() - 1


def poly_forward(limbs) -> None:
    ls = _limbs(limbs)
    call("yell_poly_forward", _ptr_array(ls), len(ls), _log_n_of(ls))


def poly_forward_lazy(limbs) -> None:
    ls = _limbs(limbs)
    call("yell_poly_forward_lazy", _ptr_array(ls), len(ls), _log_n_of(ls))


def poly_backward(limbs) -> None:
    ls = _limbs(limbs)
    call("yell_poly_backward", _ptr_array(ls), len(ls), _log_n_of(ls))


def _binary(name, dst, a, b):
    d, x, y = _limbs(dst), _limbs(a), _limbs(b)
    L = min(len(x), len(y))
    call(name, _ptr_array(d[:L]), _ptr_array(x[:L]), _ptr_array(y[:L]), L, _log_n_of(x))


def poly_mulmod(dst, a, b) -> None:
    _binary("yell_poly_mulmod", dst, a, b)


def poly_addmod(dst, a, b) -> None:
    _binary("yell_poly_addmod", dst, a, b)


def poly_submod(dst, a, b) -> None:
    _binary("yell_poly_submod", dst, a, b)


def poly_add_product_of(acc, a, b) -> None:
    _binary("yell_poly_add_product_of", acc, a, b)


def poly_negate(limbs) -> None:
    ls = _limbs(limbs)
    call("yell_poly_negate", _ptr_array(ls), len(ls), _log_n_of(ls))


class PinnedBuffer:
    """Page-locked host memory from yell_host_alloc, viewed as a numpy array."""

    def __init__(self, shape, dtype=np.uint64):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._ptr = load().yell_host_alloc(max(nbytes, 1))
        if not self._ptr:
            raise MemoryError(f"yell_host_alloc({nbytes}) failed")
        buf = (ctypes.c_uint8 * nbytes).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self._ptr:
            self.array = None
            load().yell_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def set_host_access(enable: bool) -> None:
    """Host-pointer calls move limbs by kernels that access host memory in place
    (where the device supports it) or, when disabled, by copies."""
    call("yell_set_host_access", 1 if enable else 0)


def host_access() -> bool:
    """Whether host-pointer calls on the current device use direct host access."""
    v = ctypes.c_int()
    call("yell_host_access", ctypes.byref(v))
    return bool(v.value)


def polymul_host(a, b, log_n: int, cm0: int = 0, out=None) -> np.ndarray:
    """Fused c = a*b mod (X^N+1) on host arrays shaped (pairs, L, N)."""
    a = _u64(a)
    b = _u64(b)
    if a.shape != b.shape or a.ndim != 3 or a.shape[2] != 1 << log_n:
        raise ValueError("a and b must both be (pairs, L, N)")
    c = np.empty_like(a) if out is None else out
    call("yell_polymul_host", _addr(c), _addr(a), _addr(b), a.shape[0], a.shape[1], log_n, cm0)
    return c


# --- device-resident calls on torch tensors ---------------------------------
def _dptr(t) -> int:
    if not t.is_cuda or not t.is_contiguous() or t.element_size() != 8:
        raise TypeError("expected a contiguous 64-bit CUDA tensor")
    return t.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        return None
    return getattr(stream, "cuda_stream", stream)


def dev_ntt(t, count: int, L: int, log_n: int, cm0: int = 0, direction: int = YELL_FORWARD,
            stream=None) -> None:
    call("yell_dev_ntt", _dptr(t), count, L, log_n, cm0, direction, _stream(stream))


def dev_ntt_limbs(limb_ptrs, cms, log_n: int, direction: int = YELL_FORWARD, stream=None) -> None:
    """limb_ptrs, cms: CUDA tensors (int64 addresses, int32 modulus indices)."""
    call("yell_dev_ntt_limbs", limb_ptrs.data_ptr(), cms.data_ptr(), limb_ptrs.numel(), log_n,
         direction, _stream(stream))


def dev_elementwise(op: int, dst, a, b, count: int, L: int, log_n: int, cm0: int = 0,
                    stream=None) -> None:
    call("yell_dev_elementwise", op, _dptr(dst), _dptr(a), _dptr(b) if b is not None else None,
         count, L, log_n, cm0, _stream(stream))


def polymul_scratch_words(pairs: int, L: int, log_n: int) -> int:
    return int(load().yell_polymul_scratch_words(pairs, L, log_n))


def dev_polymul(c, a, b, pairs: int, L: int, log_n: int, cm0: int = 0, scratch=None,
                stream=None) -> None:
    sp = _dptr(scratch) if scratch is not None else None
    sw = scratch.numel() if scratch is not None else 0
    call("yell_dev_polymul", _dptr(c), _dptr(a), _dptr(b), pairs, L, log_n, cm0, sp, sw,
         _stream(stream))


def dev_polymul_batch(items, stream=None) -> None:
    """Uneven batch: items are (c, a, b, log_n, L, cm0) with (L, N) CUDA tensors."""
    descs = (_capi.PolymulDesc * len(items))()
    for i, (c, a, b, log_n, L, cm0) in enumerate(items):
        descs[i] = _capi.PolymulDesc(_dptr(c), _dptr(a), _dptr(b), log_n, L, cm0, 0)
    call("yell_dev_polymul_batch", ctypes.addressof(descs), len(items), _stream(stream))


def dev_polymul_batch_queue(items, stream=None) -> None:
    """The uneven batch as one launch of the persistent work-queue kernel."""
    descs = (_capi.PolymulDesc * len(items))()
    for i, (c, a, b, log_n, L, cm0) in enumerate(items):
        descs[i] = _capi.PolymulDesc(_dptr(c), _dptr(a), _dptr(b), log_n, L, cm0, 0)
    call("yell_dev_polymul_batch_queue", ctypes.addressof(descs), len(items), _stream(stream))


def dev_polymul_batch_phased(items, stream=None) -> None:
    """The queue's work items as three stream-ordered launches, one per phase."""
    descs = (_capi.PolymulDesc * len(items))()
    for i, (c, a, b, log_n, L, cm0) in enumerate(items):
        descs[i] = _capi.PolymulDesc(_dptr(c), _dptr(a), _dptr(b), log_n, L, cm0, 0)
    call("yell_dev_polymul_batch_phased", ctypes.addressof(descs), len(items), _stream(stream))


def batch_queue_status() -> int:
    """Waits for queued work; returns (and clears) the queue kernel's status word."""
    st = ctypes.c_uint32()
    call("yell_batch_queue_status", ctypes.byref(st))
    return int(st.value)


def batch_queue_wait_check(timeout_s: float) -> int:
    """Runs a queue whose waits cannot be satisfied; returns the recorded status."""
    st = ctypes.c_uint32()
    call("yell_batch_queue_wait_check", int(timeout_s * 1e9), ctypes.byref(st))
    return int(st.value)


def sample_uniform(t, count: int, L: int, log_n: int, cm0: int = 0, seed: int = 0, stream=None):
    call("yell_dev_sample_uniform", _dptr(t), count, L, log_n, cm0, seed, _stream(stream))


def sample_zo(t, count: int, L: int, log_n: int, cm0: int = 0, rho: int = 0x7F, seed: int = 0,
              stream=None):
    call("yell_dev_sample_zo", _dptr(t), count, L, log_n, cm0, rho, seed, _stream(stream))


def sample_hwt(t, count: int, L: int, log_n: int, h: int, cm0: int = 0, seed: int = 0, stream=None):
    call("yell_dev_sample_hwt", _dptr(t), count, L, log_n, cm0, h, seed, _stream(stream))


def sample_gaussian(t, count: int, L: int, log_n: int, cm0: int = 0, sigma: float = 3.2,
                    tail: int = 19, amplifier: int = 1, seed: int = 0, stream=None):
    call("yell_dev_sample_gaussian", _dptr(t), count, L, log_n, cm0, sigma, tail, amplifier, seed,
         _stream(stream))


def gaussian_table(sigma: float = 3.2, tail: int = 19) -> np.ndarray:
    """The Gaussian sampler's cumulative 64-bit thresholds (2 * tail + 1)."""
    out = np.zeros(2 * tail + 1, dtype=np.uint64)
    call("yell_gaussian_table", sigma, tail, out.ctypes.data, out.size)
    return out


def crt_words(L: int, cm0: int = 0) -> int:
    """64-bit words of prod q_j over moduli cm0 .. cm0+L-1 (words per lifted coefficient)."""
    w = ctypes.c_uint32()
    call("yell_crt_words", L, cm0, ctypes.byref(w))
    return int(w.value)


def dev_crt_lift(out, t, count: int, L: int, log_n: int, cm0: int = 0, stream=None) -> None:
    """Lift count (L, N) polys to integers in [0, Q): out holds count * N * crt_words(L) words."""
    call("yell_dev_crt_lift", _dptr(out), _dptr(t), count, L, log_n, cm0, _stream(stream))


def poly_to_bigint(limbs) -> np.ndarray:
    """gmp::poly2mpz over moduli 0 .. L-1: (N, W) little-endian words per coefficient."""
    ls = _limbs(limbs)
    log_n = _log_n_of(ls)
    out = np.zeros(((1 << log_n), crt_words(len(ls))), dtype=np.uint64)
    call("yell_poly_to_bigint", _addr(out), _ptr_array(ls), len(ls), log_n)
    return out


def words_to_ints(words: np.ndarray) -> list[int]:
    """(..., W) little-endian words -> flat list of Python integers."""
    w = np.ascontiguousarray(words, dtype=np.uint64).reshape(-1, words.shape[-1])
    return [int.from_bytes(row.tobytes(), "little") for row in w]


def variants(log_n: int) -> list[str]:
    """Names of the launch variants of a degree (index = variant number)."""
    n = ctypes.c_uint32()
    call("yell_variant_count", log_n, ctypes.addressof(n))
    out = []
    for v in range(n.value):
        buf = ctypes.create_string_buffer(128)
        call("yell_variant_name", log_n, v, buf, 128)
        out.append(buf.value.decode())
    return out


def set_variant(log_n: int, v: int) -> None:
    call("yell_set_variant", log_n, v)


def get_variant(log_n: int) -> int:
    v = ctypes.c_uint32()
    call("yell_get_variant", log_n, ctypes.addressof(v))
    return v.value


def autotune(log_n: int, L: int, pairs: int) -> tuple[int, float]:
    """Times every variant of the fused polymul at this size; selects the fastest."""
    best, ms = ctypes.c_uint32(), ctypes.c_double()
    call("yell_autotune", log_n, L, pairs, ctypes.addressof(best), ctypes.addressof(ms))
    return best.value, ms.value


def calibrate_butterflies() -> tuple[float, float]:
    """Register-only butterfly rate of this GPU: (CT per s, GS per s)."""
    ct, gs = ctypes.c_double(), ctypes.c_double()
    call("yell_calibrate_butterflies", ctypes.addressof(ct), ctypes.addressof(gs))
    return ct.value, gs.value


def synchronize() -> None:
    call("yell_synchronize")


def profile_start() -> None:
    call("yell_profile_start")


def profile_stop() -> dict:
    """Stops launch profiling; returns {kernel: (launches, total_ms)}."""
    call("yell_profile_stop")
    out = {}
    lib = load()
    for i in range(lib.yell_profile_count()):
        name = ctypes.create_string_buffer(128)
        n = ctypes.c_uint64()
        ms = ctypes.c_double()
        call("yell_profile_get", i, name, 128, ctypes.addressof(n), ctypes.addressof(ms))
        out[name.value.decode()] = (int(n.value), float(ms.value))
    return out


class Poly:
    """Host polynomial mirroring yell::poly<N> (include/yell/poly.hpp:43-137):
    L limbs of N uint64 words, limb cm reduced mod prime(cm); every method
    runs on the GPU through the C ABI."""

    def __init__(self, log_n: int, L: int, limbs=None):
        self.log_n = log_n
        n = 1 << log_n
        if limbs is None:
            self.limbs = [np.zeros(n, dtype=np.uint64) for _ in range(L)]
        else:
            self.limbs = [_u64(x).copy() for x in limbs]
            assert len(self.limbs) == L and all(x.size == n for x in self.limbs)

    @property
    def moduli_count(self) -> int:
        return len(self.limbs)

    def copy(self) -> "Poly":
        return Poly(self.log_n, self.moduli_count, self.limbs)

    def forward(self) -> "Poly":
        poly_forward(self.limbs)
        return self

    def forward_lazy(self) -> "Poly":
        poly_forward_lazy(self.limbs)
        return self

    def backward(self) -> "Poly":
        poly_backward(self.limbs)
        return self

    def negate(self) -> "Poly":
        poly_negate(self.limbs)
        return self

    def add_product_of(self, a: "Poly", b: "Poly") -> "Poly":
        poly_add_product_of(self.limbs, a.limbs, b.limbs)
        return self

    def _binop(self, other, fn):
        L = min(self.moduli_count, other.moduli_count)
        out = Poly(self.log_n, L)
        fn(out.limbs, self.limbs[:L], other.limbs[:L])
        return out

    def __mul__(self, other):
        return self._binop(other, poly_mulmod)

    def __add__(self, other):
        return self._binop(other, poly_addmod)

    def __sub__(self, other):
        return self._binop(other, poly_submod)

    def __imul__(self, other):
        poly_mulmod(self.limbs, self.limbs, other.limbs)
        return self

    def __iadd__(self, other):
        poly_addmod(self.limbs, self.limbs, other.limbs)
        return self

    def __isub__(self, other):
        poly_submod(self.limbs, self.limbs, other.limbs)
        return self

    def __eq__(self, other):
        return (self.moduli_count == other.moduli_count and
                all(np.array_equal(x, y) for x, y in zip(self.limbs, other.limbs)))

    def array(self) -> np.ndarray:
        return np.stack(self.limbs)


class DevPoly:
    """A poly kept in HBM (yell_dev_poly handle): L limbs of N words, limb l
    under prime cm0 + l.  upload/download move host limbs synchronously; the
    other methods queue work on the device's library stream."""

    def __init__(self, log_n: int, L: int, cm0: int = 0, limbs=None):
        h = ctypes.c_void_p()
        call("yell_dev_poly_alloc", L, log_n, cm0, ctypes.byref(h))
        self._h = h
        self.log_n, self.L, self.cm0 = log_n, L, cm0
        if limbs is not None:
            self.upload(limbs)

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._h is None:
            raise YellError(1, "DevPoly", "poly handle already freed")
        return self._h

    def data_ptr(self) -> int:
        d = ctypes.c_void_p()
        call("yell_dev_poly_info", self.handle, ctypes.byref(d), None, None, None)
        return int(d.value)

    def upload(self, limbs) -> "DevPoly":
        ls = [_u64(x) for x in limbs]
        if len(ls) != self.L or any(x.size != 1 << self.log_n for x in ls):
            raise ValueError("limb count or size does not match the handle")
        call("yell_dev_poly_upload", self.handle, _ptr_array(ls))
        return self

    def download(self) -> np.ndarray:
        out = np.zeros((self.L, 1 << self.log_n), dtype=np.uint64)
        call("yell_dev_poly_download", self.handle, _ptr_array(list(out)))
        return out

    def forward(self) -> "DevPoly":
        call("yell_dev_poly_ntt", self.handle, YELL_FORWARD)
        return self

    def forward_lazy(self) -> "DevPoly":
        call("yell_dev_poly_ntt", self.handle, YELL_FORWARD_LAZY)
        return self

    def backward(self) -> "DevPoly":
        call("yell_dev_poly_ntt", self.handle, YELL_BACKWARD)
        return self

    def op(self, code: int, a: "DevPoly", b: "DevPoly | None" = None) -> "DevPoly":
        """self = a op b (YELL_OP_*); MULADD accumulates into self."""
        call("yell_dev_poly_op", code, self.handle, a.handle, b.handle if b is not None else None)
        return self

    def add_product_of(self, a: "DevPoly", b: "DevPoly") -> "DevPoly":
        return self.op(YELL_OP_MULADD, a, b)

    def negate(self) -> "DevPoly":
        return self.op(YELL_OP_NEGATE, self)

    def mul(self, a: "DevPoly", b: "DevPoly") -> "DevPoly":
        """self = a * b (negacyclic product of coefficient-domain polys)."""
        call("yell_dev_poly_mul", self.handle, a.handle, b.handle)
        return self

    def free(self) -> None:
        if getattr(self, "_h", None) is not None:
            call("yell_dev_poly_free", self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class BatchTicket:
    """Completion of an asynchronous yell_batch_submit."""

    def __init__(self, c, a, b):
        n = len(c)
        arr = ctypes.c_void_p * n
        t = ctypes.c_void_p()
        call("yell_batch_submit", arr(*[x.handle for x in c]), arr(*[x.handle for x in a]),
             arr(*[x.handle for x in b]), n, ctypes.byref(t))
        self._t = t
        self._keep = (c, a, b)  # the handles outlive the batch

    def wait(self, timeout_s: float = 60.0) -> None:
        if self._t is None:
            return
        call("yell_batch_wait", self._t, timeout_s)
        self._t = None
        self._keep = None

    def __del__(self):
        if getattr(self, "_t", None) is not None:
            try:
                load().yell_batch_release(self._t)
            except Exception:
                pass


def batch_submit(c, a, b) -> BatchTicket:
    return BatchTicket(list(c), list(a), list(b))
