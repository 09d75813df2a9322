"""CPU oracle for the YELL RNS-polynomial hot path (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker.  The product
(``yell_gb300``) never imports it and has no CPU fallback.

Two CPU implementations are exposed through ctypes:

* ``port``: ``liboracle.so``, the plain-C restatement in ``yell_oracle.c`` of
  the reference algorithm (fionser/YELL ``lib/ntt.cpp``, ``lib/ops.cpp``,
  ``include/yell/details/ntt.hpp``), built by ``oracle/Makefile``.
  ``samplers_oracle.c`` restates the reference's sampler rules
  (``include/yell/details/poly.hpp:195-330``) over the seeded counter stream.
  ``yell_oracle32.c`` restates the reference's 32-bit moduli mode
  (``-DYELL_USE_32BITS_MODULI``, ``include/yell/params_32.hpp``).
* ``crt.py``: pure-Python big-integer restatement of ``gmp::poly2mpz``
  (``include/yell/gmp.hpp:42-70``, ``lib/gmp.cpp:6-51``).
* ``Oracle32``: the 32-bit mode, ``port`` from ``liboracle.so`` or ``ref``
  from ``_ref/libyellref32.so`` (the reference's sources compiled in that mode).
* ``ref``: ``_ref/libyellref.so``, the reference's own sources compiled
  unmodified with ``ref_harness.cpp``; present only where the reference
  checkout was available to build it (``ref_available()``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U32P = ctypes.POINTER(ctypes.c_uint32)
_port = None
_ref = None


def build(ref_dir: str | None = None) -> None:
    """Compile liboracle.so (and _ref/libyellref.so when the reference exists)."""
    cmd = ["make", "-s", "-C", _HERE, "oracle"]
    subprocess.run(cmd, check=True)
    ref = ref_dir or os.environ.get("YELL_REFERENCE_DIR", "/root/reference")
    if os.path.isdir(os.path.join(ref, "lib")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={ref}"], check=True)
        subprocess.run(["make", "-s", "-C", _HERE, "ref_samplers", f"REF={ref}"], check=True)


def _bind(lib, prefix: str):
    u32, u64, sz = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
    sig = {
        "prime": (u64, [u32]),
        "pn": (u64, [u32]),
        "primitive_root": (u64, [u32]),
        "forward": (ctypes.c_int, [_U64P, u32, u32]),
        "forward_lazy": (ctypes.c_int, [_U64P, u32, u32]),
        "backward": (ctypes.c_int, [_U64P, u32, u32]),
        "ntt_tables": (ctypes.c_int, [u32, u32, _U64P, _U64P]),
        "barrett": (u64, [u64, u64, u32]),
        "shoupify": (u64, [u64, u32]),
        "mulmod_n": (None, [_U64P, _U64P, _U64P, sz, u32]),
        "addmod_n": (None, [_U64P, _U64P, _U64P, sz, u32]),
        "submod_n": (None, [_U64P, _U64P, _U64P, sz, u32]),
        "muladd_n": (None, [_U64P, _U64P, _U64P, sz, u32]),
        "mulmod_shoup_n": (None, [_U64P, _U64P, u64, sz, u32]),
        "negacyclic_forward_lazy": (ctypes.c_int, [_U64P, u64, _U64P, _U64P, u64]),
        "negacyclic_backward_lazy": (ctypes.c_int, [_U64P, u64, _U64P, _U64P, u64]),
    }
    if prefix == "orc_":
        sig.update({
            "negate_n": (None, [_U64P, sz, u32]),
            "negacyclic_schoolbook": (ctypes.c_int, [_U64P, _U64P, _U64P, u32, u32]),
            "polymul": (ctypes.c_int, [_U64P, _U64P, _U64P, u32, u32, u32]),
            "polymul_batch": (ctypes.c_double, [_U64P, _U64P, _U64P, u32, u32, u32, u32, u32]),
            "sample_uniform": (None, [_U64P, u32, u32, u32, u32, u64]),
            "32_prime": (u32, [u32]),
            "32_pn": (u32, [u32]),
            "32_primitive_root": (u32, [u32]),
            "32_ntt_tables": (ctypes.c_int, [u32, u32, _U32P, _U32P]),
            "32_forward": (ctypes.c_int, [_U32P, u32, u32]),
            "32_forward_lazy": (ctypes.c_int, [_U32P, u32, u32]),
            "32_backward": (ctypes.c_int, [_U32P, u32, u32]),
            "32_barrett": (u32, [u64, u32]),
            "32_mulmod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "32_addmod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "32_submod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "32_muladd_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "32_negate_n": (None, [_U32P, sz, u32]),
            "32_polymul": (ctypes.c_int, [_U32P, _U32P, _U32P, u32, u32, u32]),
            "sample_zo": (None, [_U64P, u32, u32, u32, u32, u32, u64]),
            "sample_hwt": (ctypes.c_int, [_U64P, u32, u32, u32, u32, u32, u64]),
            "gaussian_cdt": (u32, [ctypes.c_double, u32, _U64P]),
            "sample_gaussian": (None, [_U64P, u32, u32, u32, u32, _U64P, u32, u32, u64, u64]),
        })
    else:
        sig["polymul_batch"] = (ctypes.c_double, [_U64P, _U64P, _U64P, u32, u32, u32, u32])
    for name, (res, args) in sig.items():
        # "32_x" entries are the 32-bit mode's orc32_x functions
        fn = getattr(lib, (prefix[:-1] + name) if name.startswith("32_") else prefix + name)
        fn.restype = res
        fn.argtypes = args
    return lib


def _load_port():
    global _port
    if _port is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _port = _bind(ctypes.CDLL(path), "orc_")
    return _port


def ref_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libyellref.so"))


def _load_ref():
    global _ref
    if _ref is None:
        _ref = _bind(ctypes.CDLL(os.path.join(_HERE, "_ref", "libyellref.so")), "ref_")
    return _ref


def _ptr(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_U64P)


class Oracle:
    """numpy-facing wrapper; ``which`` is "port" (the C restatement) or "ref"."""

    def __init__(self, which: str = "port"):
        self.which = which
        self.lib = _load_port() if which == "port" else _load_ref()
        self.pre = "orc_" if which == "port" else "ref_"

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    # --- params ---------------------------------------------------------
    def prime(self, cm: int) -> int:
        return int(self._f("prime")(cm))

    def pn(self, cm: int) -> int:
        return int(self._f("pn")(cm))

    def primitive_root(self, cm: int) -> int:
        return int(self._f("primitive_root")(cm))

    def primes(self, L: int, cm0: int = 0) -> np.ndarray:
        return np.array([self.prime(cm0 + i) for i in range(L)], dtype=np.uint64)

    # --- NTT on one limb (in place on a copy) ----------------------------
    def _ntt(self, name, x, log_n, cm):
        y = np.ascontiguousarray(x, dtype=np.uint64).copy()
        assert y.size == 1 << log_n
        rc = self._f(name)(_ptr(y), log_n, cm)
        if rc != 0:
            raise ValueError(f"oracle {name}: bad arguments log_n={log_n} cm={cm}")
        return y

    def forward(self, x, log_n, cm):
        return self._ntt("forward", x, log_n, cm)

    def forward_lazy(self, x, log_n, cm):
        return self._ntt("forward_lazy", x, log_n, cm)

    def backward(self, x, log_n, cm):
        return self._ntt("backward", x, log_n, cm)

    def tables(self, log_n, cm):
        n = 1 << log_n
        out = np.zeros(4 * n, dtype=np.uint64)
        sc = np.zeros(4, dtype=np.uint64)
        rc = self._f("ntt_tables")(log_n, cm, _ptr(out), _ptr(sc))
        if rc != 0:
            raise ValueError("oracle tables: bad arguments")
        return out.reshape(4, n), sc

    # --- whole-poly helpers: x has shape (L, N), limb l uses prime cm0+l --
    def poly_forward(self, x, log_n, cm0=0, lazy=False):
        x = np.asarray(x, dtype=np.uint64).reshape(-1, 1 << log_n)
        f = self.forward_lazy if lazy else self.forward
        return np.stack([f(x[i], log_n, cm0 + i) for i in range(x.shape[0])])

    def poly_backward(self, x, log_n, cm0=0):
        x = np.asarray(x, dtype=np.uint64).reshape(-1, 1 << log_n)
        return np.stack([self.backward(x[i], log_n, cm0 + i) for i in range(x.shape[0])])

    # --- element-wise ops on one limb -------------------------------------
    def _ew(self, name, a, b, cm):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        d = np.zeros_like(a)
        self._f(name)(_ptr(d), _ptr(a), _ptr(b), a.size, cm)
        return d

    def negacyclic_lazy(self, x, w, ws, p, inverse=False):
        """The free functions with caller tables (details/ntt.hpp:10-23)."""
        a = np.ascontiguousarray(x, dtype=np.uint64).copy()
        w = np.ascontiguousarray(w, dtype=np.uint64)
        ws = np.ascontiguousarray(ws, dtype=np.uint64)
        fn = self._f("negacyclic_backward_lazy" if inverse else "negacyclic_forward_lazy")
        if fn(_ptr(a), a.size, _ptr(w), _ptr(ws), p) != 0:
            raise ValueError("negacyclic_lazy: bad arguments")
        return a

    def mulmod(self, a, b, cm):
        return self._ew("mulmod_n", a, b, cm)

    def addmod(self, a, b, cm):
        return self._ew("addmod_n", a, b, cm)

    def submod(self, a, b, cm):
        return self._ew("submod_n", a, b, cm)

    def muladd(self, rop, a, b, cm):
        r = np.ascontiguousarray(rop, dtype=np.uint64).copy()
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        self._f("muladd_n")(_ptr(r), _ptr(a), _ptr(b), a.size, cm)
        return r

    def mulmod_shoup(self, a, y, cm):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        d = np.zeros_like(a)
        self._f("mulmod_shoup_n")(_ptr(d), _ptr(a), int(y), a.size, cm)
        return d

    def negate(self, a, cm):
        assert self.which == "port"
        r = np.ascontiguousarray(a, dtype=np.uint64).copy()
        self.lib.orc_negate_n(_ptr(r), r.size, cm)
        return r

    def barrett(self, x: int, cm: int) -> int:
        return int(self._f("barrett")((x >> 64) & (2**64 - 1), x & (2**64 - 1), cm))

    def shoupify(self, x: int, cm: int) -> int:
        return int(self._f("shoupify")(x, cm))

    # --- polymul ------------------------------------------------------------
    def schoolbook(self, a, b, log_n, cm):
        assert self.which == "port"
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        c = np.zeros_like(a)
        if self.lib.orc_negacyclic_schoolbook(_ptr(c), _ptr(a), _ptr(b), log_n, cm) != 0:
            raise ValueError("schoolbook: log_n must be <= 13")
        return c

    def polymul(self, a, b, log_n, cm0=0):
        """Reference-style polymul on (L, N) polys: forward, mulmod, backward."""
        n = 1 << log_n
        a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, n)
        b = np.ascontiguousarray(b, dtype=np.uint64).reshape(-1, n)
        if self.which == "port":
            c = np.zeros_like(a)
            rc = self.lib.orc_polymul(_ptr(c), _ptr(a), _ptr(b), a.shape[0], log_n, cm0)
            if rc != 0:
                raise ValueError("polymul: bad arguments")
            return c
        out = []
        for i in range(a.shape[0]):
            fa = self.forward(a[i], log_n, cm0 + i)
            fb = self.forward(b[i], log_n, cm0 + i)
            out.append(self.backward(self.mulmod(fa, fb, cm0 + i), log_n, cm0 + i))
        return np.stack(out)

    def polymul_batch(self, a, b, pairs, L, log_n, threads):
        """Batch of `pairs` polymuls laid out (pairs, L, N); returns (c, seconds)."""
        n = 1 << log_n
        a = np.ascontiguousarray(a, dtype=np.uint64).reshape(pairs, L, n)
        b = np.ascontiguousarray(b, dtype=np.uint64).reshape(pairs, L, n)
        c = np.zeros_like(a)
        if self.which == "port":
            t = self.lib.orc_polymul_batch(_ptr(c), _ptr(a), _ptr(b), pairs, L, log_n, 0, threads)
        else:
            t = self.lib.ref_polymul_batch(_ptr(c), _ptr(a), _ptr(b), pairs, L, log_n, threads)
        if t < 0:
            raise ValueError("polymul_batch: bad arguments")
        return c, float(t)

    # --- samplers (port only) ------------------------------------------------
    def _polys(self, count, L, log_n):
        return np.zeros((count, L, 1 << log_n), dtype=np.uint64)

    def sample_uniform(self, count, L, log_n, cm0=0, seed=0):
        out = self._polys(count, L, log_n)
        self.lib.orc_sample_uniform(_ptr(out), count, L, log_n, cm0, seed)
        return out

    def sample_zo(self, count, L, log_n, cm0=0, rho=0x7F, seed=0):
        out = self._polys(count, L, log_n)
        self.lib.orc_sample_zo(_ptr(out), count, L, log_n, cm0, rho, seed)
        return out

    def sample_hwt(self, count, L, log_n, h, cm0=0, seed=0):
        out = self._polys(count, L, log_n)
        if self.lib.orc_sample_hwt(_ptr(out), count, L, log_n, cm0, h, seed) != 0:
            raise ValueError("sample_hwt: bad arguments")
        return out

    def gaussian_cdt(self, sigma, tail):
        out = np.zeros(2 * tail + 1, dtype=np.uint64)
        m = self.lib.orc_gaussian_cdt(sigma, tail, _ptr(out))
        return out[:m]

    def sample_gaussian(self, count, L, log_n, cm0=0, sigma=3.2, tail=19, amplifier=1, seed=0):
        cdt = self.gaussian_cdt(sigma, tail)
        out = self._polys(count, L, log_n)
        self.lib.orc_sample_gaussian(_ptr(out), count, L, log_n, cm0, _ptr(cdt), len(cdt), tail,
                                     amplifier, seed)
        return out


def ref_samplers_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libyellref_samplers.so"))


class RefSamplers:
    """The reference's own samplers, Gaussian sampler and CRT lifting
    (yell/poly.hpp set(...), FastGaussianNoise, gmp::poly2mpz) run on the
    counter stream by ref_samplers_harness.cpp; only where it was built."""

    def __init__(self):
        lib = ctypes.CDLL(os.path.join(_HERE, "_ref", "libyellref_samplers.so"))
        u32, u64, i = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        for name, args in (("refs_sample_uniform", [_U64P, u32, u32, u32, u64]),
                           ("refs_sample_zo", [_U64P, u32, u32, u32, u32, u64]),
                           ("refs_sample_hwt", [_U64P, u32, u32, u32, u32, u64]),
                           ("refs_poly2mpz", [_U64P, _U64P, u32, u32, u32]),
                           ("refs_gaussian_barriers", [ctypes.c_double, u32, u32, _U32P, _U64P, u32]),
                           ("refs_gaussian_sample", [ctypes.c_double, u32, u32, u64,
                                                     ctypes.POINTER(ctypes.c_int64), u64])):
            fn = getattr(lib, name)
            fn.restype = i
            fn.argtypes = args
        self.lib = lib

    def _polys(self, count, L, log_n):
        return np.zeros((count, L, 1 << log_n), dtype=np.uint64)

    def sample_uniform(self, count, L, log_n, seed):
        out = self._polys(count, L, log_n)
        assert self.lib.refs_sample_uniform(_ptr(out), count, L, log_n, seed) == 0
        return out

    def sample_zo(self, count, L, log_n, rho, seed):
        out = self._polys(count, L, log_n)
        assert self.lib.refs_sample_zo(_ptr(out), count, L, log_n, rho, seed) == 0
        return out

    def sample_hwt(self, count, L, log_n, h, seed):
        out = self._polys(count, L, log_n)
        assert self.lib.refs_sample_hwt(_ptr(out), count, L, log_n, h, seed) == 0
        return out

    def poly2mpz(self, limbs, log_n, W):
        """limbs: (L, N) residues of moduli 0..L-1 -> (N, W) little-endian words."""
        limbs = np.ascontiguousarray(limbs, dtype=np.uint64)
        out = np.zeros((1 << log_n, W), dtype=np.uint64)
        rc = self.lib.refs_poly2mpz(_ptr(out), _ptr(limbs), limbs.shape[0], log_n, W)
        if rc != 0:
            raise ValueError(f"poly2mpz: {rc}")
        return out

    def gaussian_barriers(self, sigma=3.2, security=128, samples=1 << 14):
        """(top 64 bits of each barrier, (barriers, bit precision, words))."""
        info = (ctypes.c_uint32 * 3)()
        top = np.zeros(4096, dtype=np.uint64)
        assert self.lib.refs_gaussian_barriers(sigma, security, samples, info, _ptr(top), top.size) == 0
        return top[:info[0]].copy(), tuple(info)

    def gaussian_sample(self, n, seed, sigma=3.2, security=128, samples=1 << 14):
        out = np.zeros(n, dtype=np.int64)
        assert self.lib.refs_gaussian_sample(sigma, security, samples, seed,
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n) == 0
        return out


def ref32_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libyellref32.so"))


def _ptr32(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_U32P)


_ref32 = None


def _load_ref32():
    global _ref32
    if _ref32 is None:
        lib = ctypes.CDLL(os.path.join(_HERE, "_ref", "libyellref32.so"))
        u32, u64, sz = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
        sig = {
            "prime": (u32, [u32]), "pn": (u32, [u32]), "primitive_root": (u32, [u32]),
            "ntt_tables": (ctypes.c_int, [u32, u32, _U32P, _U32P]),
            "forward": (ctypes.c_int, [_U32P, u32, u32]),
            "forward_lazy": (ctypes.c_int, [_U32P, u32, u32]),
            "backward": (ctypes.c_int, [_U32P, u32, u32]),
            "barrett": (u32, [u64, u32]),
            "mulmod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "addmod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "submod_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "muladd_n": (None, [_U32P, _U32P, _U32P, sz, u32]),
            "polymul_batch": (ctypes.c_double, [_U32P, _U32P, _U32P, u32, u32, u32, u32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, "ref32_" + name)
            fn.restype = res
            fn.argtypes = args
        _ref32 = lib
    return _ref32


class Oracle32:
    """32-bit moduli mode; ``which`` is "port" (yell_oracle32.c) or "ref"."""

    def __init__(self, which: str = "port"):
        self.which = which
        if which == "port":
            self.lib, self.pre = _load_port(), "orc32_"
        else:
            self.lib, self.pre = _load_ref32(), "ref32_"

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def prime(self, cm):
        return int(self._f("prime")(cm))

    def pn(self, cm):
        return int(self._f("pn")(cm))

    def primitive_root(self, cm):
        return int(self._f("primitive_root")(cm))

    def _ntt(self, name, x, log_n, cm):
        a = np.ascontiguousarray(x, dtype=np.uint32).copy()
        if self._f(name)(_ptr32(a), log_n, cm) != 0:
            raise ValueError(f"{name}: bad arguments")
        return a

    def forward(self, x, log_n, cm):
        return self._ntt("forward", x, log_n, cm)

    def forward_lazy(self, x, log_n, cm):
        return self._ntt("forward_lazy", x, log_n, cm)

    def backward(self, x, log_n, cm):
        return self._ntt("backward", x, log_n, cm)

    def tables(self, log_n, cm):
        n = 1 << log_n
        out = np.zeros(4 * n, dtype=np.uint32)
        sc = np.zeros(4, dtype=np.uint32)
        if self._f("ntt_tables")(log_n, cm, _ptr32(out), _ptr32(sc)) != 0:
            raise ValueError("ntt_tables: bad arguments")
        return out.reshape(4, n), sc

    def barrett(self, x, cm):
        return int(self._f("barrett")(x, cm))

    def _ew(self, name, a, b, cm):
        a = np.ascontiguousarray(a, dtype=np.uint32)
        b = np.ascontiguousarray(b, dtype=np.uint32)
        d = np.zeros_like(a)
        self._f(name)(_ptr32(d), _ptr32(a), _ptr32(b), a.size, cm)
        return d

    def mulmod(self, a, b, cm):
        return self._ew("mulmod_n", a, b, cm)

    def addmod(self, a, b, cm):
        return self._ew("addmod_n", a, b, cm)

    def submod(self, a, b, cm):
        return self._ew("submod_n", a, b, cm)

    def muladd(self, rop, a, b, cm):
        r = np.ascontiguousarray(rop, dtype=np.uint32).copy()
        a = np.ascontiguousarray(a, dtype=np.uint32)
        b = np.ascontiguousarray(b, dtype=np.uint32)
        self._f("muladd_n")(_ptr32(r), _ptr32(a), _ptr32(b), r.size, cm)
        return r

    def negate(self, a, cm):
        assert self.which == "port"
        r = np.ascontiguousarray(a, dtype=np.uint32).copy()
        self.lib.orc32_negate_n(_ptr32(r), r.size, cm)
        return r

    def polymul(self, a, b, log_n, cm0=0):
        """(L, N) polys, limb l under cm0 + l."""
        n = 1 << log_n
        a = np.ascontiguousarray(a, dtype=np.uint32).reshape(-1, n)
        b = np.ascontiguousarray(b, dtype=np.uint32).reshape(-1, n)
        if self.which == "port":
            c = np.zeros_like(a)
            if self.lib.orc32_polymul(_ptr32(c), _ptr32(a), _ptr32(b), a.shape[0], log_n, cm0) != 0:
                raise ValueError("polymul: bad arguments")
            return c
        out = []
        for l in range(a.shape[0]):
            fa, fb = self.forward(a[l], log_n, cm0 + l), self.forward(b[l], log_n, cm0 + l)
            out.append(self.backward(self.mulmod(fa, fb, cm0 + l), log_n, cm0 + l))
        return np.stack(out)
