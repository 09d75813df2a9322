"""Seeded synthetic inputs for the polynomial workloads.

The reference's samplers are unseeded (Salsa20 keyed from /dev/urandom,
lib/prng/fastrandombytes.cpp:21-34), so every workload here is drawn from
splitmix64(seed) instead, and the same buffers feed the GPU path and the CPU
oracle.

Layout of a batch: (polys, L, N) uint64, limb l of every poly reduced modulo
the prime with index cm0 + l.  Element k of the flattened batch takes the
k-th splitmix64 output of the stream started at ``seed`` (the stream's first
output is splitmix64 applied once to ``seed``).
"""
from __future__ import annotations

import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Outputs offset .. offset+count-1 of the splitmix64 stream at ``seed``."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform_polys(seed: int, polys: int, L: int, log_n: int, primes, offset: int = 0) -> np.ndarray:
    """(polys, L, N) residues uniform in [0, q_l) (splitmix64 output mod q_l)."""
    n = 1 << log_n
    q = np.asarray(primes, dtype=np.uint64)[:L].reshape(1, L, 1)
    raw = splitmix64(seed, polys * L * n, offset).reshape(polys, L, n)
    return raw % q


# Discrete Gaussian by cumulative-distribution table: P(e) ~ exp(-e^2 / 2s^2)
# on |e| <= tail, with 64-bit thresholds; one splitmix64 output per sample.
def _gaussian_cdt(sigma: float, tail: int) -> np.ndarray:
    es = np.arange(-tail, tail + 1)
    w = np.exp(-(es.astype(np.float64) ** 2) / (2.0 * sigma * sigma))
    cdf = np.cumsum(w) / w.sum()
    thr = np.floor(cdf * 2.0**64)
    thr = np.minimum(thr, 2.0**64 - 1).astype(np.float64)
    out = np.array([int(t) if t < 2.0**64 else 2**64 - 1 for t in thr], dtype=np.uint64)
    out[-1] = np.uint64(2**64 - 1)
    return out


def gaussian_ints(seed: int, count: int, sigma: float = 3.2, tail_sigmas: float = 6.0,
                  offset: int = 0) -> np.ndarray:
    """Centred discrete Gaussian integers, |e| <= floor(tail_sigmas*sigma)."""
    tail = int(math.floor(tail_sigmas * sigma))
    cdt = _gaussian_cdt(sigma, tail)
    u = splitmix64(seed, count, offset)
    idx = np.searchsorted(cdt, u, side="right")
    idx = np.minimum(idx, 2 * tail)
    return idx.astype(np.int64) - tail


def gaussian_polys(seed: int, polys: int, L: int, log_n: int, primes, sigma: float = 3.2,
                   tail_sigmas: float = 6.0, offset: int = 0) -> np.ndarray:
    """(polys, L, N): one integer Gaussian poly per entry, reduced mod each q_l
    the way the reference maps signed noise, r < 0 ? p + r : r
    (include/yell/details/poly.hpp:252-257)."""
    n = 1 << log_n
    e = gaussian_ints(seed, polys * n, sigma, tail_sigmas, offset).reshape(polys, 1, n)
    q = np.asarray(primes, dtype=np.uint64)[:L].reshape(1, L, 1)
    pos = np.broadcast_to(e, (polys, L, n))
    out = np.where(pos < 0, q - np.abs(pos).astype(np.uint64), pos.astype(np.uint64))
    return np.ascontiguousarray(out.astype(np.uint64))
