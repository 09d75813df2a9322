"""Big-integer CRT lifting oracle (test infrastructure only).

Pure-Python restatement of the reference's ``gmp::poly2mpz``
(fionser/YELL include/yell/gmp.hpp:42-70) and its tables
(lib/gmp.cpp:6-51), step for step with Python integers in place of mpz_t:

* moduli_product Q = prod P[j]                                (gmp.cpp:10-14)
* shift = bits(Q) + 62 + floor(log2 L) + 1, modulus_shoup = floor(2^shift / Q)
                                                              (gmp.cpp:16-26)
* lifting_integers[j] = ((Q/P[j])^-1 mod P[j]) * (Q/P[j])    (gmp.cpp:32-46)
* per coefficient: rop = sum_j lifting_integers[j] * op(j, i);
  tmp = (rop * modulus_shoup) >> shift; rop -= tmp * Q; rop -= Q if rop >= Q
                                                              (gmp.hpp:55-66)
"""
from __future__ import annotations

import math

import numpy as np

K_MODULUS_BITS = 62  # params::kModulusRepresentationBitsize, params_64.hpp:23


class CrtTable:
    def __init__(self, primes):
        self.primes = [int(p) for p in primes]
        L = len(self.primes)
        Q = 1
        for p in self.primes:
            Q *= p
        self.Q = Q
        self.bits = Q.bit_length()
        self.shift = self.bits + K_MODULUS_BITS + int(math.log2(L)) + 1
        self.shoup = (1 << self.shift) // Q
        self.lift = []
        for p in self.primes:
            quot = Q // p
            self.lift.append(pow(quot, -1, p) * quot)

    def lift_coeff(self, residues) -> int:
        rop = 0
        for j, r in enumerate(residues):
            r = int(r)
            if r:
                rop += self.lift[j] * r
        tmp = (rop * self.shoup) >> self.shift
        rop -= tmp * self.Q
        if rop >= self.Q:
            rop -= self.Q
        return rop

    def words(self) -> int:
        return (self.bits + 63) // 64


def poly2bigint(limbs: np.ndarray, primes) -> list[int]:
    """limbs: (L, N) residues -> N Python integers (the reference's poly2mpz)."""
    t = CrtTable(primes)
    L, n = limbs.shape
    cols = [[int(v) for v in limbs[j]] for j in range(L)]
    return [t.lift_coeff([cols[j][i] for j in range(L)]) for i in range(n)]


def to_words(values, W: int) -> np.ndarray:
    """Python integers -> (len, W) little-endian uint64 words."""
    out = np.zeros((len(values), W), dtype=np.uint64)
    mask = (1 << 64) - 1
    for i, v in enumerate(values):
        for w in range(W):
            out[i, w] = (v >> (64 * w)) & mask
    return out
