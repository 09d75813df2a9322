"""Generates prime_table.inc: the 62-bit NTT prime table of the library.

The table is the one YELL's params use (include/yell/params_64.hpp:16-38), and
it has to be identical for the NTT outputs to match bit for bit.  It is not
copied: it is regenerated from the rule that header states.
  * P[k]  = the k-th value of 2^62 - i * 2^21 + 1 (i = 1, 2, ...) that is prime
  * Pn[k] = the low 64 bits of floor(2^128 / P[k])
  * root[k] = g^((P[k] - 1) / 2^21) mod P[k], g the least primitive root of
    P[k]: a primitive 2^21-th root of unity (2 * kMaxPolyDegree).
Run:  python yell_gb300/csrc/gen_prime_table.py > yell_gb300/csrc/prime_table.inc
"""
from __future__ import annotations

import sys

import numpy as np

MAX_MODULI = 1000
LOG_ROOT_ORDER = 21


def is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 2^64."""
    if n < 2:
        return False
    bases = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)
    for b in bases:
        if n % b == 0:
            return n == b
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for b in bases:
        x = pow(b, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def odd_prime_factors(m: int) -> list[int]:
    """Distinct odd prime factors of m (m < 2^42) by vectorised trial division."""
    while m % 2 == 0:
        m //= 2
    out = []
    limit = int(m ** 0.5) + 2
    cand = np.arange(3, limit + 1, 2, dtype=np.int64)
    hits = cand[(np.int64(m) % cand) == 0]
    for f in hits.tolist():
        if m % f == 0:
            out.append(f)
            while m % f == 0:
                m //= f
    if m > 1:
        out.append(m)
    return out


def least_primitive_root(p: int) -> int:
    factors = [2] + odd_prime_factors(p - 1)
    g = 2
    while any(pow(g, (p - 1) // f, p) == 1 for f in factors):
        g += 1
    return g


def generate(count: int = MAX_MODULI):
    primes, i = [], 1
    while len(primes) < count:
        p = (1 << 62) - i * (1 << LOG_ROOT_ORDER) + 1
        if is_prime(p):
            primes.append(p)
        i += 1
    pn = [((1 << 128) // p) & ((1 << 64) - 1) for p in primes]
    roots = [pow(least_primitive_root(p), (p - 1) >> LOG_ROOT_ORDER, p) for p in primes]
    return primes, pn, roots


def render(primes, pn, roots) -> str:
    lines = ["// Generated by gen_prime_table.py; do not edit.",
             "// {P, Pn, primitive 2^21-th root} per modulus index cm."]
    for p, n, r in zip(primes, pn, roots):
        lines.append(f"{{{p}ULL, {n}ULL, {r}ULL}},")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    sys.stdout.write(render(*generate()))
