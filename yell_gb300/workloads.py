"""Seeded polymul request mixes.

The uneven mix (512 polymuls, log2 N uniform in 10..16, L uniform in
1..16) is drawn from splitmix64(seed): entry i takes outputs 2i and 2i+1 of
the stream, log2 N = lo + out(2i) mod (hi - lo + 1), L = 1 + out(2i+1) mod
max_L.  Operand words are drawn afterwards, per entry, from the same seed at
a fixed offset so the mix and the data are reproducible independently.
"""
from __future__ import annotations

import numpy as np

from .inputs import splitmix64, uniform_polys


def uneven_mix(seed: int = 4, count: int = 512, lo: int = 10, hi: int = 16, max_L: int = 16):
    u = splitmix64(seed, 2 * count)
    log_ns = (lo + (u[0::2] % np.uint64(hi - lo + 1))).astype(int)
    Ls = (1 + (u[1::2] % np.uint64(max_L))).astype(int)
    return list(zip(log_ns.tolist(), Ls.tolist()))


def mix_operands(mix, primes, seed: int = 4):
    """Per entry (a, b) as (L, N) uint64 arrays with residues uniform mod P[l]."""
    out = []
    base = 1 << 40
    for i, (log_n, L) in enumerate(mix):
        a = uniform_polys(seed, 1, L, log_n, primes, offset=base + (2 * i) * (1 << 24))[0]
        b = uniform_polys(seed, 1, L, log_n, primes, offset=base + (2 * i + 1) * (1 << 24))[0]
        out.append((a, b))
    return out


def mix_limb_ntts(mix) -> int:
    """Limb-NTTs of a polymul mix: NTT(a), NTT(b), INTT(c) per limb."""
    return sum(3 * L for _, L in mix)
