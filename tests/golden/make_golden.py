"""Generates tests/golden/yell_ref_vectors.npz from the reference itself.

Runs the reference's own lib/{ntt,ops,math,params}.cpp (compiled unmodified
into oracle/_ref/libyellref.so by oracle/Makefile) on seeded inputs and
stores inputs and outputs; sizes too large to store are kept as SHA-256
digests of the output words.  Needs the reference checkout, so it runs only
where that exists:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from yell_gb300.inputs import splitmix64  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "yell_ref_vectors.npz")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def seeded(seed: int, n: int, bound: int) -> np.ndarray:
    """splitmix64(seed) outputs reduced mod bound (bound < 2^64)."""
    return splitmix64(seed, n) % np.uint64(bound)


def main() -> None:
    if not oracle.ref_available():
        sys.exit("oracle/_ref/libyellref.so missing: run `make -C oracle ref` with the reference present")
    ref = oracle.Oracle("ref")
    out: dict[str, np.ndarray] = {}
    digests: list[str] = []

    # params_64.hpp tables, all 1000 entries
    out["P"] = np.array([ref.prime(i) for i in range(1000)], dtype=np.uint64)
    out["Pn"] = np.array([ref.pn(i) for i in range(1000)], dtype=np.uint64)
    out["roots"] = np.array([ref.primitive_root(i) for i in range(1000)], dtype=np.uint64)

    # config 1: N = 1024, L = 1, q = P[0], seed 1
    p0 = int(out["P"][0])
    a = splitmix64(1, 1024) % np.uint64(p0)
    b = splitmix64(1, 1024, offset=1024) % np.uint64(p0)
    fa = ref.forward(a, 10, 0)
    fb = ref.forward(b, 10, 0)
    prod = ref.mulmod(fa, fb, 0)
    out.update(cfg1_a=a, cfg1_b=b, cfg1_fwd_a=fa, cfg1_fwd_b=fb,
               cfg1_fwd_lazy_a=ref.forward_lazy(a, 10, 0), cfg1_prod=prod,
               cfg1_c=ref.backward(prod, 10, 0))

    # small NTTs at both ends of the prime table
    for log_n in (3, 4, 5, 8, 11):
        for cm in (0, 999):
            p = int(out["P"][cm])
            x4 = seeded(1000 + 10 * log_n + cm, 1 << log_n, 4 * p)
            x2 = seeded(2000 + 10 * log_n + cm, 1 << log_n, 2 * p)
            key = f"ntt_{log_n}_{cm}"
            out[key + "_x4"] = x4
            out[key + "_fwd_lazy"] = ref.forward_lazy(x4, log_n, cm)
            out[key + "_fwd"] = ref.forward(x4, log_n, cm)
            out[key + "_x2"] = x2
            out[key + "_bwd"] = ref.backward(x2, log_n, cm)

    # digests of larger transforms: (log_n, cm, op, seed, bound multiple)
    for log_n, cm in ((13, 2), (14, 1), (15, 7), (16, 31), (17, 3), (18, 4), (19, 9), (20, 0)):
        p = int(out["P"][cm])
        x4 = seeded(3000 + log_n, 1 << log_n, 4 * p)
        x2 = seeded(4000 + log_n, 1 << log_n, 2 * p)
        digests.append(f"forward_lazy {log_n} {cm} {3000 + log_n} 4 {digest(ref.forward_lazy(x4, log_n, cm))}")
        digests.append(f"forward {log_n} {cm} {3000 + log_n} 4 {digest(ref.forward(x4, log_n, cm))}")
        digests.append(f"backward {log_n} {cm} {4000 + log_n} 2 {digest(ref.backward(x2, log_n, cm))}")

    # twiddle tables (include/yell/details/ntt.hpp:97-146)
    t, sc = ref.tables(4, 0)
    out["tables_4_0"] = t
    out["tables_4_0_scalars"] = sc
    for log_n, cm in ((12, 5), (16, 31)):
        t, sc = ref.tables(log_n, cm)
        digests.append(f"tables {log_n} {cm} 0 0 {digest(np.concatenate([t.ravel(), sc]))}")

    # element-wise ops on full-range words (the formulas wrap like the reference)
    for cm in (0, 999):
        x = splitmix64(5000 + cm, 512)
        y = splitmix64(6000 + cm, 512)
        z = splitmix64(7000 + cm, 512)
        out[f"ew_{cm}_x"], out[f"ew_{cm}_y"], out[f"ew_{cm}_z"] = x, y, z
        out[f"ew_{cm}_mulmod"] = ref.mulmod(x, y, cm)
        out[f"ew_{cm}_addmod"] = ref.addmod(x, y, cm)
        out[f"ew_{cm}_submod"] = ref.submod(x, y, cm)
        out[f"ew_{cm}_muladd"] = ref.muladd(z, x, y, cm)
        out[f"ew_{cm}_mulmod_shoup"] = ref.mulmod_shoup(x, int(y[0]) % int(out['P'][cm]), cm)

    out["digests"] = np.array(digests)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(out)} arrays, {len(digests)} digests, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
