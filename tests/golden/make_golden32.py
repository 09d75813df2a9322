"""Generates tests/golden/yell_ref32_vectors.npz from the reference itself in
its 32-bit moduli mode.

Runs the reference's own lib/{ntt,ops,math,params}.cpp compiled unmodified
with -DYELL_USE_32BITS_MODULI (oracle/_ref/libyellref32.so, built by
oracle/Makefile) on seeded inputs; sizes too large to store are kept as
SHA-256 digests of the output words.  Needs the reference checkout:

    make -C oracle ref && python tests/golden/make_golden32.py
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

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "yell_ref32_vectors.npz")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def seeded32(seed: int, n: int, bound: int) -> np.ndarray:
    """splitmix64(seed) outputs reduced mod bound, as uint32 (bound < 2^32)."""
    return (splitmix64(seed, n) % np.uint64(bound)).astype(np.uint32)


def main() -> None:
    if not oracle.ref32_available():
        sys.exit("oracle/_ref/libyellref32.so missing: run `make -C oracle ref` with the reference present")
    ref = oracle.Oracle32("ref")
    out: dict[str, np.ndarray] = {}
    digests: list[str] = []
    M = 291
    out["P"] = np.array([ref.prime(i) for i in range(M)], dtype=np.uint32)
    out["Pn"] = np.array([ref.pn(i) for i in range(M)], dtype=np.uint32)
    out["roots"] = np.array([ref.primitive_root(i) for i in range(M)], dtype=np.uint32)

    for log_n in (3, 4, 5, 8, 11):
        for cm in (0, 290):
            p = int(out["P"][cm])
            x4 = seeded32(11000 + 10 * log_n + cm, 1 << log_n, 4 * p)
            x2 = seeded32(12000 + 10 * log_n + cm, 1 << log_n, 2 * p)
            key = f"ntt_{log_n}_{cm}"
            out[key + "_x4"] = x4
            out[key + "_fwd_lazy"] = ref.forward_lazy(x4, log_n, cm)
            out[key + "_fwd"] = ref.forward(x4, log_n, cm)
            out[key + "_x2"] = x2
            out[key + "_bwd"] = ref.backward(x2, log_n, cm)

    for log_n, cm in ((12, 2), (13, 100), (14, 1), (15, 7)):
        p = int(out["P"][cm])
        x4 = seeded32(13000 + log_n, 1 << log_n, 4 * p)
        x2 = seeded32(14000 + log_n, 1 << log_n, 2 * p)
        digests.append(f"forward_lazy {log_n} {cm} {13000 + log_n} 4 {digest(ref.forward_lazy(x4, log_n, cm))}")
        digests.append(f"forward {log_n} {cm} {13000 + log_n} 4 {digest(ref.forward(x4, log_n, cm))}")
        digests.append(f"backward {log_n} {cm} {14000 + log_n} 2 {digest(ref.backward(x2, log_n, cm))}")

    t, sc = ref.tables(4, 0)
    out["tables_4_0"], out["tables_4_0_scalars"] = t, sc
    for log_n, cm in ((12, 5), (15, 290)):
        t, sc = ref.tables(log_n, cm)
        digests.append(f"tables {log_n} {cm} 0 0 {digest(np.concatenate([t.ravel(), sc]))}")

    # element-wise ops on reduced operands, products of lazy [0, 4p) words for muladd
    for cm in (0, 290):
        p = int(out["P"][cm])
        x = seeded32(15000 + cm, 512, p)
        y = seeded32(16000 + cm, 512, p)
        z = seeded32(17000 + cm, 512, p)
        x4 = seeded32(18000 + cm, 512, 4 * p)
        out[f"ew_{cm}_x"], out[f"ew_{cm}_y"], out[f"ew_{cm}_z"], out[f"ew_{cm}_x4"] = x, y, z, x4
        out[f"ew_{cm}_mulmod"] = ref.mulmod(x, y, cm)
        out[f"ew_{cm}_addmod"] = ref.addmod(x, y, cm)
        out[f"ew_{cm}_submod"] = ref.submod(x, y, cm)
        out[f"ew_{cm}_muladd"] = ref.muladd(z, x4, x4, cm)
        w = splitmix64(19000 + cm, 256)
        out[f"barrett_{cm}_x"] = w
        out[f"barrett_{cm}"] = np.array([ref.barrett(int(v) % (16 * p * p), cm) for v in w], dtype=np.uint32)

    # a polymul at N = 2^12, L = 3
    ps = [int(out["P"][l]) for l in range(3)]
    a = np.stack([seeded32(20000 + l, 4096, ps[l]) for l in range(3)])
    b = np.stack([seeded32(21000 + l, 4096, ps[l]) for l in range(3)])
    out["pm_a"], out["pm_b"], out["pm_c"] = a, b, ref.polymul(a, b, 12)

    out["digests"] = np.array(digests)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {len(out)} arrays, {len(digests)} digests, {os.path.getsize(OUT)} bytes")


if __name__ == "__main__":
    main()
