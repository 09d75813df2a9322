"""Generates tests/golden/yell_ref_samplers.npz from the reference itself.

Runs the reference's own samplers (yell::poly<N>::set(uniform / ZO_dist /
hwt_dist), include/yell/details/poly.hpp:195-330), its Gaussian sampler
(FastGaussianNoise<uint16_t, uint64_t, 2>, include/yell/prng/
FastGaussianNoise.hpp, as example.cpp:7-9 instantiates it) and its CRT
lifting (gmp::poly2mpz, include/yell/gmp.hpp:42-70 with lib/gmp.cpp:6-51),
compiled unmodified into oracle/_ref/libyellref_samplers.so by oracle/Makefile
with yell::fastrandombytes defined as the library's counter stream
(oracle/ref_samplers_harness.cpp).  Needs the reference checkout and the GMP /
MPFR runtimes, so it runs only where those exist:

    make -C oracle ref_samplers && python tests/golden/make_golden_samplers.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from yell_gb300.inputs import splitmix64  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "yell_ref_samplers.npz")

# (count, L, log_n, seed) per case
UNIFORM = [(3, 4, 10, 77), (2, 2, 3, 5), (1, 3, 12, 9)]
ZO = [(2, 3, 10, 0x7F, 21), (2, 2, 10, 0, 22), (2, 2, 10, 0xFF, 23), (1, 2, 3, 0x7F, 24), (1, 2, 12, 5, 25)]
HWT = [(3, 2, 10, 1, 31), (3, 2, 10, 64, 32), (2, 2, 10, 512, 33), (2, 2, 10, 1024, 34), (2, 2, 3, 1, 35),
       (2, 2, 3, 4, 36), (2, 2, 3, 8, 37), (1, 2, 12, 192, 38), (1, 1, 14, 64, 39)]
GAUSS = [(3.2, 128, 1 << 14), (3.2, 80, 1 << 10), (8.0, 128, 1 << 16)]
GAUSS_DRAWS = 20000
CRT_L = [1, 2, 5, 32]
CRT_LOG_N = 6


def main() -> None:
    if not oracle.ref_samplers_available():
        sys.exit("oracle/_ref/libyellref_samplers.so missing: run `make -C oracle ref_samplers` "
                 "with the reference and the GMP/MPFR runtimes present")
    ref = oracle.RefSamplers()
    port = oracle.Oracle("port")
    out = {}
    for i, (count, L, log_n, seed) in enumerate(UNIFORM):
        out[f"uniform_{i}"] = ref.sample_uniform(count, L, log_n, seed)
        out[f"uniform_{i}_args"] = np.array([count, L, log_n, seed], dtype=np.uint64)
    for i, (count, L, log_n, rho, seed) in enumerate(ZO):
        out[f"zo_{i}"] = ref.sample_zo(count, L, log_n, rho, seed)
        out[f"zo_{i}_args"] = np.array([count, L, log_n, rho, seed], dtype=np.uint64)
    for i, (count, L, log_n, h, seed) in enumerate(HWT):
        out[f"hwt_{i}"] = ref.sample_hwt(count, L, log_n, h, seed)
        out[f"hwt_{i}_args"] = np.array([count, L, log_n, h, seed], dtype=np.uint64)
    for i, (sigma, security, samples) in enumerate(GAUSS):
        top, info = ref.gaussian_barriers(sigma, security, samples)
        out[f"gauss_{i}_top64"] = top
        out[f"gauss_{i}_info"] = np.array(info, dtype=np.uint64)
        out[f"gauss_{i}_args"] = np.array([sigma, security, samples], dtype=np.float64)
        out[f"gauss_{i}_draws"] = ref.gaussian_sample(GAUSS_DRAWS, 1000 + i, sigma, security, samples)
    n = 1 << CRT_LOG_N
    for L in CRT_L:
        primes = [port.prime(j) for j in range(L)]
        limbs = np.stack([splitmix64(500 + j, n) % np.uint64(primes[j]) for j in range(L)])
        # edge residues: all zero, all p - 1, and a small integer in every limb
        limbs[:, 0] = 0
        limbs[:, 1] = [p - 1 for p in primes]
        limbs[:, 2] = 12345
        W = (sum(p.bit_length() for p in primes) + 63) // 64 + 1
        out[f"crt_{L}_limbs"] = limbs
        out[f"crt_{L}_words"] = ref.poly2mpz(limbs, CRT_LOG_N, W)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
