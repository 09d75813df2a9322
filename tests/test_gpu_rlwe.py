"""The RLWE loop the reference's example.cpp builds from poly<N> calls, kept
on the device from sampling to lifting: key generation, encryption of a
message scaled by Delta = floor(Q / t), decryption by c0 + c1 * s, and the
CRT lift that returns round(t * x / Q).  Every device step is one library
call (samplers, NTT, element-wise ops, CRT lifting); the ciphertext words are
checked against the oracle run on the same sampled polynomials, and the
decrypted message against the plaintext.
(include/yell/details/poly.hpp:118-157,195-330; include/yell/gmp.hpp:42-70)"""
import numpy as np
import pytest

import yell_gb300 as y
from yell_gb300._capi import (YELL_BACKWARD, YELL_FORWARD, YELL_OP_ADDMOD, YELL_OP_MULMOD,
                              YELL_OP_SUBMOD)
from yell_gb300.inputs import splitmix64

pytestmark = pytest.mark.gpu


def test_rlwe_encrypt_decrypt_on_device(cuda, orc):
    torch = cuda
    log_n, L, t = 12, 4, 1 << 16
    n = 1 << log_n
    ps = [int(p) for p in y.primes(L)]
    Q = 1
    for p in ps:
        Q *= p
    delta = Q // t
    y.init_ntt_tables(log_n, L)

    def new():
        return torch.empty((L, n), dtype=torch.int64, device="cuda")

    def host(d):
        return d.cpu().numpy().view(np.uint64).copy()

    def fwd(d):
        out = d.clone()
        y.dev_ntt(out, 1, L, log_n, 0, YELL_FORWARD)
        return out

    def op(code, a, b):
        out = new()
        y.dev_elementwise(code, out, a, b, 1, L, log_n, 0)
        return out

    # key generation: s ternary of weight 64, a uniform, e Gaussian; b = e - a s (NTT domain)
    s, a, e = new(), new(), new()
    y.sample_hwt(s, 1, L, log_n, 64, seed=11)
    y.sample_uniform(a, 1, L, log_n, seed=12)
    y.sample_gaussian(e, 1, L, log_n, seed=13)
    s_n, a_n, e_n = fwd(s), fwd(a), fwd(e)
    b_n = op(YELL_OP_SUBMOD, e_n, op(YELL_OP_MULMOD, a_n, s_n))

    # encryption of m: u ternary (ZO), e1, e2 Gaussian
    m = (splitmix64(14, n) % np.uint64(t)).astype(np.uint64)
    dm = np.stack([np.array([(delta * int(v)) % p for v in m], dtype=np.uint64) for p in ps])
    dm_d = torch.from_numpy(dm.view(np.int64)).cuda()
    u, e1, e2 = new(), new(), new()
    y.sample_zo(u, 1, L, log_n, seed=15)
    y.sample_gaussian(e1, 1, L, log_n, seed=16)
    y.sample_gaussian(e2, 1, L, log_n, seed=17)
    u_n = fwd(u)
    c0 = op(YELL_OP_ADDMOD, op(YELL_OP_MULMOD, b_n, u_n), fwd(op(YELL_OP_ADDMOD, e1, dm_d)))
    c1 = op(YELL_OP_ADDMOD, op(YELL_OP_MULMOD, a_n, u_n), fwd(e2))

    # decryption: x = c0 + c1 s in coefficients, lifted to [0, Q)
    d = op(YELL_OP_ADDMOD, c0, op(YELL_OP_MULMOD, c1, s_n))
    y.dev_ntt(d, 1, L, log_n, 0, YELL_BACKWARD)
    W = y.crt_words(L)
    lifted = torch.empty(n * W, dtype=torch.int64, device="cuda")
    y.dev_crt_lift(lifted, d, 1, L, log_n, 0)
    y.synchronize()
    xs = y.words_to_ints(lifted.cpu().numpy().view(np.uint64).reshape(n, W))
    got = np.array([((t * x + Q // 2) // Q) % t for x in xs], dtype=np.uint64)
    assert np.array_equal(got, m)
    # the noise e u + e1 + e2 s stays far below Delta / 2
    noise = max(abs(((x - delta * int(v) + Q // 2) % Q) - Q // 2) for x, v in zip(xs, m))
    assert noise < 1 << 20

    # the same steps in the oracle, on the sampled polynomials, give the same words
    hs, ha, he, hu, he1, he2 = (host(v) for v in (s, a, e, u, e1, e2))
    F = [[orc.forward(v[l], log_n, l) for l in range(L)] for v in (hs, ha, he, hu)]
    o_s, o_a, o_e, o_u = F
    o_b = [orc.submod(o_e[l], orc.mulmod(o_a[l], o_s[l], l), l) for l in range(L)]
    o_c0 = [orc.addmod(orc.mulmod(o_b[l], o_u[l], l), orc.forward(orc.addmod(he1[l], dm[l], l), log_n, l), l)
            for l in range(L)]
    o_c1 = [orc.addmod(orc.mulmod(o_a[l], o_u[l], l), orc.forward(he2[l], log_n, l), l) for l in range(L)]
    gc0, gc1 = host(c0), host(c1)
    for l in range(L):
        assert np.array_equal(gc0[l], o_c0[l]), l
        assert np.array_equal(gc1[l], o_c1[l]), l
