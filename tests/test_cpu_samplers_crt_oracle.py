"""Oracle checks for the sampler and CRT-lifting rows (CPU only).

Distribution checks of the sampler oracle against the reference's stated
laws (include/yell/details/poly.hpp:195-330, include/yell/poly.hpp:27-41),
and of the CRT oracle against the CRT itself: its output x must satisfy
x = r_j mod q_j and 0 <= x < Q, which determines x uniquely.  Word-for-word
pins to the reference's own code are in test_cpu_samplers_ref_pin.py.
"""
import math

import numpy as np
import pytest

from oracle.crt import CrtTable, poly2bigint, to_words
from yell_gb300.inputs import splitmix64


def test_uniform_rule(orc):
    L, log_n = 3, 12
    out = orc.sample_uniform(2, L, log_n, cm0=4, seed=11)
    n = 1 << log_n
    w = splitmix64(11, 2 * L * n).reshape(2, L, n)
    for l in range(L):
        p = orc.prime(4 + l)
        mask = (1 << p.bit_length()) - 1
        want = w[:, l] & np.uint64(mask)
        want = np.where(want >= np.uint64(p), want - np.uint64(p), want)
        assert np.array_equal(out[:, l], want)
        assert int(out[:, l].max()) < p
        assert abs(out[:, l].astype(np.float64).mean() / p - 0.5) < 0.02


@pytest.mark.parametrize("rho", [0, 0x7F, 0xFF])
def test_zo_distribution(orc, rho):
    L, log_n = 2, 14
    out = orc.sample_zo(2, L, log_n, rho=rho, seed=5)
    p0, p1 = orc.prime(0), orc.prime(1)
    e0 = np.where(out[:, 0] == np.uint64(p0 - 1), -1, out[:, 0].astype(np.int64))
    e1 = np.where(out[:, 1] == np.uint64(p1 - 1), -1, out[:, 1].astype(np.int64))
    assert np.array_equal(e0, e1)  # same integers in every limb
    assert set(np.unique(e0)) <= {-1, 0, 1}
    # exact law of the rule for a uniform byte r: +1 when r <= rho and bit 1 of
    # r is clear, -1 when r <= rho and it is set
    plus = sum(1 for r in range(rho + 1) if not r & 2) / 256
    minus = sum(1 for r in range(rho + 1) if r & 2) / 256
    assert abs(np.mean(e0 == 1) - plus) < 0.01
    assert abs(np.mean(e0 == -1) - minus) < 0.01


@pytest.mark.parametrize("h", [1, 64, 4096])
def test_hwt_weight(orc, h):
    L, log_n = 3, 12
    out = orc.sample_hwt(4, L, log_n, h=h, seed=9)
    for i in range(4):
        nz = [np.flatnonzero(out[i, l]) for l in range(L)]
        assert all(np.array_equal(nz[0], z) for z in nz)
        assert len(nz[0]) == h
        for l in range(L):
            p = orc.prime(l)
            v = out[i, l][nz[0]]
            assert np.all((v == 1) | (v == np.uint64(p - 1)))


def test_gaussian_table_and_moments(orc):
    sigma, tail = 3.2, 19
    cdt = orc.gaussian_cdt(sigma, tail)
    assert len(cdt) == 2 * tail + 1 and int(cdt[-1]) == 2**64 - 1
    ws = [math.exp(-(e * e) / (2 * sigma * sigma)) for e in range(-tail, tail + 1)]
    tot = sum(ws)
    acc = 0.0
    for k in range(len(cdt) - 1):
        acc += ws[k]
        assert abs(int(cdt[k]) / 2**64 - acc / tot) < 1e-12
    out = orc.sample_gaussian(4, 1, 14, sigma=sigma, tail=tail, seed=3)
    p = orc.prime(0)
    e = out.astype(object)
    e = np.array([int(v) - p if int(v) > p // 2 else int(v) for v in out.reshape(-1)], dtype=np.int64)
    assert abs(e.mean()) < 0.05
    assert abs(e.std() - sigma) < 0.05
    assert np.abs(e).max() <= tail
    amp = orc.sample_gaussian(1, 2, 10, sigma=sigma, tail=tail, amplifier=1000, seed=3)
    base = orc.sample_gaussian(1, 2, 10, sigma=sigma, tail=tail, seed=3)
    for l in range(2):
        p = orc.prime(l)
        sb = np.array([int(v) - p if int(v) > p // 2 else int(v) for v in base[0, l]])
        sa = np.array([int(v) - p if int(v) > p // 2 else int(v) for v in amp[0, l]])
        assert np.array_equal(sa, 1000 * sb)


@pytest.mark.parametrize("L", [1, 2, 5, 16])
def test_crt_oracle_is_the_crt(orc, L):
    primes = [orc.prime(j) for j in range(L)]
    t = CrtTable(primes)
    n = 64
    limbs = np.stack([splitmix64(100 + j, n) % np.uint64(primes[j]) for j in range(L)])
    xs = poly2bigint(limbs, primes)
    for i, x in enumerate(xs):
        assert 0 <= x < t.Q
        for j in range(L):
            assert x % primes[j] == int(limbs[j, i])
    # small integers and Q - 1 lift to themselves
    for x in [0, 1, 2, 12345, t.Q - 1, t.Q // 3]:
        assert t.lift_coeff([x % p for p in primes]) == x
    w = to_words(xs, t.words())
    assert w.shape == (n, t.words())
    assert all(int.from_bytes(w[i].tobytes(), "little") == xs[i] for i in range(n))


def test_hwt_positions_uniform(orc):
    """Positions of the reservoir HWT sampler follow the reference's law.

    The reference draws the replacement index for item k uniformly from
    [0, k) (include/yell/details/poly.hpp:296-315), not [0, k] as reservoir
    sampling over k + 1 items would, so the set is not a uniform h-subset:
    item k >= h is kept with probability (h/k) * prod_{m>k} (1 - 1/m) =
    h/(N-1) and each of the first h items with (h-1)/(N-1).  Chi-square
    against that law; pairs co-occur h(h-1)/(N(N-1)) of the time on average,
    as for any fixed-size subset."""
    log_n, h, cnt = 6, 5, 20000
    n = 1 << log_n
    nz = orc.sample_hwt(cnt, 1, log_n, h=h, seed=21)[:, 0] != 0
    counts = nz.sum(0)
    e = cnt * np.where(np.arange(n) < h, (h - 1) / (n - 1), h / (n - 1))
    chi2 = float(((counts - e) ** 2 / e).sum())
    assert chi2 < 2.0 * (n - 1)  # dof 63: mean 63, sd ~11
    e_uniform = cnt * h / n
    assert float(((counts - e_uniform) ** 2 / e_uniform).sum()) > 3.0 * (n - 1)  # the bias is real
    z = nz.astype(np.float64)
    co = z.T @ z
    exp = cnt * h * (h - 1) / (n * (n - 1))
    off = co[~np.eye(n, dtype=bool)]
    assert abs(off.mean() / exp - 1) < 0.02
    assert ((off - exp) ** 2 / exp).mean() < 2.0
