"""GPU samplers (poly<N>::set(uniform / ZO_dist / hwt_dist / gaussian),
include/yell/details/poly.hpp:195-330) against the oracle word for word on
seeded streams, plus full-size distribution checks and argument errors."""
import numpy as np
import pytest

import yell_gb300 as y

pytestmark = pytest.mark.gpu


def _empty(torch, count, L, log_n):
    return torch.zeros(count * L << log_n, dtype=torch.int64, device="cuda")


def _host(t, count, L, log_n):
    return t.cpu().numpy().view(np.uint64).reshape(count, L, 1 << log_n)


@pytest.mark.parametrize("count,L,log_n,cm0,seed", [(1, 1, 3, 0, 0), (2, 3, 6, 0, 3), (5, 1, 7, 11, 4),
                                                    (2, 3, 10, 7, 1), (3, 4, 13, 0, 99), (1, 2, 17, 500, 5)])
def test_uniform_matches_oracle(cuda, orc, count, L, log_n, cm0, seed):
    t = _empty(cuda, count, L, log_n)
    y.sample_uniform(t, count, L, log_n, cm0, seed=seed)
    cuda.cuda.synchronize()
    assert np.array_equal(_host(t, count, L, log_n), orc.sample_uniform(count, L, log_n, cm0, seed))


@pytest.mark.parametrize("rho", [0, 1, 0x7F, 0xFF])
@pytest.mark.parametrize("log_n", [3, 12])
def test_zo_matches_oracle(cuda, orc, rho, log_n):
    count, L = 2, 3
    t = _empty(cuda, count, L, log_n)
    y.sample_zo(t, count, L, log_n, 2, rho=rho, seed=17)
    cuda.cuda.synchronize()
    assert np.array_equal(_host(t, count, L, log_n), orc.sample_zo(count, L, log_n, 2, rho, 17))


@pytest.mark.parametrize("log_n,h", [(3, 1), (3, 8), (10, 64), (12, 4096), (14, 192), (17, 1), (20, 1000)])
def test_hwt_matches_oracle(cuda, orc, log_n, h):
    count, L = (3, 2) if log_n < 20 else (2, 1)
    t = _empty(cuda, count, L, log_n)
    y.sample_hwt(t, count, L, log_n, h, cm0=1, seed=h + log_n)
    cuda.cuda.synchronize()
    got = _host(t, count, L, log_n)
    assert np.array_equal(got, orc.sample_hwt(count, L, log_n, h, 1, h + log_n))
    for i in range(count):
        assert np.count_nonzero(got[i, 0]) == h


@pytest.mark.parametrize("log_n,h", [(3, 8), (10, 64), (12, 4096), (13, 7)])
def test_hwt_draw_order_path(cuda, orc, monkeypatch, log_n, h):
    """The one-thread reservoir in draw order (taken when a draw is rejected,
    forced here) gives the same polys as the parallel draws."""
    count, L = 2, 2
    monkeypatch.setenv("YELL_GB300_HWT_SEQUENTIAL", "1")
    t = _empty(cuda, count, L, log_n)
    y.sample_hwt(t, count, L, log_n, h, seed=5 + h)
    cuda.cuda.synchronize()
    assert np.array_equal(_host(t, count, L, log_n), orc.sample_hwt(count, L, log_n, h, 0, 5 + h))


def test_samplers_match_reference_fixture(cuda):
    """GPU output against the reference's own set(uniform / ZO_dist /
    hwt_dist) on the same stream (tests/golden/yell_ref_samplers.npz)."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "yell_ref_samplers.npz"))
    checked = 0
    for kind in ("uniform", "zo", "hwt"):
        i = 0
        while f"{kind}_{i}" in g:
            want = g[f"{kind}_{i}"]
            args = [int(v) for v in g[f"{kind}_{i}_args"]]
            count, L, log_n = args[:3]
            t = _empty(cuda, count, L, log_n)
            if kind == "uniform":
                y.sample_uniform(t, count, L, log_n, seed=args[3])
            elif kind == "zo":
                y.sample_zo(t, count, L, log_n, rho=args[3], seed=args[4])
            else:
                y.sample_hwt(t, count, L, log_n, args[3], seed=args[4])
            cuda.cuda.synchronize()
            assert np.array_equal(_host(t, count, L, log_n), want), (kind, i)
            checked += 1
            i += 1
    assert checked == 17


@pytest.mark.parametrize("sigma,tail,amp", [(3.2, 19, 1), (3.2, 19, 1 << 20), (0.5, 4, 1), (40.0, 1024, 3)])
def test_gaussian_matches_oracle(cuda, orc, sigma, tail, amp):
    count, L, log_n = 2, 3, 12
    t = _empty(cuda, count, L, log_n)
    y.sample_gaussian(t, count, L, log_n, 3, sigma=sigma, tail=tail, amplifier=amp, seed=41)
    cuda.cuda.synchronize()
    want = orc.sample_gaussian(count, L, log_n, 3, sigma=sigma, tail=tail, amplifier=amp, seed=41)
    assert np.array_equal(_host(t, count, L, log_n), want)


def test_full_size_distributions(cuda, orc):
    """N = 2^16, L = 32, 16 polys: ranges and moments of every sampler."""
    count, L, log_n = 16, 32, 16
    ps = [orc.prime(l) for l in range(L)]
    pv = cuda.tensor([p for p in ps], dtype=cuda.int64, device="cuda").view(1, L, 1)
    t = _empty(cuda, count, L, log_n)
    y.sample_uniform(t, count, L, log_n, seed=1)
    u = t.view(count, L, -1)
    assert bool(((u >= 0) & (u < pv)).all())
    frac = (u.double() / pv.double()).mean().item()
    assert abs(frac - 0.5) < 1e-3
    y.sample_gaussian(t, count, L, log_n, seed=2)
    g = t.view(count, L, -1)
    e = cuda.where(g > pv // 2, g - pv, g)
    assert bool((e == e[:, :1]).all())  # same integer in every limb
    ef = e[:, 0].double()
    assert abs(ef.mean().item()) < 0.01 and abs(ef.std().item() - 3.2) < 0.01
    y.sample_hwt(t, count, L, log_n, 192, seed=3)
    assert bool(((t.view(count, L, -1) != 0).sum(-1) == 192).all())


def test_sampler_errors(cuda):
    t = _empty(cuda, 1, 1, 10)
    with pytest.raises(y.YellError):
        y.sample_zo(t, 1, 1, 10, rho=256)
    with pytest.raises(y.YellError):
        y.sample_hwt(t, 1, 1, 10, h=0)
    with pytest.raises(y.YellError):
        y.sample_hwt(t, 1, 1, 10, h=1025)
    with pytest.raises(y.YellError):
        y.sample_gaussian(t, 1, 1, 10, sigma=-1.0)
    with pytest.raises(y.YellError):
        y.sample_gaussian(t, 1, 1, 10, tail=19, amplifier=1 << 60)
    with pytest.raises(y.YellError):
        y.sample_uniform(t, 1, 1, 21)  # above the largest degree: rejected before any launch
