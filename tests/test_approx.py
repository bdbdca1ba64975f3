"""Zolotarev's optimal approximation to sgn(x) (Approx::zolotarev, Zolotarev.cc:296-417),
computed on the host by the library (no device work): the Cayley form
R(x) = (1 - T(x)) / (1 + T(x)), T(x) = prod (x - gamma_j) / (x + gamma_j), is pinned by the
defining properties of the optimum -- its maximum error on [epsilon, 1] is the returned
Delta and is reached at both ends and at interior extrema (equioscillation) -- and by
Zolotarev's error bound falling geometrically with n."""
import numpy as np
import pytest

import grid_gb300 as g


def cayley_error(gamma, eps, npts=200001):
    x = np.geomspace(eps, 1.0, npts)
    T = np.prod([(x - c) / (x + c) for c in gamma], axis=0)
    return np.abs((1 - T) / (1 + T) - 1.0)


@pytest.mark.parametrize("eps,n", [(0.1, 10), (0.05, 12), (0.2, 7), (0.01, 8), (0.3, 5), (0.003, 16)])
def test_zolotarev_equioscillates_at_delta(eps, n):
    """Type 0, the form the Cayley operators use (MobiusZolotarevFermion.h:60)."""
    gamma, delta = g.zolotarev(eps, n, 0)
    assert gamma.shape == (n,) and np.all(gamma > 0) and 0 < delta < 1
    e = cayley_error(gamma, eps)
    assert abs(e.max() - delta) < 1e-3 * delta
    assert abs(e[0] - delta) < 1e-3 * delta and abs(e[-1] - delta) < 1e-3 * delta
    peaks = [i for i in range(1, e.size - 1) if e[i] >= e[i - 1] and e[i] >= e[i + 1] and e[i] > 0.99 * delta]
    assert len(peaks) >= n - 1


def test_zolotarev_type1_shares_delta():
    """Type 1 (R(0) = infinity) has the same maximum error (Zolotarev.cc:357-359 computes
    Delta before the type switch); its Cayley zeros are positive and approach
    equioscillation as n grows.  Only type 0 feeds the Cayley operators."""
    for eps, n in ((0.1, 10), (0.01, 8), (0.3, 5)):
        g0, d0 = g.zolotarev(eps, n, 0)
        g1, d1 = g.zolotarev(eps, n, 1)
        assert d1 == d0 and np.all(g1 > 0) and not np.array_equal(g0, g1)
        assert abs(cayley_error(g1, eps).max() - d1) < 0.01 * d1


def test_zolotarev_error_falls_with_degree():
    deltas = [g.zolotarev(0.05, n)[1] for n in (4, 6, 8, 10, 12)]
    ratios = [b / a for a, b in zip(deltas, deltas[1:])]
    assert all(r < 0.2 for r in ratios)


def test_zolotarev_rejects_bad_arguments():
    for args in ((0.0, 8), (1.0, 8), (0.1, 0)):
        with pytest.raises(g.GridError):
            g.zolotarev(*args)


def test_higham_is_moebius():
    assert np.array_equal(g.higham(0.1, 6), np.ones(6))


# ---- Approx::computeZmobiusGamma (ZMobius.cc) ------------------------------------------
def zmobius_sign(gamma, bpc_out, x):
    om = np.asarray(gamma) / bpc_out
    fp = np.prod([x + w for w in om], axis=0)
    fm = np.prod([-x + w for w in om], axis=0)
    return ((fp - fm) / (fp + fm)).real


def mobius_sign(Ls, bpc, x):
    r = ((1.0 / bpc - x) / (1.0 / bpc + x)) ** Ls
    return (1 - r) / (1 + r)


@pytest.mark.parametrize("Lo,Li,bpc,lam", [(10, 24, 2.0, 1.42), (8, 16, 2.0, 1.42), (12, 24, 2.0, 1.42),
                                           (6, 12, 1.0, 1.0)])
def test_zmobius_gamma_is_the_minimax_approximation(Lo, Li, bpc, lam):
    """The ZMobius sign function of the returned gammas approximates the Moebius one with
    error reaching its maximum, with alternating signs, at Ls_out + 1 points of (0, lambda]
    (the Chebyshev alternation that characterises the minimax rational approximation)."""
    gamma, err = g.computeZmobiusGamma(bpc, Lo, bpc, Li, lam)
    assert gamma.shape == (Lo,) and 0 < err < 1e-2
    x = np.linspace(lam * 1e-6, lam, 400001)
    e = zmobius_sign(gamma, bpc, x) - mobius_sign(Li, bpc, x)
    assert abs(np.abs(e).max() - err) < 1e-3 * err
    signs, prev = [], 0
    for i in np.flatnonzero(np.abs(e) > 0.999 * err):
        s = np.sign(e[i])
        if s != prev:
            signs.append(s)
            prev = s
    assert len(signs) >= Lo + 1
    # real coefficients: the omegas are closed under conjugation
    assert np.allclose(np.sort_complex(gamma), np.sort_complex(gamma.conj()), atol=1e-9)
    # Grid's placement: the largest omegas at the two ends of the fifth dimension
    re = gamma.real
    assert re[0] == re.max() and re[-1] == np.sort(re)[-2]


def test_zmobius_gamma_error_falls_with_ls_and_scales_with_bpc_out():
    errs = [g.computeZmobiusGamma(2.0, Lo, 2.0, 24, 1.42)[1] for Lo in (6, 8, 10, 12)]
    assert all(b < 0.3 * a for a, b in zip(errs, errs[1:]))
    g1, _ = g.computeZmobiusGamma(2.0, 8, 2.0, 16, 1.42)
    g2, _ = g.computeZmobiusGamma(3.0, 8, 2.0, 16, 1.42)
    assert np.allclose(g2, 1.5 * g1, rtol=1e-12)
    with pytest.raises(g.GridError):
        g.computeZmobiusGamma(2.0, 7, 2.0, 16, 1.42)
