"""GRHD conversion in the oracle: the restated root finder against the
reference's own newton1d_brak (compiled from its source by
oracle/ref/Makefile), and the conservative <-> primitive round trip."""
import ctypes
import os

import numpy as np
import pytest

from oracle import nmo

REFLIB = os.path.join(os.path.dirname(nmo.__file__), "_ref", "libnewton1d.so")


def random_prims(npts, seed, vmax=0.95):
    rng = np.random.default_rng(seed)
    rho = 10.0 ** rng.uniform(-8, 0, npts)
    p = rho * 10.0 ** rng.uniform(-4, 1, npts)
    v = rng.normal(size=(3, npts))
    v *= rng.uniform(0, vmax, npts) / np.linalg.norm(v, axis=0)
    return np.vstack([rho, v, p])


def _funcs():
    def cubic(x, f, df):
        f[0] = x ** 3 - 2.0
        df[0] = 3 * x * x

    def cosx(x, f, df):
        f[0] = np.cos(x) - x
        df[0] = -np.sin(x) - 1.0

    def flat(x, f, df):      # df = 0 away from the root: bisection steps
        f[0] = np.tanh(50 * (x - 0.3))
        df[0] = 0.0

    def c2p(x, f, df):       # the con2prim residual of one state
        D, tau, S2, gm1, gam = 0.8, 1.7, 2.2, 1.0, 2.0
        E = tau + D + x
        v2 = S2 / (E * E)
        W = 1.0 / np.sqrt(1.0 - v2)
        rho = D / W
        eps = (tau + D * (1.0 - W) + x * (1.0 - W * W)) / (D * W)
        f[0] = gm1 * rho * eps - x
        df[0] = v2 * gam * gm1 * eps / (1.0 + gam * eps) - 1.0

    return [(cubic, 0.0, 3.0, 1.0), (cosx, -1.0, 2.0, 5.0), (flat, 0.0, 1.0, 0.5),
            (c2p, 0.0, 10.0, 0.1), (cubic, 2.0, 3.0, 2.5)]   # last: not bracketed


@pytest.mark.skipif(not os.path.exists(REFLIB), reason="reference newton1d_brak not built here")
def test_newton1d_brak_bitexact_vs_reference():
    ref = ctypes.CDLL(REFLIB)
    for fdf, x1, x2, x0 in _funcs():
        for maxits, xacc in ((100, 1e-14), (5, 1e-10), (60, 0.0)):
            a = nmo.newton1d_brak(fdf, x0, x1, x2, maxits, xacc)
            b = nmo.newton1d_brak(fdf, x0, x1, x2, maxits, xacc, lib_=ref)
            assert a == b, (fdf.__name__, maxits, a, b)


@pytest.mark.parametrize("psi", [None, "conformal"])
def test_oracle_grhd_roundtrip(psi):
    n = 4000
    prim = random_prims(n, seed=3)
    ps = None if psi is None else 1.0 + np.random.default_rng(4).uniform(0, 0.5, n)
    if ps is not None:
        prim[1:4] /= ps ** 2          # keep psi^4 v^i v^i < 1
    cons = nmo.grhd_prim2con(prim, ps)
    guess = prim.copy()
    guess[4] *= 1.3
    got, cons2, st = nmo.grhd_con2prim(cons, guess, ps)
    assert (st >= 0).all()
    assert np.array_equal(cons2, cons)
    rel = np.abs(got - prim) / np.maximum(np.abs(prim), 1e-300)
    assert rel[[0, 4]].max() <= 1e-9
    assert np.abs(got[1:4] - prim[1:4]).max() <= 1e-9


def test_oracle_grhd_atmosphere():
    prim = random_prims(6, seed=5)
    cons = nmo.grhd_prim2con(prim)
    cons[0, 0] = 1e-20                      # below the atmosphere density
    cons[4, 1] = -5.0                       # negative energy
    cons[1, 2] = 1e3 * (cons[4, 2] + cons[0, 2])   # |S| > tau + D: v > 1
    cons[:, 3] = np.nan
    got, cons2, st = nmo.grhd_con2prim(cons, prim)
    for i in range(4):
        assert st[i] < 0
        assert got[0, i] == 1e-12 and got[4, i] == 1e-14 and not got[1:4, i].any()
        assert cons2[0, i] == 1e-12 and not cons2[1:4, i].any()
    assert (st[4:] >= 0).all()


def test_oracle_grhd_fluxes_and_speeds():
    n = 2000
    prim = random_prims(n, seed=8)
    for d in range(3):
        flux, lam = nmo.grhd_fluxes(prim, d)
        cons = nmo.grhd_prim2con(prim)
        # F^d = v^d U (+ pressure terms) in flat space with alpha = 1
        assert np.allclose(flux[0], prim[1 + d] * cons[0], rtol=1e-14, atol=0)
        assert np.allclose(flux[4], prim[1 + d] * cons[4] + prim[4] * prim[1 + d],
                           rtol=1e-13, atol=1e-300)
        # subluminal, ordered, around the flow velocity
        assert (np.abs(lam) < 1).all() and (lam[0] <= prim[1 + d]).all()
        assert (lam[1] >= prim[1 + d]).all()
    # fluid at rest: lambda = -+ c_s
    rest = prim.copy()
    rest[1:4] = 0.0
    _, lam = nmo.grhd_fluxes(rest, 0)
    eps = rest[4] / rest[0]          # gamma = 2: p = rho eps
    cs = np.sqrt(2.0 * rest[4] / (rest[0] * (1.0 + eps + rest[4] / rest[0])))
    assert np.allclose(lam[1], cs, rtol=1e-13) and np.allclose(lam[0], -cs, rtol=1e-13)


def test_oracle_grhd_sources_static_fluid():
    """A static fluid (v = 0) feels only the gravity of the lapse:
    S(S_j) = psi^6 (6 alpha p d_j psi / psi - E d_j alpha), S(tau) = 0."""
    n = 500
    rng = np.random.default_rng(9)
    prim = random_prims(n, seed=10)
    prim[1:4] = 0.0
    alpha = rng.uniform(0.5, 1.0, n)
    psi = rng.uniform(1.0, 1.5, n)
    da = rng.normal(size=(3, n))
    dp = rng.normal(size=(3, n))
    src = nmo.grhd_sources(prim, alpha, psi, da, dp)
    rho, p = prim[0], prim[4]
    E = rho * (1.0 + p / rho + p / rho) - p
    for j in range(3):
        ref = psi ** 6 * (6.0 * alpha * dp[j] / psi * p - E * da[j])
        assert np.allclose(src[1 + j], ref, rtol=1e-12, atol=1e-300)
    assert not src[0].any() and not src[4].any()
