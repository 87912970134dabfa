"""Edge cases of the coupling and QuickPol entry points against the oracle: one-element grids
(lmin = lmax), a diagonal-only QuickPol band, and QuickPol grids below l'' = 2."""
import numpy as np
import pytest

from gpu_util import cond_scale, cov_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,tol", [("plain", 1e-12), ("chosen", 1e-6)])
@pytest.mark.parametrize("l", [0, 1, 2, 5, 300])
def test_one_element_grid(ctx, mode, tol, l):
    from powerspectra_gpu import synthetic as syn
    W = syn.mask_spectrum(2 * l + 1, 0.6, 30.0, seed=l)
    got = ctx.mcm_multi({s: W for s in range(4)}, l, l, mode=mode)
    for s in range(4):
        ref = o.inner_mcm(s, W, l, l)
        assert got[s].shape == (1, 1)
        assert max_err_scaled(got[s], ref, cond_scale(s, W, l, l)) < tol, (s, l)


@pytest.mark.parametrize("kind", ["TTTT", "EEEE", "TETE", "TTTE", "TEEE", "TEEE_PLANCK", "TTEE"])
def test_one_element_covariance(ctx, kind):
    from powerspectra_gpu import synthetic as syn
    l = 7
    rng = np.random.default_rng(1)
    S = [1.0 + rng.random(l + 1) for _ in range(4)]
    R = [1.0 + rng.random(l + 1) for _ in range(o.COV_NRATIOS[kind])]
    Ws = [syn.mask_spectrum(2 * l + 1, 0.5, 10.0, seed=k) for k in range(o.COV_NWINDOWS[kind])]
    for mode, tol in (("plain", 1e-12), ("chosen", 1e-6)):
        C = ctx.coupledcov(kind, S, R, Ws, l, l, mode=mode)
        ref = o.loop_cov(kind, S, R, Ws, l, l)
        assert max_err_scaled(C, ref, cov_scale(kind, S, R, Ws, l, l)) < tol, (kind, mode)


@pytest.mark.parametrize("mode,tol", [("plain", 1e-10), ("chosen", 1e-6)])
def test_quickpol_diagonal_band(ctx, mode, tol):
    lmax = 90
    W = np.exp(-np.arange(2 * lmax + 1) / 30.0)
    G = ctx.quickpol_xi(1, 0, 2, 2, W, lmax, 0, 0, mode=mode)
    R = o.quickpol_xi(1, 0, 2, 2, W, lmax, 0, 0)
    A = o.quickpol_xi(1, 0, 2, 2, W, lmax, 0, 0, absolute=True)
    assert not np.any(G - np.diag(np.diag(G)))
    d = np.arange(2, lmax + 1)
    assert np.max(np.abs(G[d, d] - R[d, d]) / A[d, d]) < tol


@pytest.mark.parametrize("mode", ["plain", "chosen"])
@pytest.mark.parametrize("lmax", [0, 1])
def test_quickpol_below_l2(ctx, mode, lmax):
    """quickpolXi! starts at l'' = 2, so grids with lmax < 2 come back all zero."""
    X = ctx.quickpol_xi(0, 0, 2, 2, np.ones(5), lmax, 3, 3, mode=mode)
    assert X.shape == (lmax + 1, lmax + 1) and not np.any(X)
