"""QuickPol beam coupling Xi (quickpolXi!, src/beam.jl:72-109) against the oracle.

General-spin families (l' l l''; s+nu, -s, -nu): the oracle's recurrence is
checked against exact 3j values for such spins in tests/test_oracle.py."""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nu1,nu2,s1,s2", [(0, 0, 0, 0), (0, 0, 2, 2), (1, -1, 2, 0), (2, 2, -2, 2), (-3, 1, 2, -2),
                                           (4, -4, 0, 2)])
@pytest.mark.parametrize("lmax,bl,bu,nWk", [(120, 10, 10, "2L"), (200, 30, 5, "L"), (60, 100, 100, "short")])
def test_quickpol_vs_oracle(ctx, nu1, nu2, s1, s2, lmax, bl, bu, nWk):
    nW = {"2L": 2 * lmax + 1, "L": lmax + 1, "short": lmax // 2}[nWk]
    rng = np.random.default_rng(lmax + 7 * nu1 + 3 * s1)
    W = rng.random(nW) * np.exp(-np.arange(nW) / 40.0)
    G = ctx.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu)
    # the oracle with the kernel's match point (both families at the larger midpoint): the same
    # algorithm in C, so the plain kernel agrees to rounding
    R = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, common_match=True)
    # the sum of |W f1 f2| behind each element: the products of two different families change
    # sign, so an element's rounding error is relative to it (never below |R|)
    scale = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, absolute=True)
    den = np.maximum(np.abs(R), scale)
    band = np.zeros_like(G, dtype=bool)
    for r in range(2, lmax + 1):
        band[r, max(2, r - bl):min(lmax, r + bu) + 1] = True
    assert not np.any(G[~band])
    err = np.abs(G - R)[band] / np.where(den[band] == 0, 1.0, den[band])
    assert np.max(err) < 1e-12


def test_quickpol_known_identity(ctx):
    """nu = s = 0 with W = 4 pi delta_l0 ... (l' l l''; 0 0 0)^2 summed against W_0 only
    picks l' = 0, i.e. l = l'': Xi is diagonal with value W_0 / (2 l + 1)."""
    lmax = 80
    W = np.zeros(2 * lmax + 1)
    W[0] = 3.0
    X = ctx.quickpol_xi(0, 0, 0, 0, W, lmax, 5, 5)
    l = np.arange(lmax + 1)
    np.testing.assert_allclose(np.diag(X)[2:], 3.0 / (2 * l[2:] + 1), rtol=1e-13)
    off = X - np.diag(np.diag(X))
    assert np.max(np.abs(off)) < 1e-15


@pytest.mark.parametrize("alm_lmax,alm_mmax,lmax,bl,bu", [(64, 64, 40, 6, 9), (100, 30, 50, 50, 50),
                                                           (200, 200, 40, 10, 10), (300, 50, 60, 20, 5)])
def test_quickpol_from_scan_weights(ctx, alm_lmax, alm_mmax, lmax, bl, bu):
    """quickpolXi!(Xi, nu1, nu2, s1, s2, omega1, omega2): W = quickpolW(omega1, omega2) on the GPU,
    then Xi, against the oracle's quickpolW and Xi.  Sets reaching beyond 2 lmax are packed to the
    rows that enter (the last two cases)."""
    rng = np.random.default_rng(alm_lmax)
    n = o.n_alms(alm_lmax, alm_mmax)
    w1 = (rng.normal(size=n) + 1j * rng.normal(size=n)) * np.exp(-np.arange(n) / 500.0)
    w2 = (rng.normal(size=n) + 1j * rng.normal(size=n)) * np.exp(-np.arange(n) / 500.0)
    for (om1, om2) in ((w1, w2), (w1, w1)):
        G = ctx.quickpol_xi_alm(2, 0, 2, -2, om1, om2, alm_lmax, lmax, bl, bu, alm_mmax=alm_mmax)
        W = o.quickpolW(om1, om2, alm_lmax, alm_mmax)
        R = o.quickpol_xi(2, 0, 2, -2, W, lmax, bl, bu, common_match=True)
        # W itself is a cancelling sum over m, known to rounding relative to sum_m |w1 w2| (Wa);
        # Xi then to rounding relative to sum |Wa f1 f2| (the absolute sums over Wa >= |W|)
        Wa = o.quickpolW(np.abs(om1).astype(complex), np.abs(om2).astype(complex), alm_lmax, alm_mmax)
        scale = o.quickpol_xi(2, 0, 2, -2, Wa, lmax, bl, bu, absolute=True)
        den = np.maximum(np.abs(R), scale)
        err = np.abs(G - R)[scale > 0] / den[scale > 0]
        assert np.max(err) < 1e-12


@pytest.mark.parametrize("nu1,nu2,s1,s2", [(0, 0, 0, 0), (0, 0, 2, 2), (1, -1, 2, 0), (2, 2, -2, 2), (-3, 1, 2, -2),
                                           (4, -4, 0, 2)])
@pytest.mark.parametrize("lmax,bl,bu,nWk", [(120, 10, 10, "2L"), (300, 30, 5, "L"), (60, 100, 100, "short")])
def test_quickpol_chosen_vs_oracle(ctx, nu1, nu2, s1, s2, lmax, bl, bu, nWk):
    """The float-float (chosen) QuickPol kernel: max error 1e-6 against the FP64 oracle, relative to
    the sum of |terms| behind each element (the sum of W f1 f2 cancels: the two families differ, so
    their product changes sign; an FP32 partial sum resolves it only to that sum's precision)."""
    nW = {"2L": 2 * lmax + 1, "L": lmax + 1, "short": lmax // 2}[nWk]
    rng = np.random.default_rng(lmax + 5 * nu2 + 11 * s2)
    W = rng.random(nW) * np.exp(-np.arange(nW) / 40.0) * 1e-30  # far from 1: the staging scale must work
    G = ctx.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, mode="chosen")
    R = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu)
    A = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, absolute=True)
    band = np.zeros_like(G, dtype=bool)
    for r in range(2, lmax + 1):
        band[r, max(2, r - bl):min(lmax, r + bu) + 1] = True
    assert not np.any(G[~band])
    err = np.abs(G - R) / np.maximum(A, 1e-300)
    assert np.max(err[band]) < 1e-6


def test_quickpol_chosen_large_l(ctx):
    """l up to 2000 with the notebook's spins (nu = 0, s = 2): chosen against the FP64 kernel."""
    lmax, band = 2000, 20
    l = np.arange(2 * lmax + 1)
    W = (1.0 + np.cos(l / 37.0)) * np.exp(-l / 900.0)
    P = ctx.quickpol_xi(0, 0, 2, 2, W, lmax, band, band, mode="plain")
    C = ctx.quickpol_xi(0, 0, 2, 2, W, lmax, band, band, mode="chosen")
    A = o.quickpol_xi(0, 0, 2, 2, W, lmax, band, band, absolute=True)
    mask = A > 0
    assert np.max(np.abs(C - P)[mask] / A[mask]) < 1e-6


@pytest.mark.parametrize("mode", ["plain", "chosen"])
def test_quickpol_band_wider_than_grid(ctx, mode):
    """Bandwidths beyond lmax cover the whole grid: the same matrix, bit for bit, as bl = bu = lmax."""
    lmax = 70
    rng = np.random.default_rng(9)
    W = rng.random(2 * lmax + 1) * np.exp(-np.arange(2 * lmax + 1) / 30.0)
    A = ctx.quickpol_xi(0, 0, 2, 2, W, lmax, lmax, lmax, mode=mode)
    B = ctx.quickpol_xi(0, 0, 2, 2, W, lmax, 10 ** 6, 10 ** 6, mode=mode)
    assert np.array_equal(A, B)
    R = o.quickpol_xi(0, 0, 2, 2, W, lmax, lmax, lmax)
    S = o.quickpol_xi(0, 0, 2, 2, W, lmax, lmax, lmax, absolute=True)
    assert np.max(np.abs(A - R)[S > 0] / S[S > 0]) < (1e-10 if mode == "plain" else 1e-6)


def test_quickpol_into_caller_output(ctx):
    """A caller-supplied (page-locked) output receives the whole matrix, zeros outside the band included."""
    torch = pytest.importorskip("torch")
    lmax = 50
    W = np.exp(-np.arange(2 * lmax + 1) / 20.0)
    out = torch.full((lmax + 1, lmax + 1), float("nan"), dtype=torch.float64).pin_memory().numpy().T
    for mode in ("plain", "chosen"):
        out[:] = np.nan
        A = ctx.quickpol_xi(0, 0, 2, 2, W, lmax, 6, 6, mode=mode, out=out)
        assert A is out
        assert np.array_equal(A, ctx.quickpol_xi(0, 0, 2, 2, W, lmax, 6, 6, mode=mode))
    rng = np.random.default_rng(3)
    om = rng.normal(size=o.n_alms(30, 30)) + 1j * rng.normal(size=o.n_alms(30, 30))
    out2 = torch.full((21, 21), float("nan"), dtype=torch.float64).pin_memory().numpy().T
    B = ctx.quickpol_xi_alm(0, 0, 2, 2, om, om, 30, 20, 4, 4, mode="chosen", out=out2)
    assert B is out2
    assert np.array_equal(B, ctx.quickpol_xi_alm(0, 0, 2, 2, om, om, 30, 20, 4, 4, mode="chosen"))


def test_quickpol_mode_error(ctx):
    import powerspectra_gpu as pg
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.quickpol_xi(0, 0, 2, 2, np.ones(10), 8, 2, 2, mode=7)
