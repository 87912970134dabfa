"""CPU checks of the oracle (test infrastructure) against golden vectors.

Pins: (1) arbitrary-precision 3j values, (2) the reference test suite's
NaMaster diagonals (test/data/mcm_{TT,EE,TE}_diag.txt), (3) analytic known
answers, (4) the committed oracle fixtures.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as o


def test_families_vs_exact():
    rows = json.load(open(os.path.join(GOLDEN, "w3j_exact.json")))["rows"]
    cache = {}
    worst = 0.0
    for l1, l2, l3, m1, m2, sval in rows:
        key = (l1, l2, m1, m2)
        if key not in cache:
            cache[key] = o.w3j_family(l1, l2, m1, m2)
        jmin, f = cache[key]
        ex = float(sval)
        got = f[l3 - jmin] if 0 <= l3 - jmin < len(f) else 0.0
        # typical family amplitude: sum_l3 (2 l3 + 1) f^2 = 1 over the family
        amp = 1.0 / math.sqrt(max((l1 + l2 + 1) ** 2 - jmin ** 2, 1))
        err = abs(got - ex)
        assert err <= 1e-12 * abs(ex) + 1e-12 * amp, (l1, l2, l3, m1, m2, got, ex)
        worst = max(worst, err / max(abs(ex), amp))
    assert worst < 1e-12


@pytest.mark.parametrize("l1,l2", [(0, 0), (1, 1), (2, 5), (17, 4), (300, 299), (1000, 3), (2500, 2400), (8191, 8190)])
@pytest.mark.parametrize("m", [(0, 0), (-2, 2)])
def test_family_orthonormal(l1, l2, m):
    jmin, f = o.w3j_family(l1, l2, *m)
    if abs(m[0]) > min(l1, l2):
        assert not np.any(f)
        return
    j = np.arange(jmin, jmin + len(f))
    assert abs(np.sum((2 * j + 1) * f * f) - 1.0) < 1e-13
    # Condon-Shortley sign at l3 = l1 + l2
    assert np.sign(f[-1]) == (-1) ** (l1 - l2)


def _namaster_design(ells, nW):
    """Rows: l = 2..766 diagonal entries; columns: W at even l3 (odd l3 never reach a diagonal)."""
    evens = np.arange(0, nW, 2)
    A = {k: np.zeros((len(ells), len(evens))) for k in ("TT", "EE", "TE")}
    for r, l in enumerate(ells):
        _, f0 = o.w3j_family(l, l, 0, 0)
        _, f2 = o.w3j_family(l, l, -2, 2)
        top = min(2 * l, nW - 1)
        l3 = evens[evens <= top]
        w = (2 * l + 1) * (2 * l3 + 1) / (4 * math.pi)
        A["TT"][r, :len(l3)] = w * f0[l3] ** 2
        A["EE"][r, :len(l3)] = w * f2[l3] ** 2
        A["TE"][r, :len(l3)] = w * f0[l3] * f2[l3]
    return A


@pytest.mark.parametrize("fit,held", [(("TT", "EE"), "TE"), (("TT", "TE"), "EE"), (("EE", "TE"), "TT")])
def test_namaster_diagonals(fit, held):
    """The reference's NaMaster golden diagonals (TT, ++, TE of one mask, lmax 767, l3 <= 767)
    depend only on W at even l3 <= 767: 384 unknowns, 765 equations per spin case.  Fitting W
    on two spin cases and predicting the third checks the oracle's 00 and 22 families, the
    TE sign, the (2l3+1)/4pi weights and the parity rules against the reference's vectors."""
    gold = dict(np.load(os.path.join(GOLDEN, "namaster_diag.npz")))
    ells = np.arange(2, 767)
    A = _namaster_design(ells, 768)
    Afit = np.vstack([A[k] for k in fit])
    bfit = np.concatenate([gold[k] for k in fit])
    W, *_ = np.linalg.lstsq(Afit, bfit, rcond=None)
    for k in fit:
        assert np.max(np.abs(A[k] @ W / gold[k] - 1)) < 1e-12
    pred = A[held] @ W
    assert np.max(np.abs(pred / gold[held] - 1)) < 1e-11


def test_full_sky_identity():
    L = 48
    W = np.zeros(2 * L + 1)
    W[0] = 4 * math.pi
    I = np.eye(L + 1)
    assert np.allclose(o.inner_mcm(0, W, 0, L), I, atol=1e-14)
    for spin, want in ((1, I), (2, I), (3, 0 * I)):
        M = o.inner_mcm(spin, W, 0, L)
        assert np.allclose(M[2:, 2:], want[2:, 2:], atol=1e-14)
        assert not np.any(M[:2, :]) and not np.any(M[:, :2])  # l < 2 rows of spin-2 cases are defined as 0


def test_row_column_weights():
    L = 30
    W = np.abs(np.random.default_rng(0).standard_normal(2 * L + 1))
    for spin in range(4):
        M = o.inner_mcm(spin, W, 0, L)
        l = np.arange(L + 1)
        # M[l1,l2] = (2l2+1) Xi, M[l2,l1] = (2l1+1) Xi  (src/modecoupling.jl:90-91)
        assert np.allclose(M / (2 * l[None, :] + 1), (M / (2 * l[None, :] + 1)).T, rtol=1e-14, atol=0)


def test_oracle_fixture_stable():
    g = dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))
    L = 40
    for nWname in ("2L1", "L1"):
        for spin in range(4):
            M = o.inner_mcm(spin, g["W_" + nWname], 0, L)
            np.testing.assert_allclose(M, g["M%d_%s" % (spin, nWname)], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(o.inner_mcm(0, g["W_2L1"], 5, L), g["M0_lmin5"], rtol=1e-13, atol=1e-300)
    S = [g["cov_S%d" % i] for i in range(4)]
    R = [g["cov_R%d" % i] for i in range(4)]
    Ws = [g["cov_W%d" % k] for k in range(8)]
    for name in o.COV_KINDS:
        C = o.loop_cov(name, S, R[:o.COV_NRATIOS[name]], Ws[:o.COV_NWINDOWS[name]], 0, 32)
        np.testing.assert_allclose(C, g["cov_" + name], rtol=1e-13, atol=1e-300)


def test_lmin_submatrix():
    """lmin only crops the grid: the families do not depend on it."""
    g = dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))
    np.testing.assert_allclose(g["M0_lmin5"], g["M0_2L1"][5:, 5:], rtol=1e-15, atol=0)


def test_covariance_symmetric_and_reference_formula():
    """TTEE at one pair written out by hand from src/covariance.jl:438-441."""
    g = dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))
    S = [g["cov_S%d" % i] for i in range(4)]
    Ws = [g["cov_W%d" % k] for k in range(2)]
    C = o.loop_cov("TTEE", S, [], Ws, 0, 32)
    assert np.array_equal(C, C.T)
    X = [o.xi(0, 0, w, 0, 32) for w in Ws]
    a, b = 7, 19
    TEip, TEiq, TEjq, TEjp = S
    want = ((TEip[a] * TEjq[b] + TEjq[a] * TEip[b]) * X[0][a, b] + (TEiq[a] * TEjp[b] + TEjp[a] * TEiq[b]) * X[1][a, b]) / 2
    assert abs(C[a, b] - want) <= 1e-14 * abs(want)


@pytest.mark.parametrize("l1,l2,m1,m2", [(40, 37, -2, -4), (100, 90, 3, -1), (200, 250, -2, 4), (1000, 1003, -6, 2),
                                         (513, 600, 2, -6), (30, 30, -4, 4), (8, 9, -3, -3)])
def test_general_spin_families_vs_exact(l1, l2, m1, m2):
    """General (m1, m2, -m1-m2) families, as QuickPol uses, against the mpmath Racah sum."""
    exact3j = pytest.importorskip("oracle.exact3j")
    jmin, f = o.w3j_family(l1, l2, m1, m2)
    amp = 1.0 / math.sqrt(max((l1 + l2 + 1) ** 2 - jmin ** 2, 1))
    for k in np.unique(np.linspace(0, len(f) - 1, 10).astype(int)):
        ex = float(exact3j.w3j(l1, l2, jmin + int(k), m1, m2, -m1 - m2))
        assert abs(f[k] - ex) <= 1e-12 * max(abs(ex), amp)


def test_quickpol_oracle_diagonal_known_answer():
    lmax = 40
    W = np.zeros(2 * lmax + 1)
    W[0] = 3.0
    X = o.quickpol_xi(0, 0, 0, 0, W, lmax, 4, 4)
    l = np.arange(lmax + 1)
    np.testing.assert_allclose(np.diag(X)[2:], 3.0 / (2 * l[2:] + 1), rtol=1e-14)
    assert np.max(np.abs(X - np.diag(np.diag(X)))) < 1e-16


def test_alm2cl_oracle_against_direct_sum_over_m():
    """The oracle's alm2cl (vectorised over l) against the definition written as a sum over
    m = -l..l, with a_{l,-m} = (-1)^m conj(a_lm) for a real field."""
    lmax, mmax = 40, 25
    rng = np.random.default_rng(11)
    n = o.n_alms(lmax, mmax)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    a[:lmax + 1] = a[:lmax + 1].real
    b[:lmax + 1] = b[:lmax + 1].real
    cl = o.alm2cl(a, b, lmax, mmax)
    for l in range(lmax + 1):
        s = 0.0 + 0.0j
        for m in range(-min(l, mmax), min(l, mmax) + 1):
            i = o.alm_index(l, abs(m), lmax)
            am = a[i] if m >= 0 else (-1) ** m * np.conj(a[i])
            bm = b[i] if m >= 0 else (-1) ** m * np.conj(b[i])
            s += am * np.conj(bm)
        assert abs(s.imag) < 1e-12
        assert abs(cl[l] - s.real / (2 * l + 1)) < 1e-13 * max(1.0, abs(s.real))


def test_alm2cl_known_answers():
    lmax, mmax = 60, 20
    ones = np.ones(o.n_alms(lmax, mmax), dtype=complex)
    l = np.arange(lmax + 1)
    np.testing.assert_allclose(o.alm2cl(ones, ones, lmax, mmax), (1 + 2 * np.minimum(l, mmax)) / (2 * l + 1.0))
    # a field with one axisymmetric mode: a_l0 = c at l = 7 only -> cl[7] = c^2 / 15
    a = np.zeros(o.n_alms(lmax, lmax), dtype=complex)
    a[o.alm_index(7, 0, lmax)] = 3.0
    cl = o.alm2cl(a, a, lmax)
    assert cl[7] == 9.0 / 15 and np.count_nonzero(cl) == 1
    # window_function_W! mean: a zero (None) term counts
    np.testing.assert_allclose(o.window_function_W([a, None], [a, a], lmax), 0.5 * cl)


def test_quickpolW_is_alm2cl_times_2l_plus_1():
    lmax = 30
    rng = np.random.default_rng(2)
    n = o.n_alms(lmax, lmax)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    W = o.quickpolW(a, a, lmax)
    for l in (0, 5, 30):
        # m = 0 enters once as Re(a conj a) = |a_l0|^2, every m > 0 twice
        direct = abs(a[o.alm_index(l, 0, lmax)]) ** 2 + sum(2 * abs(a[o.alm_index(l, m, lmax)]) ** 2
                                                            for m in range(1, l + 1))
        assert abs(W[l] - direct) < 1e-12 * direct


def test_quickpol_common_match_agrees_with_own_midpoints():
    """The oracle's two QuickPol matches (each family at its own midpoint, as a family fill does;
    both families at the larger midpoint, as the GPU kernel does) give the same Xi up to the
    recurrences' conditioning, relative to the sum of |W f1 f2| behind each element."""
    rng = np.random.default_rng(5)
    lmax, bl, bu = 150, 12, 7
    W = rng.random(2 * lmax + 1) * np.exp(-np.arange(2 * lmax + 1) / 60.0)
    for (nu1, nu2, s1, s2) in ((0, 0, 2, 2), (1, -1, 2, 0), (-3, 1, 2, -2), (4, -4, 0, 2)):
        A = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu)
        B = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, common_match=True)
        S = o.quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, absolute=True)
        m = S > 0
        assert np.max(np.abs(A - B)[m] / S[m]) < 1e-9, (nu1, nu2, s1, s2)
        assert np.array_equal(A == 0, B == 0)  # the same band and the same zero families
