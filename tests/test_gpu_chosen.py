"""The chosen form (FP32-pipe recurrences with two-word compensation and
block-floating-point windows) against FP64: the oracle at small sizes, the
plain FP64 GPU kernel at the benchmark sizes.

Bar: max elementwise relative error <= 1e-6 for every matrix (TE and
cancelling elements relative to the sum of |terms|, see gpu_util).
"""
import math

import numpy as np
import pytest

from gpu_util import cond_scale, cov_scale, gpu_cond_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu
TOL = 1e-6


def _W(nW, seed=7, fsky=0.6, cutoff=None):
    from powerspectra_gpu import synthetic as syn
    return syn.mask_spectrum(nW, fsky, cutoff or max(nW / 3.0, 5.0), seed=seed)


@pytest.mark.parametrize("L,nWk,lmin", [(40, "2L1", 0), (40, "L1", 0), (97, "2L1", 3), (64, "short", 0),
                                         (5, "2L1", 0), (0, "L1", 0), (1, "2L1", 0), (2, "2L1", 1), (200, "2L1", 0)])
def test_chosen_vs_oracle_small(ctx, L, nWk, lmin):
    nW = {"2L1": 2 * L + 1, "L1": L + 1, "short": max(L // 2, 1)}[nWk]
    W = _W(nW)
    for spin in range(4):
        G = ctx.mcm(spin, W, lmin, L, mode="chosen")
        R = o.inner_mcm(spin, W, lmin, L)
        err = max_err_scaled(G, R, cond_scale(spin, W, lmin, L))
        assert err < TOL, (spin, err)


def test_chosen_benchmark_size_vs_plain(ctx):
    """All spin cases at lmax 3071, nW 6143: every element against the plain FP64 kernel."""
    from powerspectra_gpu import synthetic as syn
    c = syn.all_spins(3071)
    Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
    P = ctx.mcm_multi(Ws, 0, 3071, mode="plain")
    C = ctx.mcm_multi(Ws, 0, 3071, mode="chosen")
    errs = {}
    for s in range(4):
        errs[s] = max_err_scaled(C[s], P[s], gpu_cond_scale(ctx, s, Ws[s], 0, 3071))
    assert max(errs.values()) < TOL, errs


def test_chosen_wide_dynamic_range(ctx):
    """Windows spanning ~1e-97 (beyond FP32's range) keep full relative precision."""
    L = 1500
    l = np.arange(2 * L + 1, dtype=np.float64)
    W = 1e-3 * (l + 1) ** -2 * np.exp(-l * (l + 1) / (2 * 150.0 ** 2))
    W[0] += 4 * math.pi * 0.3
    assert W[-1] < 1e-90 and W[-1] > 0
    P = ctx.mcm_multi({0: W, 2: W, 3: W}, 0, L, mode="plain")
    C = ctx.mcm_multi({0: W, 2: W, 3: W}, 0, L, mode="chosen")
    for s in (0, 2, 3):
        assert max_err_scaled(C[s], P[s], np.abs(P[s])) < TOL, s


def test_chosen_negative_windows(ctx):
    L = 300
    W = _W(2 * L + 1) * np.where(np.arange(2 * L + 1) % 5 == 0, -1.0, 1.0)
    for spin in range(4):
        G = ctx.mcm(spin, W, 0, L, mode="chosen")
        R = o.inner_mcm(spin, W, 0, L)
        assert max_err_scaled(G, R, cond_scale(spin, W, 0, L)) < TOL, spin


@pytest.mark.parametrize("kind", list(o.COV_KINDS))
def test_chosen_covariance(ctx, kind):
    from powerspectra_gpu import synthetic as syn
    L = 300
    spectra, noise = syn.signal_spectra(L)
    f = syn.FIELDS
    S = [spectra["TT", f[0], f[2]], spectra["EE", f[1], f[3]], spectra["TE", f[0], f[3]], spectra["TE", f[1], f[2]]]
    R = [noise["TT", f[0], f[0]], noise["EE", f[1], f[1]], noise["TT", f[0], f[2]], noise["EE", f[1], f[3]]]
    R = R[:o.COV_NRATIOS[kind]]
    Ws = [syn.window_for_key(("c", k), L) for k in range(o.COV_NWINDOWS[kind])]
    C = ctx.coupledcov(kind, S, R, Ws, 0, L, mode="chosen")
    ref = o.loop_cov(kind, S, R, Ws, 0, L)
    assert max_err_scaled(C, ref, cov_scale(kind, S, R, Ws, 0, L)) < TOL


def test_chosen_lmax_8191_sampled_rows(ctx):
    """lmax 8191, nW 16383 (the large configuration's grid): sampled rows of TT, ++, -- against the oracle."""
    from powerspectra_gpu import synthetic as syn
    big = syn.large_set(K=3)
    L, Ws = big["lmax"], big["W"]
    rows = [2, 700, 4095, 8000, 8191]
    C = ctx.mcm_multi({0: Ws[0], 2: Ws[1], 3: Ws[2]}, 0, L, mode="chosen")
    for s, W in ((0, Ws[0]), (2, Ws[1]), (3, Ws[2])):
        R = o.inner_mcm(s, W, 0, L, rows=rows)
        for r in rows:
            assert max_err_scaled(C[s][r, r:], R[r, r:], np.abs(R[r, r:])) < TOL, (s, r)
            assert max_err_scaled(C[s][r:, r], R[r:, r], np.abs(R[r:, r])) < TOL, (s, r)


def test_chosen_at_the_largest_lmax(ctx):
    """lmax 16383 (the largest the library accepts), nW 32767, TT and ++ from one window pass:
    sampled rows against the oracle.  At this size the integer factors of the step coefficients
    reach 2^16 and their products 2^64, the edge of what the float-float tables are built for."""
    from powerspectra_gpu import synthetic as syn
    L = 16383
    W = syn.mask_spectrum(2 * L + 1, 0.6, 1500.0, seed=16383)
    rows = [2, 9000, 16383]
    C = ctx.mcm_multi({0: W, 2: W}, 0, L, mode="chosen")
    for s in (0, 2):
        R = o.inner_mcm(s, W, 0, L, rows=rows)
        for r in rows:
            assert max_err_scaled(C[s][r, r:], R[r, r:], np.abs(R[r, r:])) < TOL, (s, r)
            assert max_err_scaled(C[s][r:, r], R[r:, r], np.abs(R[r:, r])) < TOL, (s, r)
