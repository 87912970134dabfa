"""GPU parity of the mode-coupling kernels against the CPU oracle, through the C ABI.

Tolerance: the plain FP64 path must match the oracle (the FP64 restatement of
the reference algorithm) to 1e-12 relative per element.  Entries of the 00x22
(TE) case, and of any case when W has negative entries, can come from
cancelling sums; those are compared relative to the size of the sum of |terms|
(gpu_util.cond_scale), which equals |M| when nothing cancels.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import cond_scale, max_err_scaled, max_rel
from oracle import oracle as o

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _W(nW, seed=7, fsky=0.6, cutoff=None):
    from powerspectra_gpu import synthetic as syn
    return syn.mask_spectrum(nW, fsky, cutoff or max(nW / 3.0, 5.0), seed=seed)


@pytest.mark.parametrize("L,nWk,lmin", [(40, "2L1", 0), (40, "L1", 0), (97, "2L1", 3), (64, "short", 0),
                                         (33, "long", 2), (5, "2L1", 0), (0, "L1", 0), (1, "2L1", 0), (2, "2L1", 1)])
def test_each_spin_vs_oracle(ctx, L, nWk, lmin):
    nW = {"2L1": 2 * L + 1, "L1": L + 1, "short": max(L // 2, 1), "long": 3 * L + 7}[nWk]
    W = _W(nW)
    for spin in range(4):
        G = ctx.mcm(spin, W, lmin, L)
        R = o.inner_mcm(spin, W, lmin, L)
        err = max_err_scaled(G, R, cond_scale(spin, W, lmin, L))
        assert err < RTOL, (spin, err)


def test_golden_fixture(ctx):
    g = dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))
    for nWname in ("2L1", "L1"):
        W = g["W_" + nWname]
        for spin in range(4):
            G = ctx.mcm(spin, W, 0, 40)
            assert max_err_scaled(G, g["M%d_%s" % (spin, nWname)], cond_scale(spin, W, 0, 40)) < RTOL
    assert max_rel(ctx.mcm(0, g["W_2L1"], 5, 40), g["M0_lmin5"]) < RTOL


def test_multi_equals_single(ctx):
    L = 150
    Ws = {s: _W(2 * L + 1, seed=s + 3) for s in range(4)}
    multi = ctx.mcm_multi(Ws, 0, L)
    for s in range(4):
        single = ctx.mcm(s, Ws[s], 0, L)
        assert max_err_scaled(multi[s], single, cond_scale(s, Ws[s], 0, L)) < 1e-14


def test_negative_window_entries(ctx):
    """Cross-spectra can be negative: TT then has cancelling sums too."""
    L = 80
    W = _W(2 * L + 1) * np.where(np.arange(2 * L + 1) % 3 == 0, -1.0, 1.0)
    for spin in range(4):
        G = ctx.mcm(spin, W, 0, L)
        R = o.inner_mcm(spin, W, 0, L)
        assert max_err_scaled(G, R, cond_scale(spin, W, 0, L)) < RTOL


def test_full_sky_identity_at_3071(ctx):
    """W = 4 pi delta_l0 gives M00 = M02 = M++ = I (l >= 2) and M-- = 0, at the benchmark size."""
    L = 3071
    W = np.zeros(2 * L + 1)
    W[0] = 4 * math.pi
    M = ctx.mcm_multi({0: W, 1: W, 2: W, 3: W}, 0, L)
    I = np.eye(L + 1)
    assert np.max(np.abs(M[0] - I)) < 1e-12
    for s in (1, 2):
        assert np.max(np.abs(M[s][2:, 2:] - I[2:, 2:])) < 1e-12
        assert not np.any(M[s][:2, :]) and not np.any(M[s][:, :2])
    assert np.max(np.abs(M[3])) < 1e-12


def test_benchmark_size_sampled_rows(ctx):
    """All four spin cases at lmax 3071, nW 6143 (the benchmark workload): every element of a
    stratified sample of rows/columns against the oracle, plus the exact weight symmetry."""
    from powerspectra_gpu import synthetic as syn
    c = syn.all_spins(3071)
    Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
    G = ctx.mcm_multi(Ws, 0, 3071)
    rows = [0, 1, 2, 3, 17, 511, 1500, 2047, 3000, 3070, 3071]
    l = np.arange(3072)
    for s in range(4):
        R = o.inner_mcm(s, Ws[s], 0, 3071, rows=rows)
        S = cond_scale(s, Ws[s], 0, 3071, rows=rows)
        for r in rows:
            assert max_err_scaled(G[s][r, r:], R[r, r:], S[r, r:]) < RTOL, (s, r)
            assert max_err_scaled(G[s][r:, r], R[r:, r], S[r:, r]) < RTOL, (s, r)
        X = G[s] / (2 * l[None, :] + 1)
        assert np.max(np.abs(X - X.T)) <= 1e-15 * np.max(np.abs(X))


def test_argument_errors(ctx):
    import powerspectra_gpu as pg
    W = np.ones(50)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm(0, W, 5, 4)  # lmin > lmax
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm(0, W, -1, 4)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm(7, W, 0, 4)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm(0, W, 0, 20000)  # beyond the supported lmax
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm(0, W, 0, 10, out=np.zeros((5, 5), order="F"))  # leading dimension too small
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm_multi({}, 0, 10)
    # the context stays usable after errors
    assert max_rel(ctx.mcm(0, W, 0, 10), o.inner_mcm(0, W, 0, 10)) < RTOL


def test_device_entry_point(ctx):
    torch = pytest.importorskip("torch")
    L = 120
    Ws = {s: _W(2 * L + 1, seed=10 + s) for s in range(4)}
    dW = {s: torch.tensor(Ws[s], device="cuda") for s in range(4)}
    n = L + 1
    dM = {s: torch.zeros((n, n), dtype=torch.float64, device="cuda") for s in range(4)}  # row-major n x n
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.mcm_multi_device({s: dW[s].data_ptr() for s in range(4)}, 2 * L + 1, 0, L,
                             {s: dM[s].data_ptr() for s in range(4)}, n)
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    for s in range(4):
        got = dM[s].cpu().numpy().T  # column-major on the device = transpose of the row-major view
        assert max_err_scaled(got, o.inner_mcm(s, Ws[s], 0, L), cond_scale(s, Ws[s], 0, L)) < RTOL


def test_host_mirror_blocks(ctx):
    import powerspectra_gpu as pg
    L = 60
    W = _W(L + 1)
    ee_bb, eb_be = pg.mcm(("EE_BB", "EB_BE"), W, lmin=2, ctx=ctx)
    Mpp = o.inner_mcm(2, W, 2, L)
    Mmm = o.inner_mcm(3, W, 2, L)
    for blk, sgn in ((ee_bb, 1), (eb_be, -1)):
        assert max_rel(blk.getblock(0, 0).parent, Mpp) < RTOL
        assert max_rel(blk.getblock(1, 1).parent, Mpp) < RTOL
        assert max_rel(blk.getblock(0, 1).parent, sgn * Mmm) < RTOL
        assert max_rel(blk.getblock(1, 0).parent, sgn * Mmm) < RTOL
    M = pg.mcm("TT", W, lmin=2, ctx=ctx)
    assert M.axes == (range(2, L + 1), range(2, L + 1))
    assert max_rel(M.parent, o.inner_mcm(0, W, 2, L)) < RTOL
    S1 = cond_scale(1, W, 0, L)
    for spec in ("TE", "ET", "TB", "BT"):
        assert max_err_scaled(pg.mcm(spec, W, ctx=ctx).parent, o.inner_mcm(1, W, 0, L), S1) < RTOL


def test_launch_count_and_timing(ctx):
    W = _W(41)
    n0 = ctx.launch_count()
    ctx.mcm(0, W, 0, 20)
    assert ctx.launch_count() > n0
    assert ctx.last_kernel_ms() >= 0.0


@pytest.mark.parametrize("mode", ["plain", "chosen"])
def test_pinned_host_outputs_written_in_place(ctx, mode):
    """Outputs in page-locked host memory are written by the kernel directly (no staging copy);
    the result equals the pageable-output path bit for bit."""
    import torch
    from powerspectra_gpu import synthetic as syn
    L = 300
    c = syn.all_spins(L)
    Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
    n = L + 1
    pinned = {s: torch.full((n, n), np.nan, dtype=torch.float64).pin_memory().numpy().T for s in Ws}
    pageable = ctx.mcm_multi(Ws, 0, L, mode=mode)
    got = ctx.mcm_multi(Ws, 0, L, mode=mode, outs=pinned)
    for s in Ws:
        assert got[s] is pinned[s]
        assert np.array_equal(pinned[s], pageable[s])


def test_fma_probe_and_instrumentation(ctx):
    """The FMA-chain probe behind the bench roofline: both rates positive, FP32 far above FP64 on
    this part; kernel timing and launch counting advance with a call."""
    f64, f32 = ctx.fma_peak(fp64=True), ctx.fma_peak(fp64=False)
    assert f64 > 0 and f32 > 8 * f64
    n0 = ctx.launch_count()
    W = np.ones(41)
    ctx.mcm(0, W, 0, 20, mode="chosen")
    assert ctx.launch_count() > n0 and ctx.last_kernel_ms() > 0
