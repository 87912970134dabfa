"""GPU parity of the covariance and Xi kernels against the CPU oracle, through the C ABI."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import cov_scale, max_err_scaled, max_rel
from oracle import oracle as o

pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.mark.parametrize("kind", list(o.COV_KINDS))
def test_cov_kinds_vs_fixture_and_oracle(ctx, kind):
    g = dict(np.load(os.path.join(GOLDEN, "oracle_small.npz")))
    S = [g["cov_S%d" % i] for i in range(4)]
    R = [g["cov_R%d" % i] for i in range(4)][:o.COV_NRATIOS[kind]]
    Ws = [g["cov_W%d" % k] for k in range(8)][:o.COV_NWINDOWS[kind]]
    C = ctx.coupledcov(kind, S, R, Ws, 0, 32)
    assert max_err_scaled(C, g["cov_" + kind], cov_scale(kind, S, R, Ws, 0, 32)) < RTOL
    assert np.array_equal(C, C.T)
    C2 = ctx.coupledcov(kind, S, R, Ws, 3, 32)
    assert max_err_scaled(C2, o.loop_cov(kind, S, R, Ws, 3, 32), cov_scale(kind, S, R, Ws, 3, 32)) < RTOL


@pytest.mark.parametrize("kind", list(o.COV_KINDS))
def test_cov_kinds_at_400(ctx, kind):
    from powerspectra_gpu import synthetic as syn
    L = 400
    spectra, noise = syn.signal_spectra(L)
    f = syn.FIELDS
    S = [spectra["TT", f[0], f[2]], spectra["EE", f[1], f[3]], spectra["TE", f[0], f[3]], spectra["TE", f[1], f[2]]]
    R = [noise["TT", f[0], f[0]], noise["EE", f[1], f[1]], noise["TT", f[0], f[2]], noise["EE", f[1], f[3]]]
    R = R[:o.COV_NRATIOS[kind]]
    Ws = [syn.window_for_key(("t", k), L) for k in range(o.COV_NWINDOWS[kind])]
    C = ctx.coupledcov(kind, S, R, Ws, 0, L)
    assert max_err_scaled(C, o.loop_cov(kind, S, R, Ws, 0, L), cov_scale(kind, S, R, Ws, 0, L)) < RTOL


@pytest.mark.parametrize("product,parity", [(0, 0), (0, 1), (1, 1), (1, 2), (1, 0), (2, 1), (2, 0)])
def test_xi_vs_oracle(ctx, product, parity):
    from powerspectra_gpu import synthetic as syn
    L = 90
    Ws = [syn.mask_spectrum(2 * L + 1, 0.5 + 0.05 * k, 40.0, seed=k) for k in range(3)]
    Xs = ctx.xi(product, parity, Ws, 0, L)
    spin_of = {(0, 0): 0, (0, 1): 0, (1, 1): 2, (1, 2): 3, (2, 1): 1}
    for X, W in zip(Xs, Ws):
        ref = o.xi(product, parity, W, 0, L)
        if (product, parity) in spin_of:
            l = np.arange(L + 1)
            scale = o.inner_mcm(spin_of[product, parity], W, 0, L, absolute=True) / (2 * l[None, :] + 1)
            assert max_err_scaled(X, ref, scale) < RTOL
        else:
            assert max_rel(X, ref, 1e-9) < RTOL


def test_coupledcov_mirror_matches_oracle_gathering(ctx):
    import powerspectra_gpu as pg
    from powerspectra_gpu import synthetic as syn
    L = 120
    ws, spectra, noise = syn.covariance_inputs(L)
    i, j, p, q = ws.field_names
    Wf = ws.window_function_W
    for (a, b) in syn.COV_BLOCKS:
        C = pg.coupledcov(a, b, ws, spectra, noise, ctx=ctx)
        assert C.parent.shape == (L + 1, L + 1)
    # TTEE by hand: spectra and windows in the reference's gathering order (src/covariance.jl:405-418)
    C = pg.coupledcov("TT", "EE", ws, spectra, noise, ctx=ctx)
    S = [spectra["TE", i, p], spectra["TE", i, q], spectra["TE", j, q], spectra["TE", j, p]]
    Ws = [Wf("∅∅", "∅∅", i, p, "TP", j, q, "TP"), Wf("∅∅", "∅∅", i, q, "TP", j, p, "TP")]
    assert max_err_scaled(C.parent, o.loop_cov("TTEE", S, [], Ws, 0, L), cov_scale("TTEE", S, [], Ws, 0, L)) < RTOL
    # default noise ratios are ones (ConstantDict, src/covariance.jl:41-45)
    C1 = pg.coupledcov("TT", "TT", ws, spectra, ctx=ctx)
    one = np.ones(L + 1)
    S = [spectra["TT", i, p], spectra["TT", j, q], spectra["TT", i, q], spectra["TT", j, p]]
    keys = [("∅∅", "∅∅", i, p, "TT", j, q, "TT"), ("∅∅", "∅∅", i, q, "TT", j, p, "TT"),
            ("∅∅", "TT", i, p, "TT", j, q, "TT"), ("∅∅", "TT", j, q, "TT", i, p, "TT"),
            ("∅∅", "TT", i, q, "TT", j, p, "TT"), ("∅∅", "TT", j, p, "TT", i, q, "TT"),
            ("TT", "TT", i, p, "TT", j, q, "TT"), ("TT", "TT", i, q, "TT", j, p, "TT")]
    Wl = [Wf(*k) for k in keys]
    ref = o.loop_cov("TTTT", S, [one] * 4, Wl, 0, L)
    assert max_err_scaled(C1.parent, ref, cov_scale("TTTT", S, [one] * 4, Wl, 0, L)) < RTOL


def test_cov_argument_errors(ctx):
    import powerspectra_gpu as pg
    one = np.ones(11)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.coupledcov(9, [one] * 4, [], [one] * 2, 0, 10)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.coupledcov("TTEE", [one[:5]] * 4, [], [one] * 2, 0, 10)  # spectra shorter than lmax+1
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.coupledcov("TTEE", [one] * 4, [], [one] * 3, 0, 10)  # wrong window count


def test_pinned_host_output_written_in_place(ctx):
    """A page-locked covariance output is written by the kernel directly; same bits as the
    pageable path."""
    import torch
    import powerspectra_gpu as pg
    from powerspectra_gpu import synthetic as syn
    L = 200
    ws, spectra, noise = syn.covariance_inputs(L)
    kind, S, R, Ws = pg.covariance.gather("TE", "TE", ws, spectra, noise)
    ref = ctx.coupledcov(kind, S, R, Ws, 0, L, mode="chosen")
    pinned = torch.full((L + 1, L + 1), np.nan, dtype=torch.float64).pin_memory().numpy().T
    got = ctx.coupledcov(kind, S, R, Ws, 0, L, mode="chosen", out=pinned)
    assert got is pinned and np.array_equal(pinned, ref)


def test_xi_pinned_outputs(ctx):
    """ps_xi writes page-locked outputs in place; same bits as the staged path."""
    import torch
    from powerspectra_gpu import synthetic as syn
    L = 120
    Ws = [syn.mask_spectrum(2 * L + 1, 0.5, 50.0, seed=k) for k in range(3)]
    ref = ctx.xi(1, 1, Ws, 0, L, mode="chosen")
    pinned = [torch.full((L + 1, L + 1), np.nan, dtype=torch.float64).pin_memory().numpy().T for _ in Ws]
    got = ctx.xi(1, 1, Ws, 0, L, mode="chosen", outs=pinned)
    for g, p, r in zip(got, pinned, ref):
        assert g is p and np.array_equal(p, r)
