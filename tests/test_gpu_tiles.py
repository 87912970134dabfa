"""The chosen kernel's tiled task list: four rows per block over one 32-column
block counted back from lmax, rows below lmin idle, lanes left of the diagonal
idle, and each tile's row halves written through shared memory.  Grids whose
size is not a multiple of 4 or 32 and lmin > 0 exercise every partial tile;
padded leading dimensions check that nothing outside the matrix is written;
page-locked host outputs take the in-place write path; the allocation-free
entry point fills the same list on the device."""
import ctypes

import numpy as np
import pytest

from gpu_util import cond_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-6
GRIDS = [(0, 2), (1, 4), (3, 7), (0, 31), (1, 33), (5, 40), (2, 67), (7, 100), (0, 128), (30, 61)]


def _windows(lmax, seed):
    from powerspectra_gpu import synthetic as syn
    nW = 2 * lmax + 1
    return [syn.mask_spectrum(nW, 0.5 + 0.1 * s, 0.3 * lmax + 20, seed=seed + s) for s in range(4)]


@pytest.mark.parametrize("lmin,lmax", GRIDS)
def test_tiled_grids_vs_oracle(ctx, lmin, lmax):
    Ws = _windows(lmax, lmin + 7 * lmax)
    got = ctx.mcm_multi({s: Ws[s] for s in range(4)}, lmin, lmax, mode="chosen")
    for s in range(4):
        ref = o.inner_mcm(s, Ws[s], lmin, lmax)
        assert max_err_scaled(got[s], ref, cond_scale(s, Ws[s], lmin, lmax)) < TOL, (lmin, lmax, s)


@pytest.mark.parametrize("lmin,lmax", [(3, 7), (1, 33), (2, 67)])
def test_tiled_padded_leading_dimension(ctx, lmin, lmax):
    Ws = _windows(lmax, 100 + lmax)
    n, pad = lmax - lmin + 1, 5
    dW = {s: torch.tensor(Ws[s], device="cuda") for s in range(4)}
    dM = {s: torch.full((n, n + pad), float("nan"), dtype=torch.float64, device="cuda") for s in range(4)}
    ctx.mcm_multi_device({s: dW[s].data_ptr() for s in range(4)}, len(Ws[0]), lmin, lmax,
                         {s: dM[s].data_ptr() for s in range(4)}, n + pad, mode="chosen")
    torch.cuda.synchronize()
    for s in range(4):
        full = dM[s].cpu().numpy()  # row j holds column j of the matrix, then the padding
        assert np.all(np.isnan(full[:, n:])), (lmin, lmax, s)
        got = full[:, :n].T
        ref = o.inner_mcm(s, Ws[s], lmin, lmax)
        assert max_err_scaled(got, ref, cond_scale(s, Ws[s], lmin, lmax)) < TOL, (lmin, lmax, s)


@pytest.mark.parametrize("lmin,lmax", [(0, 31), (5, 40), (7, 100)])
def test_tiled_page_locked_outputs_match_pageable(ctx, lmin, lmax):
    Ws = _windows(lmax, 300 + lmax)
    n = lmax - lmin + 1
    pinned = {s: torch.full((n, n), float("nan"), dtype=torch.float64).pin_memory().numpy().T for s in range(4)}
    a = ctx.mcm_multi({s: Ws[s] for s in range(4)}, lmin, lmax, mode="chosen", outs=pinned)
    b = ctx.mcm_multi({s: Ws[s] for s in range(4)}, lmin, lmax, mode="chosen")
    for s in range(4):
        assert np.array_equal(a[s], b[s]), (lmin, lmax, s)


@pytest.mark.parametrize("kind", ["TTTT", "TETE", "TEEE"])
def test_tiled_covariance_partial_tiles(ctx, kind):
    from powerspectra_gpu import synthetic as syn
    lmin, lmax = 3, 45
    spectra, noise = syn.signal_spectra(lmax)
    f = syn.FIELDS
    S = [spectra["TT", f[0], f[2]], spectra["EE", f[1], f[3]], spectra["TE", f[0], f[3]], spectra["TE", f[1], f[2]]]
    R = [noise["TT", f[0], f[0]], noise["EE", f[1], f[1]], noise["TT", f[0], f[2]], noise["EE", f[1], f[3]]]
    R = R[:o.COV_NRATIOS[kind]]
    Ws = [syn.window_for_key(("tile", k), lmax) for k in range(o.COV_NWINDOWS[kind])]
    C = ctx.coupledcov(kind, S, R, Ws, lmin, lmax, mode="chosen")
    ref = o.loop_cov(kind, S, R, Ws, lmin, lmax)
    scale = o.loop_cov(kind, S, R, Ws, lmin, lmax, absolute=True)
    assert max_err_scaled(C, ref, scale) < TOL
    assert np.array_equal(C, C.T)


def test_noalloc_partial_tiles_match_context_path(ctx):
    import powerspectra_gpu._lib as L
    lib = L.load()
    fn = lib.ps_mcm_multi_device_noalloc
    fn.argtypes = [ctypes.c_uint, L._DPP, ctypes.c_int64, ctypes.c_int, ctypes.c_int, L._DPP, ctypes.c_int64,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    try:
        for (lmin, lmax) in ((3, 37), (1, 64), (6, 6)):
            Ws = _windows(lmax, 500 + lmax)
            n = lmax - lmin + 1
            dW = [torch.tensor(w, device="cuda") for w in Ws]
            new = [torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda") for _ in range(4)]
            ref = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for _ in range(4)]
            st = fn(0xF, L.dptr_array([d.data_ptr() for d in dW]), len(Ws[0]), lmin, lmax,
                    L.dptr_array([m.data_ptr() for m in new]), n, ctypes.c_void_p(stream.cuda_stream))
            assert st == 0
            ctx.mcm_multi_device({s: dW[s].data_ptr() for s in range(4)}, len(Ws[0]), lmin, lmax,
                                 {s: ref[s].data_ptr() for s in range(4)}, n, mode="chosen")
            torch.cuda.synchronize()
            for s in range(4):
                assert torch.equal(new[s], ref[s]), (lmin, lmax, s)
    finally:
        ctx.set_stream(0)
