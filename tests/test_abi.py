"""CPU checks of the C ABI library and the host-side mirror (no GPU needed)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _header_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(ps_[A-Za-z0-9_]+)\s*\(", txt):
            syms.add(m.group(1))
    return syms


@pytest.fixture(scope="module")
def lib():
    import build as b  # powerspectra.jl_gb300/build.py
    b.build()
    import powerspectra_gpu as pg
    return pg.load()


def test_exports_every_header_symbol(lib):
    syms = _header_symbols()
    assert len(syms) >= 14
    for s in sorted(syms):
        assert hasattr(lib, s), "symbol %s declared in include/ but not exported" % s
    from powerspectra_gpu._lib import EXPORTS
    assert set(EXPORTS) == syms


def test_null_context_is_an_argument_error(lib):
    import powerspectra_gpu._lib as L
    W = np.ones(10)
    M = np.zeros((5, 5), order="F")
    st = lib.ps_mcm(None, 0, L.dptr(W), 10, 0, 4, 0, L.dptr(M), 5)
    assert st == L.PS_ERR_ARG
    assert lib.ps_last_error(None) == b"null context"
    assert lib.ps_launch_count(None) == 0
    assert lib.ps_last_kernel_ms(None) < 0


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = lib.ps_create(0, ctypes.byref(h))
    assert st != 0 and not h.value


def test_unknown_spec_raises_argument_error():
    import powerspectra_gpu as pg
    with pytest.raises(ValueError, match="not a valid spectrum"):
        pg.mcm("XY", np.ones(20), lmax=10)
    with pytest.raises(ValueError):
        pg.mcm("TT", np.ones(5), lmax=10)  # fewer than lmax+1 entries


def test_tuple_spec_other_than_eebb_returns_none():
    import powerspectra_gpu as pg
    assert pg.mcm(("TT", "TE"), np.ones(20), lmax=10) is None


def test_spectral_array_indexing():
    from powerspectra_gpu import SpectralArray, spectralzeros, BlockSpectralMatrix
    A = spectralzeros(range(2, 6), range(2, 6))
    A[3, 5] = 7.0
    assert A.parent[1, 3] == 7.0 and A[3, 5] == 7.0
    assert A.parent.flags.f_contiguous
    with pytest.raises(IndexError):
        A[1, 2]
    B = SpectralArray(np.arange(16.0).reshape(4, 4), (range(2, 6), range(2, 6)))
    blk = BlockSpectralMatrix.hvcat([[A, B], [B, A]])
    assert blk.shape == (8, 8)
    np.testing.assert_array_equal(blk.getblock(0, 1).parent, B.parent)
    assert blk.getblock(1, 0).axes == (range(2, 6), range(2, 6))


def test_coupledcov_unknown_pair_prints_and_returns_none(capsys):
    import powerspectra_gpu as pg
    ws = pg.WindowWorkspace(("a", "b", "c", "d"), 10, lambda *k: np.ones(11))
    assert pg.coupledcov("BB", "TT", ws, {}) is None
    assert "BB,TT not implemented" in capsys.readouterr().out


def test_synthetic_forms():
    from powerspectra_gpu import synthetic as syn
    W = syn.mask_spectrum(100, 0.6, 300.0, seed=0)
    assert abs(W[0] - 0.36 * 4 * np.pi) < 1e-2
    assert np.all(W[1:] > 0)
    c = syn.all_spins(lmax=31)
    assert c["nW"] == 63 and len(c["WT"]) == 63
    ws, spectra, noise = syn.covariance_inputs(lmax=20)
    w1 = ws.window_function_W("∅∅", "∅∅", "a", "b", "TT", "c", "d", "TT")
    w2 = ws.window_function_W("∅∅", "∅∅", "a", "b", "TT", "c", "d", "TT")
    assert np.array_equal(w1, w2) and len(w1) == 21


def test_bench_work_accounting_matches_oracle():
    import bench
    from oracle import oracle as o
    for (lmin, lmax, nW) in ((0, 100, 201), (0, 100, 101), (3, 57, 40)):
        assert bench.l3_terms(lmin, lmax, nW) == int(o.l3_terms(lmin, lmax, nW))
    wl = bench.workload("all_spins_3071")
    assert wl["nW"] == 6143 and sorted(wl["Ws"]) == [0, 1, 2, 3]
    # fixed accounting: 9 (00) + 16 (22) + 3 per distinct spectrum
    assert bench.flops_per_step(wl, 1) == 9 + 16 + 3 * 3
    # the default workload: 20 spectra at lmax 8191, TT / ++ / -- by k % 3, 20 matrices
    big = bench.workload("large_8191")
    assert big["lmax"] == 8191 and big["nW"] == 16383 and len(big["windows"]) == 20
    assert [s for _, s in big["slots"]] == [(0, 2, 3)[k % 3] for k in range(20)]
    assert bench.flops_per_step(big, 1) == 9 + 16 + 3 * 20


def test_result_matrix_checks_caller_outputs():
    import numpy as np
    from powerspectra_gpu import _lib as L
    ok = np.empty((3, 3), order="F")
    assert L._result_matrix(ok, 3) is ok
    assert L._result_matrix(None, 4).shape == (4, 4)
    for bad in (np.empty((3, 3)), np.empty((3, 4), order="F"), np.empty((3, 3), dtype=np.float32, order="F")):
        with pytest.raises(L.PowerSpectraArgumentError):
            L._result_matrix(bad, 3)
