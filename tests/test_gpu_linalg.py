"""Dense solves downstream of the coupling matrices (GPU, cuSOLVER LU).

decouple_covmat: the reference's 3x3 known answer (test/test_covmat.jl:11-17,
copied to tests/golden/decouple_3x3.json) and its round-trip property
(test/test_covmat.jl:115-127): M * decouple(C, M, M) * M^T = C.
solve: M \\ pCl against numpy.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_decouple_known_answer(ctx):
    g = json.load(open(os.path.join(GOLDEN, "decouple_3x3.json")))
    A, B1, B2 = (np.array(g[k]) for k in ("A", "B1", "B2"))
    out = ctx.decouple_covmat(A, B1, B2)
    np.testing.assert_allclose(out, np.array(g["expected"]), rtol=1.5e-8, atol=0)  # Julia's default isapprox


def test_decouple_round_trip_with_coupling_matrix(ctx):
    from powerspectra_gpu import synthetic as syn
    L = 300
    W = syn.mask_spectrum(L + 1, 0.6, 100.0, seed=2)
    M = ctx.mcm(0, W, 2, L, mode="plain")
    rng = np.random.default_rng(0)
    X = rng.random(M.shape)
    C = X.T @ X
    D = ctx.decouple_covmat(C, M, M)
    np.testing.assert_allclose(M @ D @ M.T, C, rtol=1e-9, atol=1e-9 * np.abs(C).max())


def test_solve_matches_numpy(ctx):
    from powerspectra_gpu import synthetic as syn
    L = 400
    W = syn.mask_spectrum(L + 1, 0.6, 120.0, seed=5)
    M = ctx.mcm(0, W, 2, L, mode="chosen")
    b = np.random.default_rng(1).random(L - 1)
    x = ctx.solve(M, b)
    np.testing.assert_allclose(x, np.linalg.solve(M, b), rtol=1e-9, atol=1e-12)
    B = np.random.default_rng(2).random((L - 1, 3))
    np.testing.assert_allclose(ctx.solve(M, B), np.linalg.solve(M, B), rtol=1e-9, atol=1e-12)


def test_singular_is_an_argument_error(ctx):
    import powerspectra_gpu as pg
    Z = np.zeros((4, 4))
    with pytest.raises(pg.PowerSpectraArgumentError, match="singular"):
        ctx.decouple_covmat(np.eye(4), Z, np.eye(4))
    assert np.allclose(ctx.solve(np.eye(3) * 2, np.ones(3)), 0.5)  # context still usable


def test_decouple_device_matches_host(ctx):
    """ps_decouple_covmat_device on a covariance that stays on the GPU."""
    import torch
    from powerspectra_gpu import synthetic as syn
    L = 256
    W = syn.mask_spectrum(L + 1, 0.6, 100.0, seed=3)
    M = ctx.mcm(0, W, 2, L, mode="plain")
    rng = np.random.default_rng(4)
    X = rng.random(M.shape)
    C = X.T @ X
    n = M.shape[0]
    dC, dM = (torch.from_numpy(np.asfortranarray(x).ravel(order="F")).cuda() for x in (C, M))
    dout = torch.empty(n * (n + 3), dtype=torch.float64, device="cuda")  # ldout = n + 3
    ctx.decouple_covmat_device(dC.data_ptr(), dM.data_ptr(), dM.data_ptr(), n, n, dout.data_ptr(), n + 3)
    got = dout.cpu().numpy().reshape((n + 3, n), order="F")[:n]
    np.testing.assert_allclose(got, ctx.decouple_covmat(C, M, M), rtol=1e-12, atol=1e-14 * np.abs(got).max())
