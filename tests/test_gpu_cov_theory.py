"""Covariance blocks on the reference test suite's spectra (test/data/theory.csv, noise.csv,
copied to tests/golden/theory_noise.npz), with the inputs built the way the reference's
"isotropic noise limit" test builds them (test/test_covmat.jl:27-83): two half-mission fields,
every signal spectrum the same theory curve, noise ratios sqrt(N_l / N_white) on the auto
spectra and ones on the crosses, N_white the pixel area of an nside-256 map.  The masks of that
test are not shipped, so seeded mask spectra stand in for its windows.  Every block is checked
against the oracle: plain FP64 to 1e-12 and chosen to 1e-6 of the sum of |terms|."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import cov_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu

L = 767
F1, F2 = "143_hm1", "143_hm2"


def _inputs():
    import powerspectra_gpu as pg
    from powerspectra_gpu import synthetic as syn
    d = np.load(os.path.join(GOLDEN, "theory_noise.npz"))
    n_white = 4.0 * math.pi / (12 * 256 ** 2)  # pixsize of the nside-256 test maps
    one = np.ones(L + 1)
    spectra, ratios = {}, {}
    for a in (F1, F2):
        for b in (F1, F2):
            spectra["TT", a, b] = d["cltt"]
            spectra["EE", a, b] = d["clee"]
            spectra["TE", a, b] = d["clte"]
            ratios["TT", a, b] = np.sqrt(d["nltt"] / n_white) if a == b else one
            ratios["EE", a, b] = np.sqrt(d["nlee"] / n_white) if a == b else one
    ws = pg.WindowWorkspace((F1, F2, F1, F2), L, lambda *key: syn.window_for_key(key, L))
    return ws, spectra, ratios


@pytest.mark.parametrize("mode,tol", [("plain", 1e-12), ("chosen", 1e-6)])
@pytest.mark.parametrize("block", [("TT", "TT"), ("TT", "TE"), ("TE", "TE"), ("TT", "EE"), ("EE", "EE"),
                                   ("TE", "EE", False), ("TE", "EE", True)])
def test_theory_spectra_blocks(ctx, block, mode, tol):
    import powerspectra_gpu as pg
    ws, spectra, ratios = _inputs()
    ch1, ch2 = block[0], block[1]
    if len(block) == 3:
        planck = block[2]
        C = pg.spectralzeros(range(0, L + 1), range(0, L + 1))
        pg.covariance.coupledcovTEEE(C, ws, spectra, ratios, planck=planck, mode=mode, ctx=ctx)
        kind, S, R, Ws = pg.covariance.gather(ch1, ch2, ws, spectra, ratios, planck=planck)
    else:
        C = pg.coupledcov(ch1, ch2, ws, spectra, ratios, mode=mode, ctx=ctx)
        kind, S, R, Ws = pg.covariance.gather(ch1, ch2, ws, spectra, ratios)
    ref = o.loop_cov(kind, S, R, Ws, 0, L)
    assert max_err_scaled(C.parent, ref, cov_scale(kind, S, R, Ws, 0, L)) < tol
    assert np.allclose(C.parent, C.parent.T, rtol=0, atol=0)  # symmetric, as the reference fills it
