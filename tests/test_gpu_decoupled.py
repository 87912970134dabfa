"""The decoupled spectrum: the error of the chosen form in what a user of `master`
consumes, C = M \\ pCl (src/modecoupling.jl:358, src/blockspectralmatrix.jl:124-129).

pCl = M_fp64 C_true is built from the FP64 matrix, then decoupled with the
chosen M and with the FP64 M by ps_solve (FP64 LU on the GPU).  An elementwise
error of at most 1e-6 in M can grow by the condition number of M in the
solution; for these masks (f_sky 0.5-0.7) the measured growth is small, and
the bar is 1e-5 relative per multipole, for TT (M00), TE (M02) and the EE/BB
2x2 block [[M++, M--], [M--, M++]] on l >= 2 (the block of mcm(:EE_BB),
src/modecoupling.jl:210-216).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
BAR = 1e-5


def _spectra(ls):
    base = ((ls + 2.0) / 80.0) ** -2.4
    return {"TT": 1000.0 * base, "EE": 40.0 * base, "BB": 4.0 * base, "TE": 200.0 * base}


@pytest.mark.parametrize("L", [767, 1535])
def test_decoupled_chosen_vs_fp64(ctx, L):
    from powerspectra_gpu import synthetic as syn
    c = syn.all_spins(L, seed=11)
    Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
    P = ctx.mcm_multi(Ws, 0, L, mode="plain")
    G = ctx.mcm_multi(Ws, 0, L, mode="chosen")
    C = _spectra(np.arange(0, L + 1, dtype=np.float64))

    def decouple_err(Mc, Mp, truth):
        p = Mp @ truth
        xc, xp = ctx.solve(Mc, p), ctx.solve(Mp, p)
        assert np.max(np.abs(xp - truth) / np.abs(truth)) < 1e-9  # the FP64 solve recovers C_true
        return float(np.max(np.abs(xc - xp) / np.abs(xp)))

    errs = {"TT": decouple_err(G[0], P[0], C["TT"]),
            "TE": decouple_err(G[1][2:, 2:], P[1][2:, 2:], C["TE"][2:])}
    blk = lambda M: np.block([[M[2][2:, 2:], M[3][2:, 2:]], [M[3][2:, 2:], M[2][2:, 2:]]])
    errs["EE_BB"] = decouple_err(blk(G), blk(P), np.concatenate([C["EE"][2:], C["BB"][2:]]))
    assert max(errs.values()) < BAR, errs
