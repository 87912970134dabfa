"""Host logic of the window-spectrum workspace mirror (src/workspace.jl:141-213) on the CPU.

A stand-in context computes ps_window_W with the oracle, so the weight-term mapping (TT -> II,
PP -> QQ/UU), the zero-set handling, the mean over terms and the W_spectra cache are checked
without a GPU."""
import numpy as np

import powerspectra_gpu as pg
from oracle import oracle as o


class OracleWindowContext:
    """Answers window_W like the library, with the oracle; records each call."""

    def __init__(self):
        self.calls = []

    def window_W(self, A, B, lmax, mmax=None, lout=None):
        self.calls.append((len(A), sum(a is None for a in A) + sum(b is None for b in B)))
        return o.window_function_W(A, B, lmax, mmax, lout)


def _set(lmax, seed):
    rng = np.random.default_rng(seed)
    n = o.n_alms(lmax, lmax)
    return rng.normal(size=n) + 1j * rng.normal(size=n)


def test_wterms_mapping():
    assert pg.wterms("TT") == ("II",)
    assert pg.wterms("PP") == ("QQ", "UU")
    assert pg.wterms("∅∅") == ("∅∅",)


def test_window_function_W_terms_and_cache():
    L = 24
    sets = {}

    def ew(A, i, j, alpha):
        if A != "∅∅" and i != j:
            return None
        return sets.setdefault((A, i, j, alpha), _set(L, len(sets) + 1))

    ctx = OracleWindowContext()
    ws = pg.AlmWindowWorkspace(("a", "b", "a", "b"), L, ew, ctx=ctx)
    # PP x TT: (QQ, UU) x (II): two terms, both with i == j so no zero sets
    W = ws.window_function_W("PP", "TT", "a", "a", "PP", "b", "b", "TT")
    A = [sets["QQ", "a", "a", "PP"], sets["UU", "a", "a", "PP"]]
    B = [sets["II", "b", "b", "TT"], sets["II", "b", "b", "TT"]]
    np.testing.assert_allclose(W, 0.5 * (o.alm2cl(A[0], B[0], L) + o.alm2cl(A[1], B[1], L)), rtol=1e-14)
    assert ctx.calls == [(2, 0)]
    # the cache answers a repeat without a call
    assert ws.window_function_W("PP", "TT", "a", "a", "PP", "b", "b", "TT") is W
    assert len(ctx.calls) == 1
    # cross-field weights are the reference's zero Alm: they count in the mean but add nothing
    Wx = ws.window_function_W("TT", "TT", "a", "b", "TT", "a", "b", "TT")
    assert ctx.calls[-1] == (1, 2) and not np.any(Wx)
    # the unweighted mask product (∅∅) has one term and exists for i != j
    W0 = ws.window_function_W("∅∅", "∅∅", "a", "b", "TT", "a", "b", "TT")
    s0 = sets["∅∅", "a", "b", "TT"]
    np.testing.assert_allclose(W0, o.alm2cl(s0, s0, L), rtol=1e-14)


def test_spectral_vector_view():
    L = 8
    ctx = OracleWindowContext()
    ws = pg.AlmWindowWorkspace(("a",) * 4, L, lambda *k: _set(L, 3), ctx=ctx)
    V = ws.spectral("∅∅", "∅∅", "a", "a", "TT", "a", "a", "TT")
    assert V.axes[0] == range(0, L + 1)
