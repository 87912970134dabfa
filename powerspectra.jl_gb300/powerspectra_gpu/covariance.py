"""Analytic covariance blocks through the GPU library, mirroring src/covariance.jl.

`coupledcov(ch1, ch2, workspace, spectra, noiseratios)` keeps the reference's
dispatch (src/covariance.jl:34-61), the spectra / noise-ratio / window
gathering of each coupledcov*! wrapper (:64-418) and the symmetric
SpectralArray result; the loop_cov*! bodies (:92-446) run on the GPU.

The reference's CovarianceWorkspace computes its window spectra W with
spherical-harmonic transforms of mask products (src/workspace.jl:141-213).
Here the workspace is any object with `field_names` (i, j, p, q), `lmax` and
`window_function_W(X, Y, i, j, alpha, p, q, beta)` returning a 0-indexed
spectrum of lmax+1 entries -- e.g. WindowWorkspace below, fed with spectra
computed elsewhere.
"""
import numpy as np

from . import _lib
from .spectralarray import spectralones, spectralzeros

NN = "∅∅"  # the reference's :∅∅ (unweighted mask product)


class ConstantDict(dict):
    """Returns the same value for every key (src/util.jl:51-54)."""

    def __init__(self, value):
        super().__init__()
        self.value = value

    def __getitem__(self, key):
        return self.value

    def __len__(self):
        return 1


class WindowWorkspace:
    """Minimal stand-in for CovarianceWorkspace: field names, lmax and a
    window-spectrum provider keyed like window_function_W! (src/workspace.jl:174)."""

    def __init__(self, field_names, lmax, windows):
        self.field_names = tuple(field_names)
        self.lmax = int(lmax)
        self._windows = windows

    def window_function_W(self, X, Y, i, j, alpha, p, q, beta):
        key = (X, Y, i, j, alpha, p, q, beta)
        W = self._windows(*key) if callable(self._windows) else self._windows[key]
        W = np.asarray(getattr(W, "parent", W), dtype=np.float64)
        if len(W) < self.lmax + 1:
            raise _lib.PowerSpectraArgumentError(_lib.PS_ERR_ARG, "window %r has fewer than lmax+1 entries" % (key,))
        return W[:self.lmax + 1]


def _vec(x):
    return np.asarray(getattr(x, "parent", x), dtype=np.float64)


def _run(kind, C, S, R, Ws, mode, ctx):
    if C.axes[0] != C.axes[1]:
        raise _lib.PowerSpectraArgumentError(_lib.PS_ERR_ARG, "covariance matrix must be square in l")
    lmin, lmax = C.axes[0].start, C.axes[0].stop - 1
    c = ctx if ctx is not None else _lib.default_context()
    c.coupledcov(kind, [_vec(s) for s in S], [_vec(r) for r in R], [_vec(w) for w in Ws], lmin, lmax, mode=mode,
                 out=C.parent)
    return C


# ---- loop_cov*! drop-ins: same argument order as the reference ----
def loop_covTTTT(C, TTip, TTjq, TTiq, TTjp, r_ip, r_jq, r_iq, r_jp, W1, W2, W3, W4, W5, W6, W7, W8, mode="plain",
                 ctx=None):
    return _run("TTTT", C, [TTip, TTjq, TTiq, TTjp], [r_ip, r_jq, r_iq, r_jp], [W1, W2, W3, W4, W5, W6, W7, W8],
                mode, ctx)


def loop_covEEEE(C, EEip, EEjq, EEiq, EEjp, r_ip, r_jq, r_iq, r_jp, W1, W2, W3, W4, W5, W6, W7, W8, mode="plain",
                 ctx=None):
    return _run("EEEE", C, [EEip, EEjq, EEiq, EEjp], [r_ip, r_jq, r_iq, r_jp], [W1, W2, W3, W4, W5, W6, W7, W8],
                mode, ctx)


def loop_covTTTE(C, TTip, TTjp, TEiq, TEjq, r_ip, r_jp, W1, W2, W3, W4, mode="plain", ctx=None):
    return _run("TTTE", C, [TTip, TTjp, TEiq, TEjq], [r_ip, r_jp], [W1, W2, W3, W4], mode, ctx)


def loop_covTETE(C, TTip, EEjq, TEiq, TEjp, r_TT_ip, r_PP_jq, W1, W2, W3, W4, W5, mode="plain", ctx=None):
    return _run("TETE", C, [TTip, EEjq, TEiq, TEjp], [r_TT_ip, r_PP_jq], [W1, W2, W3, W4, W5], mode, ctx)


def loop_covTEEE(C, EEjq, EEjp, TEip, TEiq, r_EE_jq, r_EE_jp, W1, W2, W3, W4, mode="plain", ctx=None):
    return _run("TEEE", C, [EEjq, EEjp, TEip, TEiq], [r_EE_jq, r_EE_jp], [W1, W2, W3, W4], mode, ctx)


def loop_covTEEE_planck(C, EEjq, EEjp, TEip, TEiq, r_EE_jq, r_EE_jp, W1, W2, W3, W4, mode="plain", ctx=None):
    return _run("TEEE_PLANCK", C, [EEjq, EEjp, TEip, TEiq], [r_EE_jq, r_EE_jp], [W1, W2, W3, W4], mode, ctx)


def loop_covTTEE(C, TEip, TEiq, TEjq, TEjp, W1, W2, mode="plain", ctx=None):
    return _run("TTEE", C, [TEip, TEiq, TEjq, TEjp], [], [W1, W2], mode, ctx)


# ---- coupledcov*! wrappers (src/covariance.jl:64-418) ----
def gather(ch1, ch2, ws, spectra, nr, planck=True):
    """(kind, spectra, noise ratios, windows) of the block (ch1, ch2), in the
    order the reference's coupledcov*! wrapper passes them to its loop_cov*!."""
    i, j, p, q = ws.field_names
    W = ws.window_function_W
    if (ch1, ch2) == ("TT", "TT"):  # src/covariance.jl:64-88
        return ("TTTT", [spectra["TT", i, p], spectra["TT", j, q], spectra["TT", i, q], spectra["TT", j, p]],
                [nr["TT", i, p], nr["TT", j, q], nr["TT", i, q], nr["TT", j, p]],
                [W(NN, NN, i, p, "TT", j, q, "TT"), W(NN, NN, i, q, "TT", j, p, "TT"),
                 W(NN, "TT", i, p, "TT", j, q, "TT"), W(NN, "TT", j, q, "TT", i, p, "TT"),
                 W(NN, "TT", i, q, "TT", j, p, "TT"), W(NN, "TT", j, p, "TT", i, q, "TT"),
                 W("TT", "TT", i, p, "TT", j, q, "TT"), W("TT", "TT", i, q, "TT", j, p, "TT")])
    if (ch1, ch2) == ("EE", "EE"):  # src/covariance.jl:125-149
        return ("EEEE", [spectra["EE", i, p], spectra["EE", j, q], spectra["EE", i, q], spectra["EE", j, p]],
                [nr["EE", i, p], nr["EE", j, q], nr["EE", i, q], nr["EE", j, p]],
                [W(NN, NN, i, p, "PP", j, q, "PP"), W(NN, NN, i, q, "PP", j, p, "PP"),
                 W(NN, "PP", i, p, "PP", j, q, "PP"), W(NN, "PP", j, q, "PP", i, p, "PP"),
                 W(NN, "PP", i, q, "PP", j, p, "PP"), W(NN, "PP", j, p, "PP", i, q, "PP"),
                 W("PP", "PP", i, p, "PP", j, q, "PP"), W("PP", "PP", i, q, "PP", j, p, "PP")])
    if (ch1, ch2) == ("TT", "TE"):  # src/covariance.jl:186-204
        return ("TTTE", [spectra["TT", i, p], spectra["TT", j, p], spectra["TE", i, q], spectra["TE", j, q]],
                [nr["TT", i, p], nr["TT", j, p]],
                [W(NN, NN, i, p, "TT", j, q, "TP"), W(NN, NN, i, q, "TP", j, p, "TT"),
                 W(NN, "TT", j, q, "TP", i, p, "TT"), W(NN, "TT", i, q, "TP", j, p, "TT")])
    if (ch1, ch2) == ("TE", "TE"):  # src/covariance.jl:238-257
        return ("TETE", [spectra["TT", i, p], spectra["EE", j, q], spectra["TE", i, q], spectra["TE", j, p]],
                [nr["TT", i, p], nr["EE", j, q]],
                [W(NN, NN, i, p, "TT", j, q, "PP"), W(NN, NN, i, q, "TP", j, p, "PT"),
                 W(NN, "PP", i, p, "TT", j, q, "PP"), W(NN, "TT", j, q, "PP", i, p, "TT"),
                 W("TT", "PP", i, p, "TT", j, q, "PP")])
    if (ch1, ch2) == ("TE", "EE"):  # src/covariance.jl:305-333
        return ("TEEE_PLANCK" if planck else "TEEE",
                [spectra["EE", j, q], spectra["EE", j, p], spectra["TE", i, p], spectra["TE", i, q]],
                [nr["EE", j, q], nr["EE", j, p]],
                [W(NN, NN, i, p, "TP", j, q, "PP"), W(NN, NN, i, q, "TP", j, p, "PP"),
                 W(NN, "PP", i, p, "TP", j, q, "PP"), W(NN, "PP", i, q, "TP", j, p, "PP")])
    if (ch1, ch2) == ("TT", "EE"):  # src/covariance.jl:405-418
        return ("TTEE", [spectra["TE", i, p], spectra["TE", i, q], spectra["TE", j, q], spectra["TE", j, p]], [],
                [W(NN, NN, i, p, "TP", j, q, "TP"), W(NN, NN, i, q, "TP", j, p, "TP")])
    return None


def coupledcovTTTT(C, ws, spectra, nr, mode="plain", ctx=None):
    return _run(*_kind_args(gather("TT", "TT", ws, spectra, nr), C), mode, ctx)


def coupledcovEEEE(C, ws, spectra, nr, mode="plain", ctx=None):
    return _run(*_kind_args(gather("EE", "EE", ws, spectra, nr), C), mode, ctx)


def coupledcovTTTE(C, ws, spectra, nr, mode="plain", ctx=None):
    return _run(*_kind_args(gather("TT", "TE", ws, spectra, nr), C), mode, ctx)


def coupledcovTETE(C, ws, spectra, nr, mode="plain", ctx=None):
    return _run(*_kind_args(gather("TE", "TE", ws, spectra, nr), C), mode, ctx)


def coupledcovTEEE(C, ws, spectra, nr, planck=True, mode="plain", ctx=None):
    return _run(*_kind_args(gather("TE", "EE", ws, spectra, nr, planck=planck), C), mode, ctx)


def coupledcovTTEE(C, ws, spectra, nr, mode="plain", ctx=None):
    return _run(*_kind_args(gather("TT", "EE", ws, spectra, nr), C), mode, ctx)


def _kind_args(g, C):
    kind, S, R, Ws = g
    return kind, C, S, R, Ws


def coupledcov(ch1, ch2, workspace, spectra, noiseratios=None, lmin=0, lmax=None, mode="plain", ctx=None):
    """Coupled covariance block between spectra ch1 and ch2 (src/covariance.jl:34-61)."""
    lmax = workspace.lmax if lmax is None else lmax
    C = spectralzeros(range(lmin, lmax + 1), range(lmin, lmax + 1))
    if not noiseratios:  # default: do not rescale for noise
        noiseratios = ConstantDict(spectralones(range(0, lmax + 1)))
    table = {("TT", "TT"): coupledcovTTTT, ("EE", "EE"): coupledcovEEEE, ("TE", "TE"): coupledcovTETE,
             ("TT", "TE"): coupledcovTTTE, ("TT", "EE"): coupledcovTTEE, ("TE", "EE"): coupledcovTEEE}
    f = table.get((ch1, ch2))
    if f is None:
        print("%s,%s not implemented" % (ch1, ch2))  # the reference prints and returns nothing
        return None
    return f(C, workspace, spectra, noiseratios, mode=mode, ctx=ctx)
