"""Mask power spectra for the covariance workspace, mirroring src/workspace.jl.

The reference's `window_function_W!` (src/workspace.jl:174-213) averages
alm2cl over the weight terms of two (field, spectrum) keys: TT stands for the
single II term, PP for the QQ and UU terms (Planck 2015 eq. C.11-C.16).  Each
term's coefficients come from `effective_weight_alm!` (src/workspace.jl:141-171),
a spherical-harmonic transform of a mask product; that transform is not part of
this library, so the caller supplies those coefficient sets (or None where the
reference returns its all-zero Alm).  The alm2cl sums run on the GPU
(`ps_window_W`).

Coefficient sets are complex128 vectors in the HEALPix m-major order, (l, m) at
m (2 lmax + 1 - m) / 2 + l, as Healpix.jl's `Alm` stores them.
"""
import numpy as np

from . import _lib
from .spectralarray import SpectralVector

_WTERMS = {"TT": ("II",), "PP": ("QQ", "UU")}


def _ctx(ctx):
    return ctx if ctx is not None else _lib.default_context()


def n_alms(lmax, mmax=None):
    """numberOfAlms(lmax, mmax)."""
    mmax = lmax if mmax is None else mmax
    return (mmax + 1) * (mmax + 2) // 2 + (mmax + 1) * (lmax - mmax)


def alm2cl(alm1, alm2, lmax, mmax=None, ctx=None):
    """Cross power spectrum of two coefficient sets, l = 0..lmax (the alm2cl of
    src/modecoupling.jl:197 and :357-373), computed on the GPU."""
    return _ctx(ctx).window_W([alm1], [alm2], lmax, lmax if mmax is None else mmax)


def wterms(X):
    """Weight terms of a spectrum key (src/workspace.jl:180-194)."""
    return _WTERMS.get(X, (X,))


class AlmWindowWorkspace:
    """Covariance workspace whose window spectra come from effective-weight
    coefficient sets.  `effective_weights` maps (A, i, j, alpha) -> coefficients
    (or None for the reference's zero Alm), like CovarianceWorkspace's
    effective_weights cache (src/workspace.jl:82); a callable is called with
    the same key.  `window_function_W` caches its results by the reference's
    8-tuple key (W_spectra, src/workspace.jl:176-178)."""

    def __init__(self, field_names, lmax, effective_weights, mmax=None, ctx=None):
        self.field_names = tuple(field_names)
        self.lmax = int(lmax)
        self.mmax = self.lmax if mmax is None else int(mmax)
        self._ew = effective_weights
        self._ctx = ctx
        self.W_spectra = {}

    def effective_weight_alm(self, A, i, j, alpha):
        key = (A, i, j, alpha)
        if callable(self._ew):
            return self._ew(*key)
        return self._ew.get(key)

    def window_function_W(self, X, Y, i, j, alpha, p, q, beta):
        key = (X, Y, i, j, alpha, p, q, beta)
        if key in self.W_spectra:
            return self.W_spectra[key]
        A, B = [], []
        for wX in wterms(X):
            for wY in wterms(Y):
                A.append(self.effective_weight_alm(wX, i, j, alpha))
                B.append(self.effective_weight_alm(wY, p, q, beta))
        W = _ctx(self._ctx).window_W(A, B, self.lmax, self.mmax, self.lmax)
        self.W_spectra[key] = np.asarray(W)
        return self.W_spectra[key]

    def spectral(self, *key):
        """The window as a 0-indexed SpectralVector, as the reference returns it."""
        return SpectralVector(self.window_function_W(*key))
