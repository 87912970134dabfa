"""Mode-coupling matrices through the GPU library, mirroring src/modecoupling.jl.

`mcm(spec, W; lmin, lmax)` keeps the reference's spec symbols, dispatch,
return types and errors (src/modecoupling.jl:192-246).  The reference's `mcm`
takes the two masks' alms and computes W = alm2cl(alm1, alm2)[1:lmax+1]
(src/modecoupling.jl:197) with Healpix; here the caller passes that mask
cross-spectrum W directly (0-indexed by l).  The inner_mcm* functions are the
drop-in replacements of the reference's loop bodies (src/modecoupling.jl:78-159):
they fill a SpectralArray in place through the C ABI.
"""
import numpy as np

from . import _lib
from ._lib import PS_SPIN_00, PS_SPIN_02, PS_SPIN_MM, PS_SPIN_PP, PowerSpectraArgumentError
from .spectralarray import BlockSpectralMatrix, SpectralArray, spectralzeros

SPEC_00 = ("TT", "M00", "M⁰⁰")
SPEC_02 = ("TE", "ET", "TB", "BT", "M02", "M20", "M⁰²", "M²⁰")
SPEC_PP = ("M++", "M⁺⁺")
SPEC_MM = ("M--", "M⁻⁻")


def _ctx(ctx):
    return ctx if ctx is not None else _lib.default_context()


def _check_square(M):
    if M.axes[0] != M.axes[1]:  # @assert axes(M, 1) == axes(M, 2), src/modecoupling.jl:80
        raise PowerSpectraArgumentError(_lib.PS_ERR_ARG, "mode-coupling matrix must be square in l")
    if not (M.parent.flags.f_contiguous and M.parent.dtype == np.float64):
        raise PowerSpectraArgumentError(_lib.PS_ERR_ARG, "parent must be a column-major float64 array")
    return M.axes[0].start, M.axes[0].stop - 1


def _inner(spin, M, V, mode, ctx):
    lmin, lmax = _check_square(M)
    V = np.ascontiguousarray(np.asarray(getattr(V, "parent", V), dtype=np.float64))
    _ctx(ctx).mcm(spin, V, lmin, lmax, mode=mode, out=M.parent)
    return M


def inner_mcm00(M, V, mode="plain", ctx=None):
    """inner_mcm00! (src/modecoupling.jl:78-95): TT coupling into M in place."""
    return _inner(PS_SPIN_00, M, V, mode, ctx)


def inner_mcm02(M, V, mode="plain", ctx=None):
    """inner_mcm02! (src/modecoupling.jl:99-119): TE/ET/TB/BT coupling."""
    return _inner(PS_SPIN_02, M, V, mode, ctx)


def inner_mcmPP(M, V, mode="plain", ctx=None):
    """inner_mcm++! (src/modecoupling.jl:123-139): spin-2 even-parity block."""
    return _inner(PS_SPIN_PP, M, V, mode, ctx)


def inner_mcmMM(M, V, mode="plain", ctx=None):
    """inner_mcm--! (src/modecoupling.jl:143-159): spin-2 odd-parity block."""
    return _inner(PS_SPIN_MM, M, V, mode, ctx)


def inner_mcmPPMM(Mpp, Mmm, V, mode="plain", ctx=None):
    """++ and -- from one shared 22 family per pair (one GPU pass)."""
    lmin, lmax = _check_square(Mpp)
    if _check_square(Mmm) != (lmin, lmax):
        raise PowerSpectraArgumentError(_lib.PS_ERR_ARG, "++ and -- blocks must share their l axes")
    V = np.ascontiguousarray(np.asarray(getattr(V, "parent", V), dtype=np.float64))
    _ctx(ctx).mcm_multi({PS_SPIN_PP: V, PS_SPIN_MM: V}, lmin, lmax, mode=mode,
                        outs={PS_SPIN_PP: Mpp.parent, PS_SPIN_MM: Mmm.parent})
    return Mpp, Mmm


def _spectrum(W, lmax):
    W = np.asarray(getattr(W, "parent", W), dtype=np.float64)
    if lmax is None:
        lmax = len(W) - 1
    if len(W) < lmax + 1:
        raise PowerSpectraArgumentError(_lib.PS_ERR_ARG, "mask spectrum has %d entries, need lmax+1 = %d"
                                        % (len(W), lmax + 1))
    return np.ascontiguousarray(W[:lmax + 1]), lmax  # Vij = alm2cl(...)[1:(lmax+1)], src/modecoupling.jl:197


def mcm(spec, W, lmin=0, lmax=None, mode="plain", ctx=None):
    """Mode-coupling matrix for `spec` from the mask cross-spectrum W.

    spec: "TT"/"M00"; "TE","ET","TB","BT","M02","M20"; "M++"; "M--";
    "EE_BB"; "EB_BE"; or the tuple ("EE_BB", "EB_BE").  Returns a
    SpectralArray with axes lmin:lmax, a 2x2 BlockSpectralMatrix for EE_BB /
    EB_BE, or a pair of them for the tuple form.
    """
    if isinstance(spec, tuple):
        if tuple(spec) != ("EE_BB", "EB_BE"):
            return None  # the reference's tuple method returns nothing for other tuples
        V, lmax = _spectrum(W, lmax)
        Mpp, Mmm = spectralzeros(range(lmin, lmax + 1), range(lmin, lmax + 1)), \
            spectralzeros(range(lmin, lmax + 1), range(lmin, lmax + 1))
        inner_mcmPPMM(Mpp, Mmm, V, mode, ctx)
        return (BlockSpectralMatrix.hvcat([[Mpp, Mmm], [Mmm, Mpp]]),
                BlockSpectralMatrix.hvcat([[Mpp, -Mmm], [-Mmm, Mpp]]))
    V, lmax = _spectrum(W, lmax)
    ax = range(lmin, lmax + 1)
    if spec in SPEC_00:
        return inner_mcm00(spectralzeros(ax, ax), V, mode, ctx)
    if spec in SPEC_02:
        return inner_mcm02(spectralzeros(ax, ax), V, mode, ctx)
    if spec in SPEC_PP:
        return inner_mcmPP(spectralzeros(ax, ax), V, mode, ctx)
    if spec in SPEC_MM:
        return inner_mcmMM(spectralzeros(ax, ax), V, mode, ctx)
    if spec in ("EE_BB", "EB_BE"):
        Mpp, Mmm = spectralzeros(ax, ax), spectralzeros(ax, ax)
        inner_mcmPPMM(Mpp, Mmm, V, mode, ctx)
        if spec == "EE_BB":
            return BlockSpectralMatrix.hvcat([[Mpp, Mmm], [Mmm, Mpp]])
        return BlockSpectralMatrix.hvcat([[Mpp, -Mmm], [-Mmm, Mpp]])
    raise PowerSpectraArgumentError(_lib.PS_ERR_ARG, "%s not a valid spectrum." % (spec,))  # :225
