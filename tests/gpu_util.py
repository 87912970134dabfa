"""Shared helpers of the GPU parity tests."""
import numpy as np


def max_rel(got, ref, floor_frac=0.0):
    """Largest elementwise |got - ref| / max(|ref|, floor_frac * max|ref|)."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    den = np.maximum(np.abs(ref), floor_frac * np.max(np.abs(ref)))
    den = np.where(den == 0, 1.0, den)
    bad = (den == 1.0) & (ref == 0)
    err = np.abs(got - ref) / den
    err[bad] = np.abs(got[bad] - ref[bad])
    return float(np.max(err)) if err.size else 0.0


def cond_scale(spin, W, lmin, lmax, rows=None):
    """Sum of |terms| behind each mode-coupling element (the oracle's loops on
    |3j product| |W|).  It equals |M| when nothing cancels (W >= 0 and a squared
    family); an FP64 sum cannot resolve an element below eps times it."""
    from oracle import oracle as o
    return o.inner_mcm(spin, W, lmin, lmax, rows=rows, absolute=True)


def cov_scale(kind, S, R, Ws, lmin, lmax):
    """Sum of |terms| behind each covariance element (oracle formula on absolute values)."""
    from oracle import oracle as o
    return o.loop_cov(kind, S, R, Ws, lmin, lmax, absolute=True)


def max_err_scaled(got, ref, scale):
    """Largest |got - ref| / max(|ref|, scale) (elements with zero scale compare absolutely)."""
    den = np.maximum(np.abs(ref), scale)
    den = np.where(den == 0, 1.0, den)
    return float(np.max(np.abs(np.asarray(got) - ref) / den)) if np.size(ref) else 0.0


def gpu_cond_scale(ctx, spin, W, lmin, lmax):
    """cond_scale computed with the GPU's plain FP64 path (for sizes the oracle is too slow
    for): |M| of |W| for squared families; for 00x22 the Cauchy-Schwarz bound
    sqrt(M00(|W|) (M++(|W|) + M--(|W|)))."""
    A = np.abs(np.asarray(W, dtype=np.float64))
    if spin != 1:
        return np.abs(ctx.mcm(spin, A, lmin, lmax, mode="plain"))
    m = ctx.mcm_multi({0: A, 2: A, 3: A}, lmin, lmax, mode="plain")
    return np.sqrt(np.abs(m[0] * (m[2] + m[3])))
