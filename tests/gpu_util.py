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
