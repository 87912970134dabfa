"""ctypes binding of the C oracle (oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle restates, in plain FP64 C with OpenMP,
the reference algorithm of PowerSpectra.jl for the mode-coupling hot path:
  src/modecoupling.jl:3-159   Xi projectors, fill_3j!, inner_mcm00!/02!/++!/--!
  src/covariance.jl:92-446    loop_cov{TTTT,EEEE,TTTE,TETE,TEEE,TEEE_planck,TTEE}!
  src/beam.jl:17-109          Xisum / quickpolXi!
  src/workspace.jl:174-213    window_function_W! (alm2cl of coefficient sets; plain numpy below)
Matrices are column-major (Julia layout): element (l1, l2) of an (n x n)
result with lmin offset lives at [l1 - lmin, l2 - lmin] of a Fortran-ordered
numpy array.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

SPIN_00, SPIN_02, SPIN_PP, SPIN_MM = 0, 1, 2, 3
PROD_00_00, PROD_22_22, PROD_00_22 = 0, 1, 2
PARITY_ALL, PARITY_EVEN, PARITY_ODD = 0, 1, 2
COV_KINDS = {"TTTT": 0, "EEEE": 1, "TTTE": 2, "TETE": 3, "TEEE": 4, "TEEE_PLANCK": 5, "TTEE": 6}
COV_NWINDOWS = {"TTTT": 8, "EEEE": 8, "TTTE": 4, "TETE": 5, "TEEE": 4, "TEEE_PLANCK": 4, "TTEE": 2}
COV_NRATIOS = {"TTTT": 4, "EEEE": 4, "TTTE": 2, "TETE": 2, "TEEE": 2, "TEEE_PLANCK": 2, "TTEE": 0}


def build():
    """Compile oracle.c with the committed Makefile (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        src = os.path.join(_HERE, "oracle.c")
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        cl, ci = ctypes.c_long, ctypes.c_int
        lib.or_w3j_family.argtypes = [ci, ci, ci, ci, dp, ip]
        lib.or_w3j_family.restype = ci
        lib.or_inner_mcm.argtypes = [ci, dp, cl, ci, ci, dp, cl, ip, ci, ci]
        lib.or_inner_mcm.restype = ci
        lib.or_inner_mcm_abs.argtypes = [ci, dp, cl, ci, ci, dp, cl, ip, ci, ci]
        lib.or_inner_mcm_abs.restype = ci
        lib.or_loop_cov_abs.argtypes = [ci, ctypes.POINTER(dp), ctypes.POINTER(dp), ctypes.POINTER(dp), cl, ci, ci, dp,
                                        cl, ip, ci, ci]
        lib.or_loop_cov_abs.restype = ci
        lib.or_quickpol_xi.argtypes = [ci, ci, ci, ci, dp, cl, ci, ci, ci, dp, cl, ci]
        lib.or_quickpol_xi.restype = ci
        lib.or_quickpol_xi_abs.argtypes = [ci, ci, ci, ci, dp, cl, ci, ci, ci, dp, cl, ci]
        lib.or_quickpol_xi_abs.restype = ci
        lib.or_quickpol_xi_common.argtypes = [ci, ci, ci, ci, dp, cl, ci, ci, ci, dp, cl, ci]
        lib.or_quickpol_xi_common.restype = ci
        lib.or_xi.argtypes = [ci, ci, dp, cl, ci, ci, dp, cl, ci]
        lib.or_xi.restype = ci
        lib.or_loop_cov.argtypes = [ci, ctypes.POINTER(dp), ctypes.POINTER(dp), ctypes.POINTER(dp), cl, ci, ci, dp, cl,
                                    ip, ci, ci]
        lib.or_loop_cov.restype = ci
        lib.or_cov_nwindows.argtypes = [ci]
        lib.or_cov_nwindows.restype = ci
        lib.or_max_threads.argtypes = []
        lib.or_max_threads.restype = ci
        lib.or_l3_terms.argtypes = [ci, ci, cl, ip, ci]
        lib.or_l3_terms.restype = ctypes.c_double
        _lib = lib
        return lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _rows(rows):
    if rows is None:
        return None, None, 0
    r = np.ascontiguousarray(rows, dtype=np.int32)
    return r, r.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(r)


def max_threads():
    return _load().or_max_threads()


def w3j_family(l1, l2, m1, m2):
    """(jmin, values) of the family (l1 l2 l3; m1 m2 -m1-m2) over l3 = jmin..l1+l2."""
    lib = _load()
    out = np.zeros(2 * min(l1, l2) + 2, dtype=np.float64)
    jmin = ctypes.c_int(0)
    n = lib.or_w3j_family(l1, l2, m1, m2, _dptr(out), ctypes.byref(jmin))
    return jmin.value, out[:n].copy()


def inner_mcm(spin, W, lmin, lmax, rows=None, nthreads=0, out=None, absolute=False):
    """One spin-case mode-coupling matrix (inner_mcm00!/02!/++!/--!).  With
    absolute=True: the same sums over |3j product| * |W| (sum of |terms|)."""
    lib = _load()
    W = np.ascontiguousarray(W, dtype=np.float64)
    n = lmax - lmin + 1
    M = np.zeros((n, n), dtype=np.float64, order="F") if out is None else out
    r, rp, nr = _rows(rows)
    fn = lib.or_inner_mcm_abs if absolute else lib.or_inner_mcm
    st = fn(int(spin), _dptr(W), len(W), lmin, lmax, _dptr(M), n, rp, nr, nthreads)
    if st:
        raise RuntimeError("oracle inner_mcm failed (%d)" % st)
    return M


def xi(product, parity, W, lmin, lmax, nthreads=0):
    lib = _load()
    W = np.ascontiguousarray(W, dtype=np.float64)
    n = lmax - lmin + 1
    X = np.zeros((n, n), dtype=np.float64, order="F")
    st = lib.or_xi(int(product), int(parity), _dptr(W), len(W), lmin, lmax, _dptr(X), n, nthreads)
    if st:
        raise RuntimeError("oracle xi failed (%d)" % st)
    return X


def loop_cov(kind, spectra, ratios, windows, lmin, lmax, rows=None, nthreads=0, absolute=False):
    """Covariance block by the reference loop_cov*! formula for `kind`.  With
    absolute=True: the formula on absolute values (sum of |terms| per element)."""
    lib = _load()
    k = COV_KINDS[kind] if isinstance(kind, str) else int(kind)
    name = [n for n, v in COV_KINDS.items() if v == k][0]
    if len(windows) != COV_NWINDOWS[name] or len(spectra) != 4 or len(ratios) != COV_NRATIOS[name]:
        raise ValueError("wrong number of spectra/ratios/windows for %s" % name)
    S = [np.ascontiguousarray(s, dtype=np.float64) for s in spectra]
    R = [np.ascontiguousarray(s, dtype=np.float64) for s in ratios]
    Wl = [np.ascontiguousarray(s, dtype=np.float64) for s in windows]
    for a in S + R:
        if len(a) < lmax + 1:
            raise ValueError("spectra and noise ratios need lmax+1 entries")
    nW = min(len(w) for w in Wl)
    DP = ctypes.POINTER(ctypes.c_double)
    Sa = (DP * 4)(*[_dptr(a) for a in S])
    Ra = (DP * max(len(R), 1))(*([_dptr(a) for a in R] or [None]))
    Wa = (DP * len(Wl))(*[_dptr(a) for a in Wl])
    n = lmax - lmin + 1
    C = np.zeros((n, n), dtype=np.float64, order="F")
    r, rp, nr = _rows(rows)
    fn = lib.or_loop_cov_abs if absolute else lib.or_loop_cov
    st = fn(k, Sa, Ra, Wa, nW, lmin, lmax, _dptr(C), n, rp, nr, nthreads)
    if st:
        raise RuntimeError("oracle loop_cov failed (%d)" % st)
    return C


def l3_terms(lmin, lmax, nW, rows=None):
    """l3-terms of one family summed over the (l1 <= l2) pairs of the rows, l3 <= nW-1."""
    r, rp, nr = _rows(rows)
    return _load().or_l3_terms(lmin, lmax, nW, rp, nr)


def quickpol_xi(nu1, nu2, s1, s2, W, lmax, bl, bu, nthreads=0, absolute=False, common_match=False):
    """quickpolXi! (src/beam.jl:72-109) as a dense (lmax+1)^2 matrix, zeros outside the band.
    absolute=True: the sums over |W f1 f2| (sum of |terms|, no sign).  common_match=True: both
    families of an element matched at the larger of their midpoints, as the GPU kernel does (the
    default matches each family at its own midpoint)."""
    lib = _load()
    W = np.ascontiguousarray(W, dtype=np.float64)
    n = lmax + 1
    X = np.zeros((n, n), dtype=np.float64, order="F")
    if absolute and common_match:
        raise ValueError("absolute sums do not depend on the match point")
    fn = lib.or_quickpol_xi_abs if absolute else (lib.or_quickpol_xi_common if common_match else lib.or_quickpol_xi)
    st = fn(int(nu1), int(nu2), int(s1), int(s2), _dptr(W), len(W), lmax, bl, bu, _dptr(X), n,
                            nthreads)
    if st:
        raise RuntimeError("oracle quickpol_xi failed (%d)" % st)
    return X


def alm_index(l, m, lmax):
    """Position of a_lm in the HEALPix m-major coefficient order (Healpix.jl almIndex, 0-based)."""
    return m * (2 * lmax + 1 - m) // 2 + l


def n_alms(lmax, mmax):
    return (mmax + 1) * (mmax + 2) // 2 + (mmax + 1) * (lmax - mmax)


def alm2cl(a, b, lmax, mmax=None):
    """Cross-spectrum of two coefficient sets of real fields (the HEALPix alm2cl definition that
    src/modecoupling.jl:197 and src/workspace.jl:202 call, from the third-party Healpix.jl):
    cl[l] = (Re a_l0 b*_l0 + 2 sum_{m=1}^{min(l,mmax)} Re a_lm b*_lm) / (2l+1).  Plain loops over m
    in FP64, one l-vector per m."""
    mmax = lmax if mmax is None else mmax
    cl = np.zeros(lmax + 1)
    for m in range(mmax + 1):
        i0 = alm_index(m, m, lmax)
        x = a[i0:i0 + lmax + 1 - m]
        y = b[i0:i0 + lmax + 1 - m]
        term = x.real * y.real + x.imag * y.imag
        cl[m:] += term if m == 0 else 2.0 * term
    return cl / (2.0 * np.arange(lmax + 1) + 1.0)


def window_function_W(A, B, lmax, mmax=None, lout=None):
    """window_function_W! (src/workspace.jl:174-213): the mean over the (wX, wY) terms of
    alm2cl(A[t], B[t])[0:lout]; None is an all-zero set (effective_weight_alm!'s zero Alm,
    src/workspace.jl:167-170), which still counts in the mean."""
    lout = lmax if lout is None else lout
    res = np.zeros(lout + 1)
    for a, b in zip(A, B):
        if a is not None and b is not None:
            res += alm2cl(a, b, lmax, mmax)[:lout + 1]
    return res * (1.0 / len(A))


def quickpolW(a, b, lmax, mmax=None):
    """quickpolW (src/beam.jl:40-53): sum over m = -l..l of a_lm conj(b_lm), i.e. alm2cl without
    the 1/(2l+1)."""
    return alm2cl(a, b, lmax, mmax) * (2.0 * np.arange(lmax + 1) + 1.0)
