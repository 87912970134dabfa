"""ctypes binding of libpowerspectra_gpu.so (the C ABI in include/powerspectra_gpu.h).

The library is built in-tree by powerspectra.jl_gb300/build.py.  There is no
CPU fallback: if the shared library is missing or no CUDA device is visible,
every call raises.
"""
import ctypes
import os
import threading

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "lib", "libpowerspectra_gpu.so")

PS_OK, PS_ERR_ARG, PS_ERR_CUDA, PS_ERR_OOM, PS_ERR_TIMEOUT, PS_ERR_UNSUPPORTED = 0, 1, 2, 3, 4, 5
PS_SPIN_00, PS_SPIN_02, PS_SPIN_PP, PS_SPIN_MM = 0, 1, 2, 3
PS_MODE_PLAIN_FP64, PS_MODE_CHOSEN = 0, 1
PS_PROD_00_00, PS_PROD_22_22, PS_PROD_00_22 = 0, 1, 2
PS_PARITY_ALL, PS_PARITY_EVEN, PS_PARITY_ODD = 0, 1, 2
COV_KINDS = {"TTTT": 0, "EEEE": 1, "TTTE": 2, "TETE": 3, "TEEE": 4, "TEEE_PLANCK": 5, "TTEE": 6}
COV_NWINDOWS = {0: 8, 1: 8, 2: 4, 3: 5, 4: 4, 5: 4, 6: 2}
COV_NRATIOS = {0: 4, 1: 4, 2: 2, 3: 2, 4: 2, 5: 2, 6: 0}
MODES = {"plain": PS_MODE_PLAIN_FP64, "fp64": PS_MODE_PLAIN_FP64, "chosen": PS_MODE_CHOSEN}

# every symbol declared in include/powerspectra_gpu.h
EXPORTS = ("ps_create", "ps_destroy", "ps_last_error", "ps_set_stream", "ps_synchronize", "ps_mcm", "ps_mcm_multi",
           "ps_mcm_multi_device", "ps_xi", "ps_coupledcov", "ps_coupledcov_device", "ps_coupledcov_set_device", "ps_mcm_set_device",
           "ps_batch_prepare", "ps_batch_run", "ps_batch_graph_launch", "ps_batch_autotune", "ps_last_kernel_ms",
           "ps_launch_count", "ps_probe_fma_peak", "ps_mcm_multi_device_noalloc", "ps_decouple_covmat", "ps_solve",
           "ps_quickpol_xi", "ps_decouple_covmat_device", "ps_window_W", "ps_window_W_device",
           "ps_quickpol_xi_alm", "ps_mcm_set", "ps_set_tensor_cores")


class PowerSpectraGPUError(RuntimeError):
    """A non-zero status from the C ABI; `.code` holds it."""

    def __init__(self, code, msg):
        super().__init__("powerspectra_gpu error %d: %s" % (code, msg))
        self.code = code


class PowerSpectraArgumentError(PowerSpectraGPUError, ValueError):
    """PS_ERR_ARG: the reference raises ArgumentError / fails an @assert here."""


_lib = None
_lock = threading.RLock()
_DP = ctypes.POINTER(ctypes.c_double)
_DPP = ctypes.POINTER(_DP)


class PSProblem(ctypes.Structure):
    """struct ps_problem of include/powerspectra_gpu.h"""
    _fields_ = [("lmin", ctypes.c_int), ("lmax", ctypes.c_int), ("cases", ctypes.c_uint), ("K", ctypes.c_int),
                ("nW", ctypes.c_int64), ("W", _DPP), ("M", _DPP), ("ldm", ctypes.c_int64)]


def _result_matrix(out, n):
    """An (n, n) F-ordered float64 result: `out` if given (checked), else a new array."""
    if out is None:
        return np.empty((n, n), dtype=np.float64, order="F")
    if out.shape != (n, n) or out.dtype != np.float64 or not out.flags.f_contiguous:
        raise PowerSpectraArgumentError(PS_ERR_ARG, "out must be an F-ordered float64 array of shape (%d, %d)" % (n, n))
    return out


def load(path=None):
    """Load the shared library (no build, no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError("libpowerspectra_gpu.so not found at %s: run powerspectra.jl_gb300/build.py "
                               "(there is no CPU fallback)" % p)
        lib = ctypes.CDLL(p)
        vp, ci, i64, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64
        lib.ps_create.argtypes = [ci, ctypes.POINTER(vp)]
        lib.ps_create.restype = ci
        lib.ps_destroy.argtypes = [vp]
        lib.ps_destroy.restype = None
        lib.ps_last_error.argtypes = [vp]
        lib.ps_last_error.restype = ctypes.c_char_p
        lib.ps_set_stream.argtypes = [vp, vp]
        lib.ps_set_stream.restype = ci
        lib.ps_synchronize.argtypes = [vp]
        lib.ps_synchronize.restype = ci
        lib.ps_set_tensor_cores.argtypes = [vp, ci]
        lib.ps_set_tensor_cores.restype = ci
        lib.ps_mcm.argtypes = [vp, ci, _DP, i64, ci, ci, ci, _DP, i64]
        lib.ps_mcm.restype = ci
        lib.ps_mcm_multi.argtypes = [vp, ctypes.c_uint, _DPP, i64, ci, ci, ci, _DPP, i64]
        lib.ps_mcm_multi.restype = ci
        lib.ps_mcm_multi_device.argtypes = [vp, ctypes.c_uint, _DPP, i64, ci, ci, ci, _DPP, i64]
        lib.ps_mcm_multi_device.restype = ci
        lib.ps_xi.argtypes = [vp, ci, ci, _DPP, ci, i64, ci, ci, ci, _DPP, i64]
        lib.ps_xi.restype = ci
        lib.ps_coupledcov.argtypes = [vp, ci, _DPP, _DPP, _DPP, i64, ci, ci, ci, _DP, i64]
        lib.ps_coupledcov.restype = ci
        lib.ps_coupledcov_device.argtypes = [vp, ci, _DPP, _DPP, _DPP, i64, ci, ci, ci, _DP, i64]
        lib.ps_coupledcov_device.restype = ci
        lib.ps_coupledcov_set_device.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(_DPP),
                                                 ctypes.POINTER(_DPP), ctypes.POINTER(_DPP), i64, ci, ci, ci, _DPP, i64]
        lib.ps_coupledcov_set_device.restype = ci
        lib.ps_mcm_set_device.argtypes = [vp, ctypes.c_uint, _DPP, ci, i64, ci, ci, ci, _DPP, i64]
        lib.ps_mcm_set_device.restype = ci
        lib.ps_mcm_set.argtypes = [vp, ctypes.c_uint, _DPP, ci, i64, ci, ci, ci, _DPP, i64]
        lib.ps_mcm_set.restype = ci
        lib.ps_batch_prepare.argtypes = [vp, ctypes.POINTER(PSProblem), ci, ci, ci]
        lib.ps_batch_prepare.restype = ci
        lib.ps_batch_run.argtypes = [vp]
        lib.ps_batch_run.restype = ci
        lib.ps_batch_graph_launch.argtypes = [vp]
        lib.ps_batch_graph_launch.restype = ci
        lib.ps_batch_autotune.argtypes = [vp, ctypes.POINTER(PSProblem), ci, ctypes.POINTER(ci), ctypes.POINTER(ci),
                                          ctypes.POINTER(ctypes.c_double)]
        lib.ps_batch_autotune.restype = ci
        lib.ps_decouple_covmat.argtypes = [vp, _DP, _DP, _DP, i64, i64, _DP, i64]
        lib.ps_decouple_covmat.restype = ci
        lib.ps_solve.argtypes = [vp, _DP, i64, i64, _DP, ci, i64, _DP, i64]
        lib.ps_solve.restype = ci
        lib.ps_quickpol_xi.argtypes = [vp, ci, ci, ci, ci, _DP, i64, ci, ci, ci, ci, _DP, i64]
        lib.ps_quickpol_xi.restype = ci
        lib.ps_quickpol_xi_alm.argtypes = [vp, ci, ci, ci, ci, _DP, _DP, ci, ci, ci, ci, ci, ci, _DP, i64]
        lib.ps_quickpol_xi_alm.restype = ci
        lib.ps_decouple_covmat_device.argtypes = [vp, _DP, _DP, _DP, i64, i64, _DP, i64]
        lib.ps_decouple_covmat_device.restype = ci
        lib.ps_window_W.argtypes = [vp, _DPP, _DPP, ci, ci, ci, ci, _DP]
        lib.ps_window_W.restype = ci
        lib.ps_window_W_device.argtypes = [vp, _DPP, _DPP, ci, ci, ci, ci, _DP]
        lib.ps_window_W_device.restype = ci
        lib.ps_last_kernel_ms.argtypes = [vp]
        lib.ps_last_kernel_ms.restype = ctypes.c_double
        lib.ps_launch_count.argtypes = [vp]
        lib.ps_launch_count.restype = u64
        lib.ps_probe_fma_peak.argtypes = [vp, ci, ctypes.POINTER(ctypes.c_double)]
        lib.ps_probe_fma_peak.restype = ci
        _lib = lib
        return lib


def dptr(a):
    """double* of a numpy array (host) or of an int device address."""
    if isinstance(a, int):
        return ctypes.cast(ctypes.c_void_p(a), _DP)
    if a is None:
        return _DP()
    return a.ctypes.data_as(_DP)


def dptr_array(items):
    arr = (_DP * max(len(items), 1))()
    for i, a in enumerate(items):
        arr[i] = dptr(a)
    return arr


def mode_code(mode):
    if isinstance(mode, int):
        return mode
    try:
        return MODES[mode]
    except KeyError:
        raise ValueError("unknown mode %r (use 'plain' or 'chosen')" % (mode,))


class Context:
    """Owns one ps_ctx (device buffers, stream, error message)."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        st = self.lib.ps_create(int(device), ctypes.byref(h))
        if st != PS_OK:
            raise PowerSpectraGPUError(st, "ps_create(%d) failed: no usable CUDA device" % device)
        self.handle = h
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ps_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        if st != PS_OK:
            msg = self.lib.ps_last_error(self.handle).decode(errors="replace")
            cls = PowerSpectraArgumentError if st == PS_ERR_ARG else PowerSpectraGPUError
            raise cls(st, msg)

    def set_stream(self, stream_handle):
        self.check(self.lib.ps_set_stream(self.handle, ctypes.c_void_p(stream_handle or 0)))

    def set_tensor_cores(self, enable):
        """Chosen-mode sets: use the tensor-core kernels where they apply (True, the default) or not."""
        self.check(self.lib.ps_set_tensor_cores(self.handle, 1 if enable else 0))

    def synchronize(self):
        self.check(self.lib.ps_synchronize(self.handle))

    def last_kernel_ms(self):
        return self.lib.ps_last_kernel_ms(self.handle)

    def launch_count(self):
        return int(self.lib.ps_launch_count(self.handle))

    def fma_peak(self, fp64=True):
        out = ctypes.c_double(0.0)
        self.check(self.lib.ps_probe_fma_peak(self.handle, 1 if fp64 else 0, ctypes.byref(out)))
        return out.value

    # ---- raw entry points (host numpy arrays) ----
    def mcm(self, spin, W, lmin, lmax, mode="plain", out=None):
        W = np.ascontiguousarray(W, dtype=np.float64)
        n = lmax - lmin + 1
        M = np.empty((n, n), dtype=np.float64, order="F") if out is None else out
        self.check(self.lib.ps_mcm(self.handle, int(spin), dptr(W), len(W), lmin, lmax, mode_code(mode), dptr(M),
                                   M.shape[0]))
        return M

    def mcm_multi(self, Ws, lmin, lmax, mode="plain", outs=None):
        """Ws: dict spin -> W.  Returns dict spin -> matrix (Fortran order)."""
        cases = 0
        wl, ml = [None] * 4, [None] * 4
        n = lmax - lmin + 1
        nW = None
        keep = []
        for s, W in Ws.items():
            W = np.ascontiguousarray(W, dtype=np.float64)
            keep.append(W)
            nW = len(W) if nW is None else min(nW, len(W))
            cases |= 1 << s
            wl[s] = W
            ml[s] = (outs[s] if outs is not None else np.empty((n, n), dtype=np.float64, order="F"))
        self.check(self.lib.ps_mcm_multi(self.handle, cases, dptr_array(wl), nW or 1, lmin, lmax, mode_code(mode),
                                         dptr_array(ml), n))
        return {s: ml[s] for s in Ws}

    def mcm_multi_device(self, dWs, nW, lmin, lmax, dMs, ldm, mode="plain"):
        """Device-pointer variant: dWs / dMs map spin -> device address (int)."""
        cases = 0
        wl, ml = [None] * 4, [None] * 4
        for s, p in dWs.items():
            cases |= 1 << s
            wl[s] = int(p)
            ml[s] = int(dMs[s])
        self.check(self.lib.ps_mcm_multi_device(self.handle, cases, dptr_array(wl), int(nW), lmin, lmax,
                                                mode_code(mode), dptr_array(ml), int(ldm)))

    def quickpol_xi(self, nu1, nu2, s1, s2, W, lmax, bl, bu, mode="plain", out=None):
        """quickpolXi! (src/beam.jl:72-109) as a dense (lmax+1)^2 matrix, zeros outside the band.
        `out` may supply the F-ordered float64 result (for example page-locked)."""
        W = np.ascontiguousarray(W, dtype=np.float64)
        n = lmax + 1
        X = _result_matrix(out, n)
        self.check(self.lib.ps_quickpol_xi(self.handle, int(nu1), int(nu2), int(s1), int(s2), dptr(W), len(W), lmax,
                                           int(bl), int(bu), mode_code(mode), dptr(X), n))
        return X

    def quickpol_xi_alm(self, nu1, nu2, s1, s2, omega1, omega2, alm_lmax, lmax, bl, bu, alm_mmax=None, mode="plain",
                        out=None):
        """quickpolXi!(Xi, nu1, nu2, s1, s2, omega1, omega2) (src/beam.jl:72-109): W = quickpolW(omega1,
        omega2) and Xi on the GPU, from complex128 scan-weight coefficient sets (HEALPix order).  `out` may
        supply the F-ordered float64 result (for example page-locked)."""
        alm_mmax = alm_lmax if alm_mmax is None else alm_mmax
        nalm = (alm_mmax + 1) * (alm_mmax + 2) // 2 + (alm_mmax + 1) * (alm_lmax - alm_mmax)
        o1 = np.ascontiguousarray(omega1, dtype=np.complex128)
        o2 = o1 if omega2 is omega1 else np.ascontiguousarray(omega2, dtype=np.complex128)
        if o1.shape != (nalm,) or o2.shape != (nalm,):
            raise PowerSpectraArgumentError(PS_ERR_ARG, "a coefficient set needs %d entries" % nalm)
        n = lmax + 1
        X = _result_matrix(out, n)
        self.check(self.lib.ps_quickpol_xi_alm(self.handle, int(nu1), int(nu2), int(s1), int(s2),
                                               dptr(o1.view(np.float64)), dptr(o2.view(np.float64)), alm_lmax,
                                               alm_mmax, lmax, int(bl), int(bu), mode_code(mode), dptr(X), n))
        return X

    def window_W(self, A, B, lmax, mmax=None, lout=None):
        """(1/nterms) sum_t alm2cl(A[t], B[t])[0:lout] for host complex128 coefficient sets in the
        HEALPix m-major order (None = all-zero set).  window_function_W!, src/workspace.jl:174-213."""
        mmax = lmax if mmax is None else mmax
        lout = lmax if lout is None else lout
        if len(A) != len(B):
            raise PowerSpectraArgumentError(PS_ERR_ARG, "A and B need the same number of terms")
        nalm = (mmax + 1) * (mmax + 2) // 2 + (mmax + 1) * (lmax - mmax)
        keep, pa, pb = [], [], []
        for lst, out in ((A, pa), (B, pb)):
            for a in lst:
                if a is None:
                    out.append(None)
                    continue
                a = np.ascontiguousarray(a, dtype=np.complex128)
                if a.shape != (nalm,):
                    raise PowerSpectraArgumentError(PS_ERR_ARG, "a coefficient set needs %d entries" % nalm)
                keep.append(a)
                out.append(a.view(np.float64))
        # an auto-spectrum term names one array twice: pass the same pointer so it is copied once
        for t in range(len(A)):
            if A[t] is not None and A[t] is B[t]:
                pb[t] = pa[t]
        W = np.empty(lout + 1, dtype=np.float64)
        self.check(self.lib.ps_window_W(self.handle, dptr_array(pa), dptr_array(pb), len(A), lmax, mmax, lout,
                                        dptr(W)))
        return W

    def window_W_device(self, dA, dB, lmax, mmax, lout, dW):
        """Device variant: dA / dB are lists of device addresses (int, or None for a zero set)."""
        self.check(self.lib.ps_window_W_device(self.handle, dptr_array([None if a is None else int(a) for a in dA]),
                                               dptr_array([None if b is None else int(b) for b in dB]), len(dA),
                                               lmax, mmax, lout, dptr(int(dW))))

    def decouple_covmat_device(self, dY, dB1, dB2, n, ld, dout, ldout):
        """decouple_covmat on device matrices (addresses as ints)."""
        self.check(self.lib.ps_decouple_covmat_device(self.handle, dptr(int(dY)), dptr(int(dB1)), dptr(int(dB2)), n,
                                                      ld, dptr(int(dout)), ldout))

    def decouple_covmat(self, Y, B1, B2):
        """B1^-1 Y B2^-T (decouple_covmat, src/covariance.jl:8-14) for square float64 matrices."""
        Y, B1, B2 = (np.asfortranarray(x, dtype=np.float64) for x in (Y, B1, B2))
        n = Y.shape[0]
        if Y.shape != (n, n) or B1.shape != (n, n) or B2.shape != (n, n):
            raise PowerSpectraArgumentError(PS_ERR_ARG, "decouple_covmat needs three n x n matrices")
        out = np.empty((n, n), dtype=np.float64, order="F")
        self.check(self.lib.ps_decouple_covmat(self.handle, dptr(Y), dptr(B1), dptr(B2), n, n, dptr(out), n))
        return out

    def solve(self, M, b):
        """M \\ b by LU on the GPU (b: vector or n x nrhs)."""
        M = np.asfortranarray(M, dtype=np.float64)
        vec = np.ndim(b) == 1
        B = np.asfortranarray(np.reshape(b, (len(b), -1)) if vec else b, dtype=np.float64)
        n = M.shape[0]
        if M.shape != (n, n) or B.shape[0] != n:
            raise PowerSpectraArgumentError(PS_ERR_ARG, "solve needs an n x n matrix and n rows of right-hand sides")
        x = np.empty_like(B, order="F")
        self.check(self.lib.ps_solve(self.handle, dptr(M), n, n, dptr(B), B.shape[1], n, dptr(x), n))
        return x[:, 0] if vec else x

    def coupledcov_device(self, kind, dS, dR, dW, nW, lmin, lmax, dC, ldc, mode="chosen"):
        """Device-pointer covariance block (addresses as ints)."""
        k = COV_KINDS[kind] if isinstance(kind, str) else int(kind)
        self.check(self.lib.ps_coupledcov_device(self.handle, k, dptr_array([int(x) for x in dS]),
                                                 dptr_array([int(x) for x in dR]), dptr_array([int(x) for x in dW]),
                                                 int(nW), lmin, lmax, mode_code(mode), dptr(int(dC)), int(ldc)))

    def coupledcov_set_device(self, blocks, nW, lmin, lmax, ldc, mode="chosen"):
        """Several covariance blocks of one grid: `blocks` is a list of (kind, dS, dR, dW, dC) with
        device addresses as ints (dR may be empty for TTEE)."""
        nb = len(blocks)
        kinds = (ctypes.c_int * nb)(*[COV_KINDS[b[0]] if isinstance(b[0], str) else int(b[0]) for b in blocks])
        keep = [(dptr_array([int(x) for x in b[1]]), dptr_array([int(x) for x in b[2]]),
                 dptr_array([int(x) for x in b[3]])) for b in blocks]
        S = (_DPP * nb)(*[ctypes.cast(k[0], _DPP) for k in keep])
        R = (_DPP * nb)(*[ctypes.cast(k[1], _DPP) if len(b[2]) else None for k, b in zip(keep, blocks)])
        W = (_DPP * nb)(*[ctypes.cast(k[2], _DPP) for k in keep])
        C = dptr_array([int(b[4]) for b in blocks])
        self.check(self.lib.ps_coupledcov_set_device(self.handle, nb, kinds, S, R, W, int(nW), lmin, lmax,
                                                     mode_code(mode), C, int(ldc)))

    def mcm_set(self, cases, Ws, lmin, lmax, mode="chosen", outs=None, slots=None):
        """mcm for a set of host spectra on one grid: returns {(k, s): matrix} for window k and each spin
        case s selected in `cases` (F-ordered float64; `outs` may supply them, e.g. page-locked).  With
        `slots` (a set of (k, s)), only those (window, case) slots are computed."""
        Ws = [np.ascontiguousarray(w, dtype=np.float64) for w in Ws]
        n = lmax - lmin + 1
        nW = min(len(w) for w in Ws)
        res, ml = {}, []
        for k in range(len(Ws)):
            for s in range(4):
                if cases & (1 << s) and (slots is None or (k, s) in slots):
                    m = outs[k, s] if outs is not None else np.empty((n, n), dtype=np.float64, order="F")
                    res[k, s] = m
                    ml.append(m)
                else:
                    ml.append(None)
        self.check(self.lib.ps_mcm_set(self.handle, int(cases), dptr_array(Ws), len(Ws), nW, lmin, lmax,
                                       mode_code(mode), dptr_array(ml), n))
        return res

    def mcm_set_device(self, cases, dW, nW, lmin, lmax, dM, ldm, mode="chosen"):
        """Many spectra on one grid: dW list of K device addresses, dM list of 4K
        device addresses (entry 4k+s for spin case s; 0 where unused)."""
        self.check(self.lib.ps_mcm_set_device(self.handle, int(cases), dptr_array([int(x) for x in dW]), len(dW),
                                              int(nW), lmin, lmax, mode_code(mode),
                                              dptr_array([int(x) for x in dM]), int(ldm)))

    def _problems(self, problems):
        arr = (PSProblem * len(problems))()
        keep = []
        for i, pr in enumerate(problems):
            W = dptr_array([int(x) for x in pr["W"]])
            M = dptr_array([int(x) for x in pr["M"]])
            keep += [W, M]
            arr[i] = PSProblem(int(pr.get("lmin", 0)), int(pr["lmax"]), int(pr["cases"]), len(pr["W"]),
                               int(pr["nW"]), ctypes.cast(W, _DPP), ctypes.cast(M, _DPP), int(pr["ldm"]))
        return arr, keep

    def batch_prepare(self, problems, group_slots=0, blocks_per_sm=0):
        """problems: dicts with lmin, lmax, cases, nW, ldm, W (K device addresses),
        M (4K device addresses).  Builds the persistent kernel's work queue."""
        arr, keep = self._problems(problems)
        self._batch_keep = (arr, keep)  # the library keeps pointers only during prepare, but be safe
        self.check(self.lib.ps_batch_prepare(self.handle, arr, len(problems), int(group_slots), int(blocks_per_sm)))

    def batch_run(self):
        self.check(self.lib.ps_batch_run(self.handle))

    def batch_graph_launch(self):
        self.check(self.lib.ps_batch_graph_launch(self.handle))

    def batch_autotune(self, problems):
        arr, keep = self._problems(problems)
        g, b, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
        self.check(self.lib.ps_batch_autotune(self.handle, arr, len(problems), ctypes.byref(g), ctypes.byref(b),
                                              ctypes.byref(ms)))
        return {"group_slots": g.value, "blocks_per_sm": b.value, "ms": ms.value}

    def xi(self, product, parity, Ws, lmin, lmax, mode="plain", outs=None):
        Ws = [np.ascontiguousarray(w, dtype=np.float64) for w in Ws]
        n = lmax - lmin + 1
        if outs is None:
            outs = [np.empty((n, n), dtype=np.float64, order="F") for _ in Ws]
        nW = min(len(w) for w in Ws)
        self.check(self.lib.ps_xi(self.handle, int(product), int(parity), dptr_array(Ws), len(Ws), nW, lmin, lmax,
                                  mode_code(mode), dptr_array(outs), n))
        return outs

    def coupledcov(self, kind, S, R, Ws, lmin, lmax, mode="plain", out=None):
        k = COV_KINDS[kind] if isinstance(kind, str) else int(kind)
        S = [np.ascontiguousarray(s, dtype=np.float64) for s in S]
        R = [np.ascontiguousarray(s, dtype=np.float64) for s in R]
        Ws = [np.ascontiguousarray(w, dtype=np.float64) for w in Ws]
        if k in COV_NWINDOWS and (len(Ws) != COV_NWINDOWS[k] or len(R) != COV_NRATIOS[k] or len(S) != 4):
            raise PowerSpectraArgumentError(PS_ERR_ARG, "kind %d takes 4 spectra, %d ratios and %d windows"
                                            % (k, COV_NRATIOS[k], COV_NWINDOWS[k]))
        for a in S + R:
            if len(a) < lmax + 1:
                raise PowerSpectraArgumentError(PS_ERR_ARG, "spectra and noise ratios need lmax+1 entries")
        n = lmax - lmin + 1
        C = np.empty((n, n), dtype=np.float64, order="F") if out is None else out
        nW = min(len(w) for w in Ws) if Ws else 1
        self.check(self.lib.ps_coupledcov(self.handle, k, dptr_array(S), dptr_array(R), dptr_array(Ws), nW, lmin,
                                          lmax, mode_code(mode), dptr(C), C.shape[0]))
        return C


_default_ctx = None


def default_context():
    """Process-wide context on device 0 (created on first use)."""
    global _default_ctx
    with _lock:
        if _default_ctx is None:
            _default_ctx = Context(int(os.environ.get("PS_GPU_DEVICE", "0")))
        return _default_ctx
