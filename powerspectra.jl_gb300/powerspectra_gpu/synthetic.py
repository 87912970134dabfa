"""Seeded synthetic inputs of the benchmark and test configurations.

The reference's own inputs (Planck / NaMaster mask maps) need network access
or are not shipped, so every workload uses mask spectra of one fixed
functional form,

    W_l = f_sky^2 * 4 pi * delta_l0 + A (l+1)^-2 exp(-l(l+1) / (2 c^2)) (1 + 0.05 N(0,1)),

and signal spectra Cl = C0 (l/80)^-2.4 (TT, EE), TE = 0.3 sqrt(TT EE), with
white noise of 10-45 uK.arcmin, N_l = (sigma pi / 10800)^2.
"""
import hashlib
import math

import numpy as np


def mask_spectrum(nW, fsky, cutoff, A=1e-3, seed=0):
    """0-indexed W_l for l = 0..nW-1 of the form above."""
    rng = np.random.default_rng(seed)
    l = np.arange(nW, dtype=np.float64)
    W = A * (l + 1.0) ** -2 * np.exp(-l * (l + 1.0) / (2.0 * cutoff * cutoff)) * (1.0 + 0.05 * rng.standard_normal(nW))
    W[0] += fsky * fsky * 4.0 * math.pi
    return W


# ---- configuration 1: plain TT, lmax 767 -------------------------------------------------------
def tt_767(seed=0):
    """One mask cross-spectrum, l = 0..1534, f_sky 0.6, cutoff 300 (TT at lmax 767)."""
    return {"lmax": 767, "W": mask_spectrum(1535, 0.6, 300.0, seed=seed)}


# ---- configuration 2: all spin cases, lmax 3071 ------------------------------------------------
def all_spins(lmax=3071, seed=1):
    """Temperature (f_sky 0.7, cutoff 800) and polarisation (f_sky 0.5, cutoff 600) mask
    spectra, plus their TxP cross-spectrum (f_sky sqrt(0.35), cutoff sqrt(800*600)), with
    nW = 2 lmax + 1 so every l3 of every family is covered."""
    nW = 2 * lmax + 1
    WT = mask_spectrum(nW, 0.7, 800.0, seed=seed)
    WP = mask_spectrum(nW, 0.5, 600.0, seed=seed + 1)
    WTP = mask_spectrum(nW, math.sqrt(0.7 * 0.5), math.sqrt(800.0 * 600.0), seed=seed + 2)
    return {"lmax": lmax, "nW": nW, "WT": WT, "WP": WP, "WTP": WTP}


# ---- configuration 3: covariance blocks, lmax 2508 ---------------------------------------------
FIELDS = ("100_hm1", "143_hm1", "100_hm2", "143_hm2")  # i, j, p, q: 2 frequencies x 2 half-missions


def _key_seed(key):
    return int.from_bytes(hashlib.sha256(repr(key).encode()).digest()[:8], "little")


def window_for_key(key, lmax):
    """Deterministic window spectrum for a window_function_W key, f_sky in 0.4-0.8."""
    s = _key_seed(key)
    rng = np.random.default_rng(s)
    fsky = float(rng.uniform(0.4, 0.8))
    cutoff = float(rng.uniform(500.0, 900.0))
    return mask_spectrum(lmax + 1, fsky, cutoff, seed=s % (2 ** 32))


def signal_spectra(lmax, fields=FIELDS, seed=3):
    l = np.arange(lmax + 1, dtype=np.float64)
    base = np.zeros(lmax + 1)
    base[2:] = (l[2:] / 80.0) ** -2.4
    TT, EE = 1000.0 * base, 40.0 * base
    TE = 0.3 * np.sqrt(TT * EE)
    spectra = {}
    for a in fields:
        for b in fields:
            spectra["TT", a, b] = TT.copy()
            spectra["EE", a, b] = EE.copy()
            spectra["TE", a, b] = TE.copy()
    rng = np.random.default_rng(seed)
    sig = {f: float(rng.uniform(10.0, 45.0)) for f in fields}  # uK.arcmin
    noise = {}
    for a in fields:
        for b in fields:
            for X in ("TT", "EE"):
                if a == b:
                    s = sig[a] * (math.sqrt(2.0) if X == "EE" else 1.0)
                    n_l = (s * math.pi / 10800.0) ** 2
                    noise[X, a, b] = np.full(lmax + 1, math.sqrt(n_l / (20.0 * math.pi / 10800.0) ** 2))
                else:
                    noise[X, a, b] = np.ones(lmax + 1)
    return spectra, noise


def covariance_inputs(lmax=2508):
    from .covariance import WindowWorkspace
    ws = WindowWorkspace(FIELDS, lmax, lambda *key: window_for_key(key, lmax))
    spectra, noise = signal_spectra(lmax)
    return ws, spectra, noise


COV_BLOCKS = (("TT", "TT"), ("EE", "EE"), ("TE", "TE"), ("TT", "TE"), ("TT", "EE"), ("TE", "EE"))


# ---- configuration 4: batched uneven problems --------------------------------------------------
def batched_problems(n=64, seed=4, lmax_choices=(511, 1023, 2047, 3071, 4095, 6143), kmax=16):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(n):
        lmax = int(rng.choice(lmax_choices))
        K = int(rng.integers(1, kmax + 1))
        spin = int(rng.choice((0, 2)))
        Ws = [mask_spectrum(lmax + 1, float(rng.uniform(0.4, 0.8)), float(rng.uniform(300, 900)),
                            seed=int(rng.integers(2 ** 31))) for _ in range(K)]
        probs.append({"lmax": lmax, "K": K, "spin": spin, "W": Ws})
    return probs


def small_batch(n=256, seed=7, lmax_choices=(64, 96, 128, 192, 256, 384, 512, 768, 1023), kmax=4):
    """Many small uneven problems (where a launch per window group is mostly ramp and tail)."""
    return batched_problems(n=n, seed=seed, lmax_choices=lmax_choices, kmax=kmax)


# ---- configuration 5: large coupling set, lmax 8191 --------------------------------------------
def large_set(lmax=8191, K=20, seed=5):
    nW = 2 * lmax + 1
    rng = np.random.default_rng(seed)
    return {"lmax": lmax, "nW": nW,
            "W": [mask_spectrum(nW, float(rng.uniform(0.4, 0.8)), float(rng.uniform(400, 1200)),
                                seed=int(rng.integers(2 ** 31))) for _ in range(K)]}
