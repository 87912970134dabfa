"""Generate the committed golden fixtures under tests/golden/.

  namaster_diag.npz   the reference test suite's NaMaster golden vectors
                      (test/data/mcm_{TT,EE,TE}_diag.txt: diagonals of the TT,
                      ++ and TE mode-coupling matrices of one mask, l = 2..766),
                      read from the reference checkout and stored as float64.
  w3j_exact.json      arbitrary-precision 3j values (mpmath Racah sum) for the
                      (0 0 0) and (-2 2 0) families at random (l1, l2, l3) up to
                      l = 8191, plus family-edge points.
  decouple_3x3.json   the 3x3 known answer of the reference's decouple_covmat test
                      (test/test_covmat.jl:11-17: A, B1, B2 and inv(B1) A inv(B2)'),
                      parsed from the reference test file.
  oracle_small.npz    oracle matrices (mode coupling, all spin cases, two window
                      lengths; all seven covariance kinds) at small lmax, to pin
                      the oracle against accidental change.
  theory_noise.npz    the reference test suite's signal and noise spectra
                      (test/data/theory.csv: cltt, clte, clee, clbb; noise.csv:
                      nltt, nlee; l = 0..767), read from the reference checkout.

Run from the repository root:  python tests/golden/make_golden.py --ref PATH
(PATH: a checkout of PowerSpectra.jl; it is needed for every fixture but oracle_small.npz).
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "powerspectra.jl_gb300"))


def make_namaster(ref):
    d = os.path.join(ref, "test", "data")
    out = {k: np.loadtxt(os.path.join(d, "mcm_%s_diag.txt" % k)) for k in ("TT", "EE", "TE")}
    np.savez(os.path.join(HERE, "namaster_diag.npz"), **out)
    print("namaster_diag.npz", {k: v.shape for k, v in out.items()})


def make_theory_noise(ref):
    d = os.path.join(ref, "test", "data")
    out = {}
    for fname in ("theory.csv", "noise.csv"):
        with open(os.path.join(d, fname)) as f:
            cols = f.readline().strip().split(",")
            data = np.loadtxt(f, delimiter=",")
        for i, c in enumerate(cols[1:], start=1):
            out[c] = data[:, i]
        assert np.array_equal(data[:, 0], np.arange(len(data)))
    np.savez(os.path.join(HERE, "theory_noise.npz"), **out)
    print("theory_noise.npz", {k: v.shape for k, v in out.items()})


def make_decouple(ref):
    import re
    src = open(os.path.join(ref, "test", "test_covmat.jl")).read()
    mats = {}
    for name in ("A", "B1", "B2"):
        m = re.search(r"^\s*%s = \[([^\]]*)\]" % name, src, flags=re.M)
        rows = [[float(x) for x in r.split()] for r in m.group(1).split(";")]
        mats[name] = rows
    A, B1, B2 = (np.array(mats[k]) for k in ("A", "B1", "B2"))
    want = np.linalg.inv(B1) @ A @ np.linalg.inv(B2).T  # Cref = inv(B1) * (A) * (inv(B2)'), test_covmat.jl:15
    with open(os.path.join(HERE, "decouple_3x3.json"), "w") as f:
        json.dump({"A": mats["A"], "B1": mats["B1"], "B2": mats["B2"], "expected": want.tolist()}, f, indent=1)
    print("decouple_3x3.json")


def make_exact():
    from oracle.exact3j import w3j
    rng = np.random.default_rng(20261203)
    pts = []
    fams = ((0, 0), (-2, 2))
    for (m1, m2) in fams:
        for i in range(60):
            lmax = [64, 767, 3071, 8191][i % 4]
            l1 = int(rng.integers(0 if m1 == 0 else 2, lmax + 1))
            l2 = int(rng.integers(0 if m1 == 0 else 2, lmax + 1))
            jmin, jmax = abs(l1 - l2), l1 + l2
            cand = [int(rng.integers(jmin, jmax + 1)), jmin, jmax, (jmin + jmax) // 2]
            for l3 in cand:
                if m1 == 0 and (l1 + l2 + l3) % 2:
                    l3 = min(l3 + 1, jmax) if (l1 + l2 + l3 + 1) % 2 == 0 and l3 + 1 <= jmax else l3 - 1
                pts.append((l1, l2, l3, m1, m2))
    # small exhaustive families
    for l1 in range(0, 7):
        for l2 in range(0, 7):
            for l3 in range(abs(l1 - l2), l1 + l2 + 1):
                for (m1, m2) in fams:
                    pts.append((l1, l2, l3, m1, m2))
    pts = sorted(set(pts))
    rows = []
    for (l1, l2, l3, m1, m2) in pts:
        v = w3j(l1, l2, l3, m1, m2, -m1 - m2)
        rows.append([l1, l2, l3, m1, m2, str(v)])
    with open(os.path.join(HERE, "w3j_exact.json"), "w") as f:
        json.dump({"note": "(l1 l2 l3; m1 m2 -m1-m2) by mpmath Racah sum, ~40 digits", "rows": rows}, f, indent=0)
    print("w3j_exact.json", len(rows), "values")


def make_oracle_small():
    from oracle import oracle as o
    from powerspectra_gpu import synthetic as syn
    out = {}
    L = 40
    for nWname, nW in (("2L1", 2 * L + 1), ("L1", L + 1)):
        W = syn.mask_spectrum(nW, 0.6, 30.0, seed=11)
        out["W_" + nWname] = W
        for spin in range(4):
            out["M%d_%s" % (spin, nWname)] = o.inner_mcm(spin, W, 0, L)
    out["M0_lmin5"] = o.inner_mcm(0, out["W_2L1"], 5, L)
    Lc = 32
    ws_key = lambda k: syn.window_for_key(("golden",) + tuple(k), Lc)
    spectra, noise = syn.signal_spectra(Lc)
    f = syn.FIELDS
    S = [spectra["TT", f[0], f[2]], spectra["EE", f[1], f[3]], spectra["TE", f[0], f[3]], spectra["TE", f[1], f[2]]]
    R = [noise["TT", f[0], f[0]], noise["EE", f[1], f[1]], noise["TT", f[0], f[2]], noise["EE", f[1], f[3]]]
    Ws = [ws_key((k,)) for k in range(8)]
    for k in range(8):
        out["cov_W%d" % k] = Ws[k]
    for i in range(4):
        out["cov_S%d" % i] = S[i]
        out["cov_R%d" % i] = R[i]
    for name, kind in o.COV_KINDS.items():
        nw, nr = o.COV_NWINDOWS[name], o.COV_NRATIOS[name]
        out["cov_" + name] = o.loop_cov(name, S, R[:nr], Ws[:nw], 0, Lc)
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("oracle_small.npz", len(out), "arrays")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="a checkout of PowerSpectra.jl (its test/ folder is read)")
    ap.add_argument("--only", default="all")
    a = ap.parse_args()
    if a.only != "oracle" and not a.ref:
        ap.error("--ref PATH (a PowerSpectra.jl checkout) is required for the fixtures read from its tests")
    if a.only in ("all", "namaster"):
        make_namaster(a.ref)
    if a.only in ("all", "decouple"):
        make_decouple(a.ref)
    if a.only in ("all", "theory"):
        make_theory_noise(a.ref)
    if a.only in ("all", "oracle"):
        make_oracle_small()
    if a.only in ("all", "exact"):
        make_exact()
