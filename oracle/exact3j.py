"""Arbitrary-precision Wigner 3j symbols (mpmath), the stand-in for the
reference's BigFloat 3j spot checks.

TEST INFRASTRUCTURE ONLY.  Racah's single-sum formula,

  (l1 l2 l3; m1 m2 m3) = (-1)^(l1-l2-m3) sqrt(Delta(l1 l2 l3) prod (l_i +- m_i)!)
      * sum_k (-1)^k / [k! (l3-l2+k+m1)! (l3-l1+k-m2)! (l1+l2-l3-k)! (l1-k-m1)! (l2-k+m2)!],

evaluated with consecutive-term ratios at a working precision chosen from the
size of the largest term, so the alternating sum keeps ~40 correct digits.
"""
import math

import mpmath as mp


def w3j(l1, l2, l3, m1, m2, m3):
    if m1 + m2 + m3 != 0 or l3 < abs(l1 - l2) or l3 > l1 + l2:
        return mp.mpf(0)
    if abs(m1) > l1 or abs(m2) > l2 or abs(m3) > l3:
        return mp.mpf(0)
    if m1 == 0 and m2 == 0 and (l1 + l2 + l3) % 2:
        return mp.mpf(0)
    kmin = max(0, l2 - l3 - m1, l1 - l3 + m2)
    kmax = min(l1 + l2 - l3, l1 - m1, l2 + m2)
    lf = lambda n: math.lgamma(n + 1)

    def lterm(k):
        return -(lf(k) + lf(l3 - l2 + k + m1) + lf(l3 - l1 + k - m2) + lf(l1 + l2 - l3 - k) + lf(l1 - k - m1)
                 + lf(l2 - k + m2))

    lpre = 0.5 * (lf(l1 + l2 - l3) + lf(l1 - l2 + l3) + lf(-l1 + l2 + l3) - lf(l1 + l2 + l3 + 1) + lf(l1 + m1)
                  + lf(l1 - m1) + lf(l2 + m2) + lf(l2 - m2) + lf(l3 + m3) + lf(l3 - m3))
    maxterm = max(lterm(k) for k in range(kmin, kmax + 1))
    canc = (lpre + maxterm + 3 * math.log(l1 + l2 + l3 + 2)) / math.log(10)
    dps = int(max(canc, 0)) + 45
    with mp.workdps(dps):
        LF = lambda n: mp.loggamma(n + 1)
        t = mp.exp(-(LF(kmin) + LF(l3 - l2 + kmin + m1) + LF(l3 - l1 + kmin - m2) + LF(l1 + l2 - l3 - kmin)
                     + LF(l1 - kmin - m1) + LF(l2 - kmin + m2)))
        tot = mp.mpf(0)
        sgn = -1 if kmin % 2 else 1
        for k in range(kmin, kmax + 1):
            tot += sgn * t
            num = (l1 + l2 - l3 - k) * (l1 - k - m1) * (l2 - k + m2)
            den = (k + 1) * (l3 - l2 + k + 1 + m1) * (l3 - l1 + k + 1 - m2)
            t = t * num / den
            sgn = -sgn
        pre = mp.exp((LF(l1 + l2 - l3) + LF(l1 - l2 + l3) + LF(-l1 + l2 + l3) - LF(l1 + l2 + l3 + 1) + LF(l1 + m1)
                      + LF(l1 - m1) + LF(l2 + m2) + LF(l2 - m2) + LF(l3 + m3) + LF(l3 - m3)) / 2)
        res = pre * tot * (-1 if (l1 - l2 - m3) % 2 else 1)
        return +res
