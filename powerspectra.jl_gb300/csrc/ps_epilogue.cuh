// ps_epilogue.cuh -- what a coupling kernel writes for one (l1 <= l2) pair once
// its Xi_k are known: mode-coupling weights (src/modecoupling.jl:90-91), bare
// symmetric Xi, or a covariance element (src/covariance.jl:110-119 and the
// other loop_cov*! formulas).
#pragma once

#include "ps_cov_epilogue.cuh"

namespace ps {

__device__ __forceinline__ void write_pair(const CouplingParams& p, int l1, int l2, const double* Xi)
{
    const long long r1 = l1 - p.lmin, r2 = l2 - p.lmin;
    if (p.epilogue == EPI_MCM) {
#pragma unroll
        for (int k = 0; k < kMaxWin; ++k) {
            if (k < p.nwin) {
                p.out[k][r1 + r2 * p.ldo] = (2.0 * l2 + 1.0) * Xi[k];
                p.out[k][r2 + r1 * p.ldo] = (2.0 * l1 + 1.0) * Xi[k];
            }
        }
    } else if (p.epilogue == EPI_XI) {
#pragma unroll
        for (int k = 0; k < kMaxWin; ++k) {
            if (k < p.nwin) {
                p.out[k][r1 + r2 * p.ldo] = Xi[k];
                p.out[k][r2 + r1 * p.ldo] = Xi[k];
            }
        }
    } else {
        double c = cov_combine(p.cov_kind, p.S, p.R, Xi, l1, l2);
        p.out[0][r1 + r2 * p.ldo] = c;
        p.out[0][r2 + r1 * p.ldo] = c;
    }
}

// l1 = 0: the only l3 is l2, f00^2 = 1/(2 l2 + 1), and the 22 family is zero.
__device__ __forceinline__ void xi_single_term(const CouplingParams& p, int l2, double* Xi)
{
#pragma unroll
    for (int k = 0; k < kMaxWin; ++k) {
        Xi[k] = 0.0;
        if (k < p.nwin && p.win[k].product == PROD_00_00 && p.win[k].parity != PAR_ODD)
            Xi[k] = __ldg(p.win[k].wW + l2) / (2.0 * l2 + 1.0) * kInv4Pi;
    }
}

}  // namespace ps
