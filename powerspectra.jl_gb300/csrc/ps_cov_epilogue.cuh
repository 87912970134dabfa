// ps_cov_epilogue.cuh -- per-pair combination of the Xi_k into a covariance
// element, one formula per loop_cov*! kernel of the reference.  The
// expressions keep the reference's operand order (left-associative products)
// so the FP64 results agree with it to rounding.
#pragma once

#include "ps_internal.cuh"

namespace ps {

// X[k] are the Xi of windows W1..Wk (already divided by 4pi); a = l1, b = l2.
__device__ __forceinline__ double cov_combine(int kind, const double* const* S, const double* const* R,
                                              const double* X, int a, int b)
{
    switch (kind) {
    case PS_COV_TTTT:
    case PS_COV_EEEE: {  // src/covariance.jl:110-118 (TTTT), :171-179 (EEEE)
        const double *ip = S[0], *jq = S[1], *iq = S[2], *jp = S[3];
        const double *rip = R[0], *rjq = R[1], *riq = R[2], *rjp = R[3];
        return sqrt(ip[a] * ip[b] * jq[a] * jq[b]) * X[0] + sqrt(iq[a] * iq[b] * jp[a] * jp[b]) * X[1] +
               sqrt(ip[a] * ip[b]) * X[2] * rjq[a] * rjq[b] + sqrt(jq[a] * jq[b]) * X[3] * rip[a] * rip[b] +
               sqrt(iq[a] * iq[b]) * X[4] * rjp[a] * rjp[b] + sqrt(jp[a] * jp[b]) * X[5] * riq[a] * riq[b] +
               X[6] * rip[a] * rjq[a] * rip[b] * rjq[b] + X[7] * riq[a] * rjp[a] * riq[b] * rjp[b];
    }
    case PS_COV_TTTE: {  // src/covariance.jl:225-230
        const double *TTip = S[0], *TTjp = S[1], *TEiq = S[2], *TEjq = S[3];
        const double *rip = R[0], *rjp = R[1];
        return (sqrt(TTip[a] * TTip[b]) * (TEjq[a] + TEjq[b]) * X[0] +
                sqrt(TTjp[a] * TTjp[b]) * (TEiq[a] + TEiq[b]) * X[1] + (TEjq[a] + TEjq[b]) * X[2] * rip[a] * rip[b] +
                (TEiq[a] + TEiq[b]) * X[3] * rjp[a] * rjp[b]) /
               2;
    }
    case PS_COV_TETE: {  // src/covariance.jl:292-297
        const double *TTip = S[0], *EEjq = S[1], *TEiq = S[2], *TEjp = S[3];
        const double *rT = R[0], *rP = R[1];
        return sqrt(TTip[a] * TTip[b] * EEjq[a] * EEjq[b]) * X[0] +
               0.5 * (TEiq[a] * TEjp[b] + TEjp[a] * TEiq[b]) * X[1] + sqrt(TTip[a] * TTip[b]) * X[2] * rP[a] * rP[b] +
               sqrt(EEjq[a] * EEjq[b]) * X[3] * rT[a] * rT[b] + X[4] * rT[a] * rT[b] * rP[a] * rP[b];
    }
    case PS_COV_TEEE:
    case PS_COV_TEEE_PLANCK: {  // src/covariance.jl:362-367 and :392-397
        const double *EEjq = S[0], *EEjp = S[1], *TEip = S[2], *TEiq = S[3];
        const double *rjq = R[0], *rjp = R[1];
        return (sqrt(EEjq[a] * EEjq[b]) * (TEip[a] + TEip[b]) * X[0] +
                sqrt(EEjp[a] * EEjp[b]) * (TEiq[a] + TEiq[b]) * X[1] + (TEip[a] + TEip[b]) * X[2] * rjq[a] * rjq[b] +
                (TEiq[a] + TEiq[b]) * X[3] * rjp[a] * rjp[b]) /
               2;
    }
    default: {  // PS_COV_TTEE, src/covariance.jl:438-441
        const double *TEip = S[0], *TEiq = S[1], *TEjq = S[2], *TEjp = S[3];
        return ((TEip[a] * TEjq[b] + TEjq[a] * TEip[b]) * X[0] + (TEiq[a] * TEjp[b] + TEjp[a] * TEiq[b]) * X[1]) / 2;
    }
    }
}

}  // namespace ps
