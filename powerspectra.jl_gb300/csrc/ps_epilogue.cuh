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

// Tiled writes.  The warps of a block hold kTileRows consecutive rows l1 of
// one 32-column block of l2 (rows outside have l1 = -1).  Each warp writes
// its column half (column l1, rows l2: 32 consecutive doubles) directly.  The
// row half (row l1, columns l2) would be 32 single doubles ldo apart; it goes
// through shared memory instead, and the block writes it as kTileRows
// consecutive doubles per column.  That matters most for page-locked host
// outputs, where single scattered doubles cross the chip-to-host link one by one.
struct TileRows {
    int l1[kTileRows];
    int l2_0[kTileRows];
    unsigned act[kTileRows];  // lanes with a pair to write
};
static_assert(kTileRows == kWarpsPerBlock, "one tile row per warp");

// `stage` holds each warp's row-half values: warp w's at stage + w * stride,
// [NOUT][32] doubles, in shared memory that warp w no longer uses.  All threads
// of the block call this once.
template <int NOUT>
__device__ __forceinline__ void write_tile(const CouplingParams& p, int l1, int l2_0, bool active, const double* Xi,
                                           double* stage, int stride, TileRows& rows, int warp, int lane)
{
    const int nout = p.epilogue == EPI_COV ? 1 : (p.nwin < NOUT ? p.nwin : NOUT);
    if (l1 >= 0) {
        const int l2 = l2_0 + lane;
        const long long r1 = l1 - p.lmin, r2 = l2 - p.lmin;
        double* st = stage + warp * stride;
        if (p.epilogue == EPI_COV) {
            const double c = active ? cov_combine(p.cov_kind, p.S, p.R, Xi, l1, l2) : 0.0;
            if (active) p.out[0][r2 + r1 * p.ldo] = c;
            st[lane] = c;
        } else {
#pragma unroll
            for (int k = 0; k < NOUT; ++k) {
                if (k < nout) {
                    const double x = Xi[k];
                    const bool mcm = p.epilogue == EPI_MCM;
                    if (active) p.out[k][r2 + r1 * p.ldo] = mcm ? (2.0 * l1 + 1.0) * x : x;
                    st[k * 32 + lane] = mcm ? (2.0 * l2 + 1.0) * x : x;
                }
            }
        }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active && l1 >= 0);
    if (lane == 0) {
        rows.l1[warp] = l1;
        rows.l2_0[warp] = l2_0;
        rows.act[warp] = act;
    }
    __syncthreads();
    // thread (column c, row q): kTileRows consecutive threads write one column's run
    const int q = threadIdx.x % kTileRows, c = threadIdx.x / kTileRows;
    if (c < 32 && ((rows.act[q] >> c) & 1u)) {
        const long long r1 = rows.l1[q] - p.lmin, r2 = rows.l2_0[q] + c - p.lmin;
        const double* st = stage + q * stride;
#pragma unroll
        for (int k = 0; k < NOUT; ++k)
            if (k < nout) p.out[k][r1 + r2 * p.ldo] = st[k * 32 + c];
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
