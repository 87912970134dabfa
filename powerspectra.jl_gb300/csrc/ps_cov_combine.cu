// ps_cov_combine.cu -- a covariance block from Xi matrices computed beforehand.
//
// ps_coupledcov_set_device computes the Xi of every window of the blocks whose
// windows all use the squared (0 0 0) family (TTTT, TTTE, TTEE) in shared
// tensor-core launches, then forms each block here with the same per-element
// formula the fused epilogue of the coupling kernel uses (ps_cov_epilogue.cuh,
// after src/covariance.jl:110-118, :225-230, :438-441).  Memory-bound: one
// read of the block's K Xi and one write of C per element.
#include "ps_internal.cuh"
#include "ps_cov_epilogue.cuh"

namespace ps {
namespace {

// blockIdx.y: column l2 - lmin; threads: rows l1 - lmin (coalesced, column-major)
__global__ void __launch_bounds__(256) k_cov_combine(const CovCombineParams p)
{
    const int j = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n || j >= p.n) return;
    double x[kMaxWin];
#pragma unroll
    for (int k = 0; k < kMaxWin; ++k) x[k] = k < p.nx ? p.X[k][i + (long long)j * p.ldx] : 0.0;
    // the formula with (a, b) = (smaller, larger) l, as the fused epilogue evaluates it for a
    // pair l1 <= l2, so that C is exactly symmetric
    p.C[i + (long long)j * p.ldc] = cov_combine(p.kind, p.S, p.R, x, p.lmin + min(i, j), p.lmin + max(i, j));
}

}  // namespace

cudaError_t launch_cov_combine(const CovCombineParams& p, cudaStream_t s)
{
    if (p.n <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((p.n + 255) / 256), (unsigned)p.n);
    k_cov_combine<<<grid, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace ps
