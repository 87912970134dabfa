// ps_window.cu -- mask power spectra W_l from harmonic coefficients (alm2cl) on the GPU.
//
// Replaces the alm2cl reductions that feed the coupling kernels:
//   * window_function_W! (src/workspace.jl:174-213): the average over the
//     (wX, wY) weight terms of alm2cl(w_X, w_Y)[0:lmax] (Planck 2015 eq. C.11-C.16);
//   * the mask cross-spectrum of mcm (src/modecoupling.jl:197, :234) and the
//     pseudo-spectra of master (src/modecoupling.jl:357-373), one term each;
//   * quickpolW (src/beam.jl:40-53), the same sum without the 1 / (2l + 1).
//
// The cross-spectrum of two coefficient sets of a real field is the published
// definition
//     cl[l] = ( Re(a_l0 conj b_l0) + 2 sum_{m=1}^{min(l, mmax)} Re(a_lm conj b_lm) ) / (2l + 1),
// with the coefficients in the HEALPix m-major order: (l, m) at
// m (2 lmax + 1 - m) / 2 + l.
//
// Each coefficient costs 16 bytes per set, read once, and two FP64 FMAs.  On
// GB300 (FP64 FMA pipe about 0.53e12 FMA/s) the two limits are close: a cross
// spectrum at lmax 8191 needs about 160 us of HBM time and 127 us of FP64 time.
// Thread l of a block reads (l, m) for the m of its block's m-chunk; the 32
// lanes of a warp hold consecutive l at the same m, so each load is 512
// contiguous bytes.  Partial sums per (term, m-chunk, l) go to a scratch array
// and a second kernel adds them in a fixed order, so results do not depend on
// scheduling (no atomics).
#include "ps_internal.cuh"

namespace ps {

namespace {

constexpr int kAlmThreads = 256;

__global__ void __launch_bounds__(kAlmThreads) k_alm2cl_partial(AlmParams p)
{
    const int l = blockIdx.x * kAlmThreads + threadIdx.x;
    const int c = blockIdx.y, t = blockIdx.z;
    const double2* __restrict__ a = p.a[t];
    const double2* __restrict__ b = p.b[t];
    const int m0 = c * p.mchunk;
    double acc = 0.0;
    if (l <= p.lout && a && b) {
        // GB300's FP64 pipe is the limit here, not HBM: each coefficient costs
        // exactly two FP64 FMAs into the running sum of the m >= 1 terms; the
        // m = 0 term is kept apart and the factor 2 applied once at the end.
        const int m1 = min(min(m0 + p.mchunk - 1, p.mmax), l);
        long long idx = (long long)m0 * (2 * p.lmax + 1 - m0) / 2 + l;  // (l, m0)
        double acc0 = 0.0, accy = 0.0;  // acc: real parts, accy: imaginary parts (two FMA chains)
        int m = m0;
        if (m == 0) {  // the (l, 0) term, counted once
            const double2 z = __ldg(a + idx), u = __ldg(b + idx);
            acc0 = fma(z.x, u.x, z.y * u.y);
            idx += p.lmax;  // (l, 1)
            m = 1;
        }
        if (a == b) {
#pragma unroll 4
            for (; m <= m1; ++m) {
                const double2 v = __ldg(a + idx);
                acc = fma(v.x, v.x, acc);
                accy = fma(v.y, v.y, accy);
                idx += p.lmax - m;  // (l, m + 1)
            }
        } else {
#pragma unroll 4
            for (; m <= m1; ++m) {
                const double2 v = __ldg(a + idx), w = __ldg(b + idx);
                acc = fma(v.x, w.x, acc);
                accy = fma(v.y, w.y, accy);
                idx += p.lmax - m;
            }
        }
        acc = fma(2.0, acc + accy, acc0);
    }
    if (l <= p.lout) p.partial[((long long)t * p.nmchunks + c) * (p.lout + 1) + l] = acc;
}

// W[l] = scale * sum_t (sum_c partial[t][c][l]) / (2l + 1), in a fixed order
// (without the 1 / (2l + 1) when per_l is 0: the scan-pattern spectrum of quickpolW).
__global__ void k_alm2cl_reduce(const double* __restrict__ partial, int nterms, int nmchunks, int lout, double scale,
                                int per_l, double* __restrict__ W)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lout) return;
    const double inv = per_l ? 1.0 / (2.0 * l + 1.0) : 1.0;
    double s = 0.0;
    for (int t = 0; t < nterms; ++t) {
        double ct = 0.0;
        const double* q = partial + (long long)t * nmchunks * (lout + 1) + l;
#pragma unroll 16
        for (int c = 0; c < nmchunks; ++c) ct += __ldg(q + (long long)c * (lout + 1));  // loads issue ahead of the adds
        s += ct * inv;
    }
    W[l] = s * scale;
}

}  // namespace

int alm2cl_chunks(int mmax) { return (mmax + kAlmChunk) / kAlmChunk; }

cudaError_t launch_alm2cl(const AlmParams& p, double scale, bool per_l, double* W, cudaStream_t s,
                          cudaEvent_t after_partial)
{
    dim3 grid((p.lout + kAlmThreads) / kAlmThreads, p.nmchunks, p.nterms);
    k_alm2cl_partial<<<grid, kAlmThreads, 0, s>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (after_partial && (e = cudaEventRecord(after_partial, s)) != cudaSuccess) return e;
    k_alm2cl_reduce<<<(p.lout + 128) / 128, 128, 0, s>>>(p.partial, p.nterms, p.nmchunks, p.lout, scale, per_l ? 1 : 0, W);
    return cudaGetLastError();
}

}  // namespace ps
