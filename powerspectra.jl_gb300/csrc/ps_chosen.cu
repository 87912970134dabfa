// ps_chosen.cu -- launches of the chosen coupling kernel (ps_chosen_task.cuh)
// for window groups of up to 5 slots, and the window preparation kernels.
// Groups of 6-8 slots are instantiated in ps_chosen8.cu, the batched kernel in
// ps_batch_chosen.cu, so the three compile in parallel.
#include "ps_chosen_task.cuh"

namespace ps {

cudaError_t launch_chosen8(const CouplingParams& p, uint32_t spec, bool n00, bool n22, cudaStream_t s);

cudaError_t launch_chosen(const CouplingParams& p, cudaStream_t s)
{
    bool n00 = false, n22 = false;
    for (int k = 0; k < p.nwin; ++k) {
        if (p.win[k].product != PROD_22_22) n00 = true;
        if (p.win[k].product != PROD_00_00) n22 = true;
    }
    const uint32_t spec = spec_of(p);
    const int nw = p.nwin;
    if (p.ntasks <= 0) return cudaSuccess;
    // the smallest instantiation whose slot list starts with this configuration
    if (spec_fits(spec, nw, W00, 1)) return launch_cfg<1, W00>(p, n00, n22, s);
    if (spec_fits(spec, nw, W02, 1)) return launch_cfg<1, W02>(p, n00, n22, s);
    if (spec_fits(spec, nw, WPP, 1)) return launch_cfg<1, WPP>(p, n00, n22, s);
    if (spec_fits(spec, nw, WMM, 1)) return launch_cfg<1, WMM>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_PPMM, 2)) return launch_cfg<2, S_PPMM>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(W00, 4), 4)) return launch_cfg<4, rep(W00, 4)>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_PPMM2, 4)) return launch_cfg<4, S_PPMM2>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_MCM4, 4)) return launch_cfg<4, S_MCM4>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(W02, 4), 4)) return launch_cfg<4, rep(W02, 4)>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(WPP, 4), 4)) return launch_cfg<4, rep(WPP, 4)>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(WMM, 4), 4)) return launch_cfg<4, rep(WMM, 4)>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_TETE, 5)) return launch_cfg<5, S_TETE>(p, n00, n22, s);
    if (nw <= 1) return launch_cfg<1, 0>(p, n00, n22, s);
    if (nw <= 2) return launch_cfg<2, 0>(p, n00, n22, s);
    if (nw <= 4) return launch_cfg<4, 0>(p, n00, n22, s);
    return launch_chosen8(p, spec, n00, n22, s);
}

// (2 l3 + 1) W[l3] in FP64 -> (float mantissa in [0.5, 1), exponent); zeros -> (0, kZeroExp)
__global__ void k_split_windows(int2* __restrict__ dst, const double* __restrict__ wW, int wlen)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < wlen; j += gridDim.x * blockDim.x) {
        double v = wW[j];
        int e = 0;
        double m = (v == 0.0) ? 0.0 : frexp(v, &e);
        dst[j] = (v == 0.0) ? make_int2(0, kZeroExp) : make_int2(__float_as_int((float)m), e);
    }
}

// All windows of a batch in one launch: pad + premultiply + split.
__global__ void k_prep_windows(const WinPrep* __restrict__ list, int n)
{
    const WinPrep w = list[blockIdx.y];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < w.wlen; j += gridDim.x * blockDim.x) {
        double v = (j < w.nW) ? (2.0 * j + 1.0) * w.src[j] : 0.0;
        w.wW[j] = v;
        int e = 0;
        double m = (v == 0.0) ? 0.0 : frexp(v, &e);
        w.bf[j] = (v == 0.0) ? make_int2(0, kZeroExp) : make_int2(__float_as_int((float)m), e);
    }
}

cudaError_t launch_prep_windows(const WinPrep* list, int n, int max_wlen, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    int threads = 256;
    int bx = (max_wlen + threads - 1) / threads;
    if (bx > 64) bx = 64;
    k_prep_windows<<<dim3(bx, n), threads, 0, s>>>(list, n);
    return cudaGetLastError();
}

cudaError_t launch_split_windows(int2* dst, const double* wW, int wlen, cudaStream_t s)
{
    int threads = 256;
    int blocks = (wlen + threads - 1) / threads;
    if (blocks > 1024) blocks = 1024;
    k_split_windows<<<blocks, threads, 0, s>>>(dst, wW, wlen);
    return cudaGetLastError();
}

}  // namespace ps
