// ps_chosen.cu -- the chosen coupling kernel: FP32-pipe recurrences with
// two-word compensation, block-floating-point windows, FP64 anchors.
//
// Same work and mapping as the plain kernel (one warp = 32 consecutive l2 of one
// l1 row; families (l1 l2 l3; 0 0 0) and (l1 l2 l3; -2 2 0) in registers,
// contracted on the fly; see ps_plain_fp64.cu for the recurrence), with the
// arithmetic moved off the FP64 pipe:
//
//  * recurrence state and coefficients are float-float values (ps_ff.cuh):
//    P(j) is formed exactly from its four integer factors, 1/sqrt(P) by an
//    FP32 estimate plus one compensated Newton step, so each step carries
//    ~2^-46 relative error instead of FP32's 2^-24;
//  * the forward (from jmin) and backward (from jmax) sweeps run interleaved
//    in one loop: two independent dependency chains per lane;
//  * windows are stored as (mantissa, exponent) pairs.  Every 32 steps each
//    warp stages the slice of every window it is about to read into shared
//    memory, scaled by 2^-E with E the largest exponent of the slice, so FP32
//    keeps full relative precision whatever the windows' dynamic range
//    (mask spectra span > 1e-45 at l ~ 8000).  The 32-step FP32 partial sums
//    are added into FP64 totals with the factor 2^E;
//  * FP64 is kept where stability and range need it: the last forward point,
//    the least-squares match of the two sweeps, the normalisation, the sign and
//    the totals.
#include "ps_internal.cuh"
#include "ps_epilogue.cuh"
#include "ps_ff.cuh"

namespace ps {

constexpr int kChunk = 32;               // steps between window restaging / FP64 flushes
constexpr int kSlots = kChunk + 32;      // staged window entries per warp, direction and window

__device__ __forceinline__ double pow2d(int e)
{
    e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
    return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ float pow2f_or_zero(int d)  // 2^d for d <= 0, 0 below the normal range
{
    return d < -126 ? 0.0f : __int_as_float((d + 127) << 23);
}

// Stage window slots [base, base + kSlots) scaled by 2^-E into dst; returns E.
__device__ __forceinline__ int stage_slice(float* dst, const int2* __restrict__ bf, int base, int wlen, int lane)
{
    int2 v[2];
    int emax = kZeroExp;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int j = base + lane + 32 * q;
        v[q] = (j >= 0 && j < wlen) ? __ldg(bf + j) : make_int2(0, kZeroExp);
        emax = max(emax, v[q].y);
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
#pragma unroll
    for (int q = 0; q < 2; ++q) dst[lane + 32 * q] = __int_as_float(v[q].x) * pow2f_or_zero(v[q].y - emax);
    return emax;
}

// squares / products of float-float values rounded to FP32 with the low words folded in
__device__ __forceinline__ float sq_ff(ff g) { return __fmaf_rn(2.0f * g.h, g.l, __fmul_rn(g.h, g.h)); }
__device__ __forceinline__ float mul_ff(ff a, ff b)
{
    return __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, __fmul_rn(a.h, b.h)));
}

template <int NWIN, bool N00, bool N22>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_coupling_chosen(const CouplingParams p)
{
    __shared__ float sW[kWarpsPerBlock][2][NWIN][kSlots];
    const int warp = threadIdx.x >> 5;
    const int gw = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (gw >= p.ntasks) return;  // warp-uniform
    const int lane = threadIdx.x & 31;
    const int2 task = p.tasks[gw];
    const int l1 = task.x;
    const int l2raw = task.y + lane;
    const bool active = l2raw <= p.lmax;
    const int l2 = active ? l2raw : p.lmax;
    const int d = l2 - l1;
    const int jmin = d, jmax = l1 + l2;
    const int T = l1;
    const bool fam22 = N22 && (l1 >= 2);
    const int jmin0 = task.y - l1, jmax0 = task.y + l1;  // lane 0's ends: lane i reads slot i + step

    double Xi[kMaxWin];
    if (T == 0) {
        xi_single_term(p, l2, Xi);
        if (active) write_pair(p, l1, l2, Xi);
        return;
    }

    // forward state (j = jmin + t) and backward state (j = jmax - t)
    ff g2c = ff_make(1.0f), g2p = ff_make(0.0f), aj = ff_make(0.0f), g0 = ff_make(1.0f);
    ff h2c = ff_make(1.0f), h2n = ff_make(0.0f), an = ff_make(0.0f), h0 = ff_make(1.0f);
    float fA = 1.0f, fB = (float)(2 * d + 1), fC = (float)(2 * l1), fD = (float)(2 * l2 + 2);
    float bA = (float)(2 * l1), bB = (float)(2 * l2), bC = 1.0f, bD = (float)(2 * l1 + 2 * l2 + 1);
    float fw = (float)(2 * jmin + 1), bw = (float)(2 * jmax + 1);
    double FW[NWIN], BW[NWIN];
#pragma unroll
    for (int k = 0; k < NWIN; ++k) FW[k] = BW[k] = 0.0;
    double FN0 = 0.0, FN2 = 0.0, BN0 = 0.0, BN2 = 0.0;

    float* sF = &sW[warp][0][0][0];
    float* sB = &sW[warp][1][0][0];

    for (int t0 = 0; t0 < T; t0 += kChunk) {
        int eF[NWIN], eB[NWIN];
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin) {
                eF[k] = stage_slice(sF + k * kSlots, p.win[k].bf, jmin0 + t0, p.wlen, lane);
                eB[k] = stage_slice(sB + k * kSlots, p.win[k].bf, jmax0 - t0 - kChunk + 1, p.wlen, lane);
            } else {
                eF[k] = eB[k] = kZeroExp;
            }
        }
        __syncwarp();
        float cF[NWIN], cB[NWIN];
#pragma unroll
        for (int k = 0; k < NWIN; ++k) cF[k] = cB[k] = 0.0f;
        float n0F = 0.0f, n2F = 0.0f, n0B = 0.0f, n2B = 0.0f;
        const int steps = min(kChunk, T - t0);
        for (int s = 0; s < steps; ++s) {
            const bool even = ((t0 + s) & 1) == 0;  // parity of l1 + l2 + l3, both directions
            const int sf = lane + s, sb = lane - s + kChunk - 1;
            // ---- accumulate the current forward and backward points ----
            {
                float x22f = N22 ? sq_ff(g2c) : 0.0f;
                float x22b = N22 ? sq_ff(h2c) : 0.0f;
                if (N22) {
                    n2F = __fmaf_rn(fw, x22f, n2F);
                    n2B = __fmaf_rn(bw, x22b, n2B);
                }
                if (even) {
                    float x00f = N00 ? sq_ff(g0) : 0.0f, x00b = N00 ? sq_ff(h0) : 0.0f;
                    float x02f = (N00 && N22) ? mul_ff(g0, g2c) : 0.0f, x02b = (N00 && N22) ? mul_ff(h0, h2c) : 0.0f;
                    if (N00) {
                        n0F = __fmaf_rn(fw, x00f, n0F);
                        n0B = __fmaf_rn(bw, x00b, n0B);
                    }
#pragma unroll
                    for (int k = 0; k < NWIN; ++k) {
                        if (k < p.nwin && p.win[k].parity != PAR_ODD) {
                            const int pr = p.win[k].product;
                            float xf = pr == PROD_00_00 ? x00f : (pr == PROD_22_22 ? x22f : x02f);
                            float xb = pr == PROD_00_00 ? x00b : (pr == PROD_22_22 ? x22b : x02b);
                            cF[k] = __fmaf_rn(xf, sF[k * kSlots + sf], cF[k]);
                            cB[k] = __fmaf_rn(xb, sB[k * kSlots + sb], cB[k]);
                        }
                    }
                } else if (N22) {
#pragma unroll
                    for (int k = 0; k < NWIN; ++k) {
                        if (k < p.nwin && p.win[k].product == PROD_22_22 && p.win[k].parity != PAR_EVEN) {
                            cF[k] = __fmaf_rn(x22f, sF[k * kSlots + sf], cF[k]);
                            cB[k] = __fmaf_rn(x22b, sB[k * kSlots + sb], cB[k]);
                        }
                    }
                }
            }
            // ---- forward step: g(j+1) from g(j), g(j-1) ----
            {
                ff P = ff_mul_raw(two_prod(fA, fB), two_prod(fC, fD));  // P(j+1)
                ff r = ff_rsqrt(P);
                ff a1 = ff_mul(P, r);
                if (N22) {
                    ff g2n = ff_neg(ff_mul(ff_add(ff_mulf(g2c, 4.0f * fw), ff_mul(aj, g2p)), r));
                    g2p = g2c;
                    g2c = g2n;
                }
                if (N00 && !even) g0 = ff_neg(ff_mul(ff_mul(aj, r), g0));  // f00(j+1) = -a(j)/a(j+1) f00(j-1)
                aj = a1;
                fA += 1.0f; fB += 1.0f; fC -= 1.0f; fD += 1.0f;
                fw += 2.0f;
            }
            // ---- backward step: h(j-1) from h(j), h(j+1) ----
            {
                ff P = ff_mul_raw(two_prod(bA, bB), two_prod(bC, bD));  // P(j)
                ff r = ff_rsqrt(P);
                ff a0 = ff_mul(P, r);
                if (N22) {
                    ff h2m = ff_neg(ff_mul(ff_add(ff_mulf(h2c, 4.0f * bw), ff_mul(an, h2n)), r));
                    h2n = h2c;
                    h2c = h2m;
                }
                if (N00 && !even) h0 = ff_neg(ff_mul(ff_mul(an, r), h0));  // f00(j-1) = -a(j+1)/a(j) f00(j+1)
                an = a0;
                bA -= 1.0f; bB -= 1.0f; bC += 1.0f; bD -= 1.0f;
                bw -= 2.0f;
            }
        }
        // ---- FP64 flush of the chunk sums ----
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            FW[k] = fma((double)cF[k], pow2d(eF[k]), FW[k]);
            BW[k] = fma((double)cB[k], pow2d(eB[k]), BW[k]);
        }
        FN0 += (double)n0F;
        FN2 += (double)n2F;
        BN0 += (double)n0B;
        BN2 += (double)n2B;
        __syncwarp();
    }

    // last forward point t = T (j = jm), in FP64; its parity is that of T
    const int jm = jmin + T;
    const bool evenT = (T & 1) == 0;
    {
        double g2d = ff_to_double(g2c), g0d = (N00 && evenT) ? ff_to_double(g0) : 0.0;
        double x22 = g2d * g2d, x00 = g0d * g0d, x02 = g0d * g2d, w = 2.0 * jm + 1.0;
        if (N22) FN2 = fma(w, x22, FN2);
        if (N00) FN0 = fma(w, x00, FN0);
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin) {
                const int pr = p.win[k].product, pa = p.win[k].parity;
                double ww = __ldg(p.win[k].wW + jm);
                if (evenT && pa != PAR_ODD)
                    FW[k] = fma(pr == PROD_00_00 ? x00 : (pr == PROD_22_22 ? x22 : x02), ww, FW[k]);
                else if (!evenT && pr == PROD_22_22 && pa != PAR_EVEN)
                    FW[k] = fma(x22, ww, FW[k]);
            }
        }
    }
    // one more forward step for g(jm + 1)
    double gm0 = ff_to_double(g2c), gm1 = 0.0, g0s;
    {
        ff P = ff_mul_raw(two_prod(fA, fB), two_prod(fC, fD));
        ff r = ff_rsqrt(P);
        if (N22) gm1 = ff_to_double(ff_neg(ff_mul(ff_add(ff_mulf(g2c, 4.0f * fw), ff_mul(aj, g2p)), r)));
        g0s = (N00 && !evenT) ? ff_to_double(ff_neg(ff_mul(ff_mul(aj, r), g0))) : ff_to_double(g0);
    }
    const double hm0 = ff_to_double(h2c), hm1 = ff_to_double(h2n), h0s = ff_to_double(h0);

    // match, normalise, sign (FP64)
    const double lam0 = N00 ? g0s / h0s : 0.0;
    const double lam2 = fam22 ? (gm0 * hm0 + gm1 * hm1) / (hm0 * hm0 + hm1 * hm1) : 0.0;
    const double N0 = fma(lam0 * lam0, BN0, FN0);
    const double N2 = fma(lam2 * lam2, BN2, FN2);
    const double inv0 = N00 ? kInv4Pi / N0 : 0.0;
    const double inv2 = fam22 ? kInv4Pi / N2 : 0.0;
    double inv02 = 0.0;
    if (N00 && fam22) inv02 = (((lam0 < 0.0) != (lam2 < 0.0)) ? -kInv4Pi : kInv4Pi) * rsqrt(N0 * N2);
#pragma unroll
    for (int k = 0; k < kMaxWin; ++k) {
        Xi[k] = 0.0;
        if (k < NWIN && k < p.nwin) {
            const int pr = p.win[k].product;
            if (pr == PROD_00_00)
                Xi[k] = fma(lam0 * lam0, BW[k], FW[k]) * inv0;
            else if (!fam22)
                Xi[k] = 0.0;
            else if (pr == PROD_22_22)
                Xi[k] = fma(lam2 * lam2, BW[k], FW[k]) * inv2;
            else
                Xi[k] = fma(lam0 * lam2, BW[k], FW[k]) * inv02;
        }
    }
    if (active) write_pair(p, l1, l2, Xi);
}

template <int NWIN>
static cudaError_t launch_nwin(const CouplingParams& p, bool n00, bool n22, cudaStream_t s)
{
    const int threads = kWarpsPerBlock * 32;
    const unsigned blocks = (unsigned)((p.ntasks + kWarpsPerBlock - 1) / kWarpsPerBlock);
    if (n00 && n22)
        k_coupling_chosen<NWIN, true, true><<<blocks, threads, 0, s>>>(p);
    else if (n22)
        k_coupling_chosen<NWIN, false, true><<<blocks, threads, 0, s>>>(p);
    else
        k_coupling_chosen<NWIN, true, false><<<blocks, threads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_chosen(const CouplingParams& p, cudaStream_t s)
{
    bool n00 = false, n22 = false;
    for (int k = 0; k < p.nwin; ++k) {
        if (p.win[k].product != PROD_22_22) n00 = true;
        if (p.win[k].product != PROD_00_00) n22 = true;
    }
    if (p.ntasks <= 0) return cudaSuccess;
    if (p.nwin <= 1) return launch_nwin<1>(p, n00, n22, s);
    if (p.nwin <= 2) return launch_nwin<2>(p, n00, n22, s);
    if (p.nwin <= 4) return launch_nwin<4>(p, n00, n22, s);
    return launch_nwin<8>(p, n00, n22, s);
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

cudaError_t launch_split_windows(int2* dst, const double* wW, int wlen, cudaStream_t s)
{
    int threads = 256;
    int blocks = (wlen + threads - 1) / threads;
    if (blocks > 1024) blocks = 1024;
    k_split_windows<<<blocks, threads, 0, s>>>(dst, wW, wlen);
    return cudaGetLastError();
}

}  // namespace ps
