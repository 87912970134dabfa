// ps_quickpol_ff.cu -- the QuickPol Xi (quickpolXi!, src/beam.jl:72-109) in the
// chosen arithmetic: the general-spin recurrences on the FP32 pipe in
// float-float, FP64 only where the FP64 kernel (ps_quickpol.cu) needs range or
// one-off precision.
//
// Same mapping and algorithm as k_quickpol_fp64 (one thread per band element (l'', l),
// rows from the top; both
// families forward from their own jmin and backward from jmax, matched at one
// common point; here the two sweeps run interleaved in one loop), with:
//   * P(j) = A(j)^2 = (j-|d|)(j+|d|)(s-j)(s+j)(j-|m3|)(j+|m3|) formed from its
//     six exact integer factors (d = l1 - l2, s = l1 + l2 + 1): three exact
//     two_prod pairs and two float-float products;
//   * 1 / (j A(j+1)) = 1/sqrt(P(j+1) j^2) by ff_rsqrt, and A(j+1) carried to
//     the next step as P(j+1) times that, times j;
//   * B(j) = -(2j+1)(m3 d s - j(j+1)(m2 - m1)) in float-float from exact
//     pieces, and the factors both families share (all of P(j) but
//     (j - |m3|)(j + |m3|), and j(j+1)) formed once per point;
//   * W staged once per call as floats scaled by 2^-E (E: the largest
//     exponent of |W|), so FP32 keeps W's relative precision; entries below
//     2^(E-149) count as zero.  The FP32 sums are flushed into FP64 every 32
//     steps, and the result is scaled back by 2^E.
// The family values start at 1 and stay within FP32 range for the small spins
// QuickPol uses (|m| <= a few) at l up to 16383.
#include "ps_internal.cuh"
#include "ps_ff.cuh"

namespace ps {

namespace {

constexpr int kQpFlush = 32;  // steps between FP64 flushes of the FP32 sums

struct QFam {
    int m1, m2, m3, am3;
    float am3f;  // |m3| as a float
    int jmin;
    ff m3ds;     // m3 * d * s (d = l1 - l2, s = l1 + l2 + 1), exact in 64-bit integers, split into two floats
    float dm;    // m2 - m1
    bool zero;
};

// The parts of one step's coefficients that both families share: at point j,
// the factor (j^2 - d^2)(s^2 - j^2) of P(j), and j (j + 1).
struct QShared {
    ff ds;   // (j - |d|)(j + |d|)(s - j)(s + j)
    ff jj1;  // j (j + 1)
};

// j, |d| and s arrive as floats (exact integers below 2^24): the loops carry j
// as a float, so no integer-to-float conversion (which shares GB300's narrow
// FP64 pipe) runs per step.
__device__ __forceinline__ QShared qp_shared(float j, float ad, float s)
{
    QShared q;
    q.ds = ff_mul_raw(two_prod(j - ad, j + ad), two_prod(s - j, s + j));
    q.jj1 = two_prod(j, j + 1.0f);
    return q;
}

// P(j) = ds(j) (j - |m3|)(j + |m3|)
__device__ __forceinline__ ff qp_P(const QShared& q, float j, float am3)
{
    return ff_mul_raw(q.ds, two_prod(j - am3, j + am3));
}

// B(j) = -(2j+1) (m3 d s - j (j+1) (m2 - m1))
__device__ __forceinline__ ff qp_B(const QShared& q, float j, const QFam& f)
{
    const ff t = ff_add_raw(f.m3ds, ff_neg(ff_mulf_raw(q.jj1, f.dm)));
    return ff_neg(ff_mulf_raw(t, __fmaf_rn(2.0f, j, 1.0f)));
}

// f(j+1) from f(j), f(j-1) with the point-(j+1) shared parts qn and the
// point-j shared parts qc; `a` carries A(j) -> A(j+1).  j = 0 only occurs for
// m3 = 0, l1 = l2, where the recurrence is f(1) = -(m2 - m1) f(0) / A(1).
__device__ __forceinline__ ff qp_fwd(float j, const QFam& f, const QShared& qc, const QShared& qn, const ff& jsq, ff fc,
                                     ff fp, ff& a)
{
    const ff P1 = qp_P(qn, j + 1.0f, f.am3f);
    if (j == 0.0f) {
        const ff r = ff_rsqrt(P1);
        a = ff_mul_raw(P1, r);
        return ff_neg(ff_mulf_raw(ff_mul_raw(fc, r), f.dm));
    }
    const ff q = ff_rsqrt(ff_mul_raw(P1, jsq));  // 1 / (j A(j+1))
    const ff num = ff_add_raw(ff_mul_raw(qp_B(qc, j, f), fc), ff_mul_raw(ff_mulf_raw(a, j + 1.0f), fp));
    a = ff_mulf_raw(ff_mul_raw(P1, q), j);
    return ff_neg(ff_mul_raw(num, q));
}

// h(j-1) from h(j), h(j+1) (needs j > jmin) with the point-j shared parts qc;
// `a` carries A(j+1) -> A(j).  j1sq = (j+1)^2.
__device__ __forceinline__ ff qp_bwd(float j, const QFam& f, const QShared& qc, const ff& j1sq, ff hc, ff hn, ff& a)
{
    const ff P0 = qp_P(qc, j, f.am3f);
    const ff q = ff_rsqrt(ff_mul_raw(P0, j1sq));  // 1 / ((j+1) A(j))
    const ff num = ff_add_raw(ff_mul_raw(qp_B(qc, j, f), hc), ff_mul_raw(ff_mulf_raw(a, j), hn));
    a = ff_mulf_raw(ff_mul_raw(P0, q), j + 1.0f);
    return ff_neg(ff_mul_raw(num, q));
}

__device__ __forceinline__ float ff_round(ff x) { return __fadd_rn(x.h, x.l); }

// W -> floats scaled by 2^-E, E the largest exponent of |W| (0 when W is all zero).  One block.
__global__ void __launch_bounds__(1024) k_quickpol_stage(const double* __restrict__ W, int n, float* __restrict__ Wf,
                                                         int* __restrict__ E_out)
{
    __shared__ int warp_max[32];
    int e = -100000;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double w = W[j];
        if (w != 0.0) e = max(e, ilogb(w));
    }
    for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x < 32) {
        e = threadIdx.x < (blockDim.x >> 5) ? warp_max[threadIdx.x] : -100000;
        for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        if (threadIdx.x == 0) warp_max[0] = e == -100000 ? 0 : e;
    }
    __syncthreads();
    const int E = warp_max[0];
    for (int j = threadIdx.x; j < n; j += blockDim.x) Wf[j] = (float)ldexp(W[j], -E);
    if (threadIdx.x == 0) *E_out = E;
}

__global__ void __launch_bounds__(128, 5) k_quickpol_ff(const float* __restrict__ Wf, const int* __restrict__ E_in,
                                                     long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1,
                                                     int s2, double* Xi, long long ldx)
{
    // one thread per band element (l'', l), numbered row by row from the top
    // (the longest families first) so that every warp is full
    const int width = bl + bu + 1;
    const long long pidx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (pidx >= (long long)(lmax - 1) * width) return;
    const int lpp = lmax - (int)(pidx / width);  // row l''
    const int l = lpp - bl + (int)(pidx % width);
    if (l < 2 || l > lmax) return;
    const int l1 = l, l2 = lpp, jmax = l1 + l2;
    const int ad = abs(l1 - l2), s = l1 + l2 + 1;
    const float adf = (float)ad, spf = (float)s;  // |d| and s as floats
    QFam F[2];
    F[0].m1 = -s1; F[0].m2 = -nu1; F[0].m3 = s1 + nu1;
    F[1].m1 = -s2; F[1].m2 = -nu2; F[1].m3 = s2 + nu2;
    bool any_zero = false;
    int jm = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        F[k].am3 = abs(F[k].m3);
        F[k].am3f = (float)F[k].am3;
        const long long m3ds = (long long)F[k].m3 * (l1 - l2) * s;  // |m3 d s| < 2^38
        const float h = (float)m3ds;
        F[k].m3ds = ff{h, (float)(m3ds - (long long)h)};
        F[k].dm = (float)(F[k].m2 - F[k].m1);
        F[k].jmin = max(ad, F[k].am3);
        F[k].zero = abs(F[k].m1) > l1 || abs(F[k].m2) > l2 || F[k].jmin > jmax;
        any_zero |= F[k].zero;
        jm = max(jm, (F[k].jmin + jmax) / 2);
    }
    double xi = 0.0;
    if (!any_zero) {
        if (jm >= jmax) jm = jmax - 1;
        const bool fwd0 = F[0].jmin <= jm, fwd1 = F[1].jmin <= jm;
        const ff zero = ff_make(0.0f), one = ff_make(1.0f);
        // The forward sweep (each family from its own jmin up to jm; values at
        // jm + 1 kept) and the backward sweep (from jmax down to jm + 1, and to
        // jmin for backward-only families) run interleaved in one loop: four
        // independent dependency chains per thread.
        ff fp0 = zero, fc0 = zero, fp1 = zero, fc1 = zero, af0 = zero, af1 = zero;
        ff hn0 = zero, hc0 = one, hn1 = zero, hc1 = one, ab0 = zero, ab1 = zero;
        ff hm0_0 = zero, hm1_0 = zero, hm0_1 = zero, hm1_1 = zero;  // h(jm), h(jm+1) per family
        double NF0 = 0.0, NF1 = 0.0, SF = 0.0, NB0 = 0.0, NB1 = 0.0, SB = 0.0;
        float nf0 = 0.0f, nf1 = 0.0f, sf = 0.0f, nb0 = 0.0f, nb1 = 0.0f, sb = 0.0f;
        const int jlo = min(fwd0 ? F[0].jmin : jm + 1, fwd1 ? F[1].jmin : jm + 1);
        const int jstop = min(fwd0 ? jm + 1 : F[0].jmin, fwd1 ? jm + 1 : F[1].jmin);
        const int nfwd = jm - jlo + 1, nbwd = jmax - jstop + 1, nit = max(nfwd, nbwd);
        QShared qc = qp_shared((float)jlo, adf, spf);  // forward: the next point's parts become the current ones
        float jf = (float)jlo, jbf = (float)jmax;      // the two sweeps' points as floats
        int cnt = 0;
        for (int it = 0; it < nit; ++it, jf += 1.0f, jbf -= 1.0f) {
            if (it < nfwd) {
                const int j = jlo + it;
                if (fwd0 && j == F[0].jmin) fc0 = one;
                if (fwd1 && j == F[1].jmin) fc1 = one;
                const float g0 = ff_round(fc0), g1 = ff_round(fc1), w = __fmaf_rn(2.0f, jf, 1.0f);
                nf0 = __fmaf_rn(w, __fmul_rn(g0, g0), nf0);
                nf1 = __fmaf_rn(w, __fmul_rn(g1, g1), nf1);
                if (j < nW) sf = __fmaf_rn(__fmul_rn(__ldg(Wf + j), g0), g1, sf);
                const QShared qn = qp_shared(jf + 1.0f, adf, spf);
                const ff jsq = two_prod(jf, jf);
                if (fwd0 && j >= F[0].jmin) {
                    const ff n = qp_fwd(jf, F[0], qc, qn, jsq, fc0, fp0, af0);
                    fp0 = fc0;
                    fc0 = n;
                }
                if (fwd1 && j >= F[1].jmin) {
                    const ff n = qp_fwd(jf, F[1], qc, qn, jsq, fc1, fp1, af1);
                    fp1 = fc1;
                    fc1 = n;
                }
                qc = qn;
            }
            if (it < nbwd) {
                const int j = jmax - it;
                const bool in0 = j >= (fwd0 ? jm + 1 : F[0].jmin), in1 = j >= (fwd1 ? jm + 1 : F[1].jmin);
                const float v0 = in0 ? ff_round(hc0) : 0.0f, v1 = in1 ? ff_round(hc1) : 0.0f;
                const float w = __fmaf_rn(2.0f, jbf, 1.0f);
                nb0 = __fmaf_rn(w, __fmul_rn(v0, v0), nb0);
                nb1 = __fmaf_rn(w, __fmul_rn(v1, v1), nb1);
                if (j < nW) sb = __fmaf_rn(__fmul_rn(__ldg(Wf + j), v0), v1, sb);
                const QShared qb = qp_shared(jbf, adf, spf);
                const ff j1sq = two_prod(jbf + 1.0f, jbf + 1.0f);
                if (in0 && j > F[0].jmin) {
                    if (j == jm + 1) hm1_0 = hc0;
                    const ff n = qp_bwd(jbf, F[0], qb, j1sq, hc0, hn0, ab0);
                    hn0 = hc0;
                    hc0 = n;
                    if (j == jm + 1) hm0_0 = hc0;
                }
                if (in1 && j > F[1].jmin) {
                    if (j == jm + 1) hm1_1 = hc1;
                    const ff n = qp_bwd(jbf, F[1], qb, j1sq, hc1, hn1, ab1);
                    hn1 = hc1;
                    hc1 = n;
                    if (j == jm + 1) hm0_1 = hc1;
                }
            }
            if (++cnt == kQpFlush) {
                NF0 += nf0; NF1 += nf1; SF += sf; NB0 += nb0; NB1 += nb1; SB += sb;
                nf0 = nf1 = sf = nb0 = nb1 = sb = 0.0f;
                cnt = 0;
            }
        }
        NF0 += nf0; NF1 += nf1; SF += sf; NB0 += nb0; NB1 += nb1; SB += sb;
        // ---- match, normalise, sign (FP64) ----
        const double p0 = ff_to_double(fp0), c0 = ff_to_double(fc0), p1 = ff_to_double(fp1), c1 = ff_to_double(fc1);
        const double a0 = ff_to_double(hm0_0), b0 = ff_to_double(hm1_0), a1 = ff_to_double(hm0_1),
                     b1 = ff_to_double(hm1_1);
        const double lam0 = fwd0 ? (p0 * a0 + c0 * b0) / (a0 * a0 + b0 * b0) : 1.0;
        const double lam1 = fwd1 ? (p1 * a1 + c1 * b1) / (a1 * a1 + b1 * b1) : 1.0;
        const double N0 = fma(lam0 * lam0, NB0, NF0), N1 = fma(lam1 * lam1, NB1, NF1);
        const double cs0 = ((l1 - l2 - F[0].m3) & 1) ? -1.0 : 1.0, cs1 = ((l1 - l2 - F[1].m3) & 1) ? -1.0 : 1.0;
        const double sg0 = (lam0 < 0.0) ? -cs0 : cs0, sg1 = (lam1 < 0.0) ? -cs1 : cs1;
        xi = ldexp(fma(lam0 * lam1, SB, SF) * sg0 * sg1 * rsqrt(N0 * N1), *E_in);
    }
    const double sgn = ((s1 + s2 + nu1 + nu2) & 1) ? -1.0 : 1.0;
    Xi[(long long)lpp + (long long)l * ldx] = sgn * xi;
}

}  // namespace

cudaError_t launch_quickpol_ff(const double* W, long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1,
                               int s2, double* Xi, long long ldx, float* wf, int* e, cudaStream_t st)
{
    if (lmax < 2) return cudaSuccess;
    k_quickpol_stage<<<1, 1024, 0, st>>>(W, (int)nW, wf, e);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    // a band wider than the grid covers the same elements as one of width lmax
    bl = bl < lmax ? bl : lmax;
    bu = bu < lmax ? bu : lmax;
    const int width = bl + bu + 1;
    const long long total = (long long)(lmax - 1) * width;  // < 2^31 for lmax <= 16383
    k_quickpol_ff<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(wf, e, nW, lmax, bl, bu, nu1, nu2, s1, s2, Xi, ldx);
    return cudaGetLastError();
}

}  // namespace ps
