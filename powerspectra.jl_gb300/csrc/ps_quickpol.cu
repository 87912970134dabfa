// ps_quickpol.cu -- the QuickPol beam-coupling matrix Xi on the GPU (FP64).
//
// Replaces the loop of quickpolXi! (src/beam.jl:72-109): for l'' = 2..lmax and
// l in the band [l'' - bl, l'' + bu] (l >= 2),
//     Xi[l'', l] = (-1)^(s1+s2+nu1+nu2) sum_l' W[l'] f1(l') f2(l'),
//     f_k(l') = (l' l l''; s_k+nu_k, -s_k, -nu_k) = (l l'' l'; -s_k, -nu_k, s_k+nu_k),
// summed over the common support of the two families (Xisum, src/beam.jl:17-28).
//
// One thread per (l'', l).  Both families follow the general Schulten-Gordon
// recurrence in l' (arbitrary m, so B(j) != 0 and A(j) carries the m3 factor),
// run forward from each family's own jmin and backward from the common jmax,
// and are matched at one common point jm (the larger of the two families'
// midpoints), so the product sum splits into a forward part and a backward part
// with scale lambda1 * lambda2.  Nothing is stored; the families stay in
// registers.  Spins are small in practice (|m| <= a few), where both families
// are classically allowed around their midpoints.
#include "ps_internal.cuh"

namespace ps {

namespace {

struct Fam {
    int m1, m2, m3;
    int jmin;
    bool zero;  // identically zero (|m| > l or empty support)
};

// P(j) = A(j)^2 = (j^2 - (l1-l2)^2) ((l1+l2+1)^2 - j^2) (j^2 - m3^2), clamped at 0
__device__ __forceinline__ double sgP(int j, int l1, int l2, int m3)
{
    double jj = (double)j * j, dd = (double)(l1 - l2) * (l1 - l2), ss = (double)(l1 + l2 + 1) * (l1 + l2 + 1);
    double p = (jj - dd) * (ss - jj) * (jj - (double)m3 * m3);
    return p > 0.0 ? p : 0.0;
}

__device__ __forceinline__ double sgB(int j, int l1, int l2, const Fam& f)
{
    double t = (double)l1 * (l1 + 1) * f.m3 - (double)l2 * (l2 + 1) * f.m3 - (double)j * (j + 1) * (double)(f.m2 - f.m1);
    return -(2.0 * j + 1.0) * t;
}

// Forward step j -> j + 1 with A(j) carried in `a`: returns f(j+1) and
// replaces `a` by A(j+1), so each step takes one square root and one division
// (a correctly rounded sqrt and quotient: the rounding of the plain formula).
// j = 0 only occurs for m3 = 0, l1 = l2, where the recurrence has no f(j-1) term.
__device__ __forceinline__ double fwd_next(int j, int l1, int l2, const Fam& f, double fc, double fp, double& a)
{
    const double a1 = sqrt(sgP(j + 1, l1, l2, f.m3));
    const double num = j == 0 ? (double)(f.m2 - f.m1) * fc : fma(sgB(j, l1, l2, f), fc, (j + 1.0) * a * fp);
    a = a1;
    return -num / (j == 0 ? a1 : (double)j * a1);
}

// Backward step j -> j - 1 with A(j+1) carried in `a` (needs j > jmin):
// returns h(j-1) and replaces `a` by A(j).
__device__ __forceinline__ double bwd_next(int j, int l1, int l2, const Fam& f, double hc, double hn, double& a)
{
    const double a0 = sqrt(sgP(j, l1, l2, f.m3));
    const double num = fma(sgB(j, l1, l2, f), hc, (double)j * a * hn);
    a = a0;
    return -num / ((j + 1.0) * a0);
}

__global__ void __launch_bounds__(128) k_quickpol_fp64(const double* __restrict__ W, long long nW, int lmax, int bl,
                                                       int bu, int nu1, int nu2, int s1, int s2, double* Xi,
                                                       long long ldx)
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
    Fam F[2];
    F[0].m1 = -s1; F[0].m2 = -nu1; F[0].m3 = s1 + nu1;
    F[1].m1 = -s2; F[1].m2 = -nu2; F[1].m3 = s2 + nu2;
    bool any_zero = false;
    int jm = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        F[k].jmin = max(abs(l1 - l2), abs(F[k].m3));
        F[k].zero = abs(F[k].m1) > l1 || abs(F[k].m2) > l2 || F[k].jmin > jmax;
        any_zero |= F[k].zero;
        jm = max(jm, (F[k].jmin + jmax) / 2);
    }
    double xi = 0.0;
    if (!any_zero) {
        if (jm >= jmax) jm = jmax - 1;
        const bool fwd0 = F[0].jmin <= jm, fwd1 = F[1].jmin <= jm;
        // ---- forward: each family from its own jmin up to jm (values at jm + 1 kept) ----
        double fp0 = 0.0, fc0 = 0.0, fp1 = 0.0, fc1 = 0.0, NF0 = 0.0, NF1 = 0.0, SF = 0.0;
        double af0 = 0.0, af1 = 0.0;  // A(j) of each family at the current point
        const int jlo = min(fwd0 ? F[0].jmin : jm + 1, fwd1 ? F[1].jmin : jm + 1);
        for (int j = jlo; j <= jm; ++j) {
            if (fwd0 && j == F[0].jmin) fc0 = 1.0;
            if (fwd1 && j == F[1].jmin) fc1 = 1.0;
            const double w = 2.0 * j + 1.0;
            NF0 = fma(w, fc0 * fc0, NF0);
            NF1 = fma(w, fc1 * fc1, NF1);
            if (j < nW) SF = fma(__ldg(W + j) * fc0, fc1, SF);
            if (fwd0 && j >= F[0].jmin) {
                double n = fwd_next(j, l1, l2, F[0], fc0, fp0, af0);
                fp0 = fc0;
                fc0 = n;
            }
            if (fwd1 && j >= F[1].jmin) {
                double n = fwd_next(j, l1, l2, F[1], fc1, fp1, af1);
                fp1 = fc1;
                fc1 = n;
            }
        }
        // now fp_k = f_k(jm), fc_k = f_k(jm + 1) for forward families
        // ---- backward: from jmax down to jm + 1 (and to jmin for backward-only families) ----
        double hn0 = 0.0, hc0 = 1.0, hn1 = 0.0, hc1 = 1.0, NB0 = 0.0, NB1 = 0.0, SB = 0.0;
        double hm0_0 = 0.0, hm1_0 = 0.0, hm0_1 = 0.0, hm1_1 = 0.0;  // h(jm), h(jm+1) per family
        double ab0 = 0.0, ab1 = 0.0;  // A(j+1) of each family (A(jmax+1) = 0: no h(jmax+1) term)
        const int jstop = min(fwd0 ? jm + 1 : F[0].jmin, fwd1 ? jm + 1 : F[1].jmin);
        for (int j = jmax; j >= jstop; --j) {
            const bool in0 = j >= (fwd0 ? jm + 1 : F[0].jmin), in1 = j >= (fwd1 ? jm + 1 : F[1].jmin);
            const double v0 = in0 ? hc0 : 0.0, v1 = in1 ? hc1 : 0.0;
            const double w = 2.0 * j + 1.0;
            NB0 = fma(w, v0 * v0, NB0);
            NB1 = fma(w, v1 * v1, NB1);
            if (j < nW) SB = fma(__ldg(W + j) * v0, v1, SB);
            if (in0 && j > F[0].jmin) {
                if (j == jm + 1) hm1_0 = hc0;
                double n = bwd_next(j, l1, l2, F[0], hc0, hn0, ab0);
                hn0 = hc0;
                hc0 = n;
                if (j == jm + 1) hm0_0 = hc0;
            }
            if (in1 && j > F[1].jmin) {
                if (j == jm + 1) hm1_1 = hc1;
                double n = bwd_next(j, l1, l2, F[1], hc1, hn1, ab1);
                hn1 = hc1;
                hc1 = n;
                if (j == jm + 1) hm0_1 = hc1;
            }
        }
        // ---- match, normalise, sign ----
        const double lam0 = fwd0 ? (fp0 * hm0_0 + fc0 * hm1_0) / (hm0_0 * hm0_0 + hm1_0 * hm1_0) : 1.0;
        const double lam1 = fwd1 ? (fp1 * hm0_1 + fc1 * hm1_1) / (hm0_1 * hm0_1 + hm1_1 * hm1_1) : 1.0;
        const double N0 = fma(lam0 * lam0, NB0, NF0), N1 = fma(lam1 * lam1, NB1, NF1);
        // Condon-Shortley: sgn f(jmax) = (-1)^(l1 - l2 - m3); the matched family has f(jmax) = lambda
        const double cs0 = ((l1 - l2 - F[0].m3) & 1) ? -1.0 : 1.0, cs1 = ((l1 - l2 - F[1].m3) & 1) ? -1.0 : 1.0;
        const double sg0 = (lam0 < 0.0) ? -cs0 : cs0, sg1 = (lam1 < 0.0) ? -cs1 : cs1;
        xi = fma(lam0 * lam1, SB, SF) * sg0 * sg1 * rsqrt(N0 * N1);
    }
    const double sgn = ((s1 + s2 + nu1 + nu2) & 1) ? -1.0 : 1.0;
    Xi[(long long)lpp + (long long)l * ldx] = sgn * xi;
}

}  // namespace

cudaError_t launch_quickpol(const double* W, long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1, int s2,
                            double* Xi, long long ldx, cudaStream_t s)
{
    if (lmax < 2) return cudaSuccess;
    // a band wider than the grid covers the same elements as one of width lmax
    bl = bl < lmax ? bl : lmax;
    bu = bu < lmax ? bu : lmax;
    const int width = bl + bu + 1;
    const long long total = (long long)(lmax - 1) * width;  // < 2^31 for lmax <= 16383
    k_quickpol_fp64<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(W, nW, lmax, bl, bu, nu1, nu2, s1, s2, Xi, ldx);
    return cudaGetLastError();
}

}  // namespace ps
