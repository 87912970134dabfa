/*
 * oracle.c -- CPU FP64 restatement of PowerSpectra.jl's Wigner-3j mode-coupling
 * and covariance hot loops.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library: it
 * is called from tests/, from __graft_entry__.smoke() and from bench.py's
 * cpu_baseline / reference leg, never from the product path.  It follows the
 * reference algorithm on purpose: for every (l1 <= l2) pair it fills a whole
 * 3j family into a per-thread buffer and then streams a dot product over it,
 * with OpenMP dynamic scheduling over l1 rows (the reference uses @qthreads).
 *
 * Reference files (paths inside the PowerSpectra.jl project):
 *   src/modecoupling.jl:3-66    Xi_TT / Xi_EE / Xi_EB / Xi_TE projectors
 *   src/modecoupling.jl:69-75   fill_3j!  (WignerFamilies.jl family fill)
 *   src/modecoupling.jl:78-159  inner_mcm00! / 02! / ++! / --!
 *   src/covariance.jl:92-446    loop_covTTTT! ... loop_covTTEE!
 *
 * The 3j family itself comes, in the reference, from the un-vendored package
 * WignerFamilies.jl (Project.toml:25, compat "1", no Manifest pins a version).
 * Its published algorithm is restated here from the literature:
 *   K. Schulten and R. G. Gordon, J. Math. Phys. 16, 1961 (1975): the
 *     three-term recurrence in j for (j l1 l2 ; -m1-m2 m1 m2);
 *   S. Luscombe and M. Luban, Phys. Rev. E 57, 7274 (1998): forward recursion
 *     from jmin and backward recursion from jmax, matched in the classical
 *     region, normalised by sum_j (2j+1) f(j)^2 = 1, sign fixed at jmax by the
 *     Condon-Shortley convention sgn f(jmax) = (-1)^(l1-l2-m3).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* A(j) of the Schulten-Gordon recurrence for the family f(j) = (l1 l2 j; m1 m2 m3). */
static inline double sg_A(int j, int l1, int l2, int m3)
{
    double jj = (double)j * (double)j;
    double dd = (double)(l1 - l2) * (double)(l1 - l2);
    double ss = (double)(l1 + l2 + 1) * (double)(l1 + l2 + 1);
    double mm = (double)m3 * (double)m3;
    double p = (jj - dd) * (ss - jj) * (jj - mm);
    return p > 0.0 ? sqrt(p) : 0.0;
}

/* B(j) = -(2j+1) [ l1(l1+1) m3 - l2(l2+1) m3 - j(j+1)(m2 - m1) ] */
static inline double sg_B(int j, int l1, int l2, int m1, int m2, int m3)
{
    double t = (double)l1 * (l1 + 1) * m3 - (double)l2 * (l2 + 1) * m3 - (double)j * (j + 1) * (double)(m2 - m1);
    return -(2.0 * j + 1.0) * t;
}

/* The family with the forward and backward sweeps matched at (jm_req, jm_req + 1)
 * instead of the family's own midpoint (jm_req < 0).  A match point past
 * jmax - 1 is clamped to jmax - 1; one before jmin leaves no forward part, and
 * the family is then the backward sweep alone, from jmax down to jmin. */
static int w3j_family_at(int l1, int l2, int m1, int m2, int jm_req, double *out, int *jmin_out);

int or_w3j_family(int l1, int l2, int m1, int m2, double *out, int *jmin_out)
{
    return w3j_family_at(l1, l2, m1, m2, -1, out, jmin_out);
}

static int w3j_family_at(int l1, int l2, int m1, int m2, int jm_req, double *out, int *jmin_out)
{
    int m3 = -m1 - m2;
    int jmin = abs(l1 - l2);
    if (abs(m3) > jmin) jmin = abs(m3);
    int jmax = l1 + l2;
    if (jmin_out) *jmin_out = jmin;
    if (l1 < 0 || l2 < 0 || jmax < jmin) return 0;
    int n = jmax - jmin + 1;
    memset(out, 0, sizeof(double) * (size_t)n);
    if (abs(m1) > l1 || abs(m2) > l2) return n; /* identically zero family */

    int jm = jm_req < 0 ? jmin + (n - 1) / 2 : jm_req; /* match at jm and jm+1 */
    if (jm > jmax - 1) jm = jmax - 1;
    if (n == 1) {
        out[0] = 1.0;
    } else if (jm < jmin) {
        /* backward only: h(jmax) = 1 down to h(jmin) */
        double h_next = 0.0, h_cur = 1.0;
        out[n - 1] = 1.0;
        for (int j = jmax; j > jmin; --j) {
            double prv = -(sg_B(j, l1, l2, m1, m2, m3) * h_cur + (double)j * sg_A(j + 1, l1, l2, m3) * h_next) /
                         ((j + 1.0) * sg_A(j, l1, l2, m3));
            out[j - 1 - jmin] = prv;
            h_next = h_cur;
            h_cur = prv;
        }
    } else {
        /* forward: g(jmin) = 1, produce g up to jm+1 */
        out[0] = 1.0;
        for (int j = jmin; j <= jm; ++j) {
            double fj = out[j - jmin];
            double fjm1 = (j - 1 >= jmin) ? out[j - 1 - jmin] : 0.0;
            double nxt;
            if (j == 0) {
                /* only reached for m3 = 0, l1 = l2: the recurrence divided by j(j+1) */
                nxt = -((double)(m2 - m1) * fj) / sg_A(1, l1, l2, m3);
            } else {
                nxt = -(sg_B(j, l1, l2, m1, m2, m3) * fj + (j + 1.0) * sg_A(j, l1, l2, m3) * fjm1) /
                      ((double)j * sg_A(j + 1, l1, l2, m3));
            }
            out[j + 1 - jmin] = nxt;
        }
        double g0 = out[jm - jmin], g1 = out[jm + 1 - jmin];
        /* backward: h(jmax) = 1, produce h down to jm (stored in a scratch walk) */
        double h_next = 0.0, h_cur = 1.0; /* h(j+1), h(j) with j = jmax */
        double h_jm1 = 0.0;               /* h(jm+1) once reached */
        out[n - 1] = 1.0;
        for (int j = jmax; j >= jm + 1; --j) {
            double prv = -(sg_B(j, l1, l2, m1, m2, m3) * h_cur + (double)j * sg_A(j + 1, l1, l2, m3) * h_next) /
                         ((j + 1.0) * sg_A(j, l1, l2, m3));
            if (j == jm + 1) h_jm1 = h_cur;
            h_next = h_cur;
            h_cur = prv;
            if (j - 1 >= jm + 1) out[j - 1 - jmin] = prv;
        }
        double h0 = h_cur; /* h(jm) */
        double lam = (g0 * h0 + g1 * h_jm1) / (h0 * h0 + h_jm1 * h_jm1);
        for (int j = jm + 1; j <= jmax; ++j) out[j - jmin] *= lam;
    }
    double norm = 0.0;
    for (int k = 0; k < n; ++k) norm += (2.0 * (jmin + k) + 1.0) * out[k] * out[k];
    double sc = 1.0 / sqrt(norm);
    int want_neg = ((l1 - l2 - m3) % 2 != 0);
    int is_neg = out[n - 1] < 0.0;
    if (want_neg != is_neg) sc = -sc;
    for (int k = 0; k < n; ++k) out[k] *= sc;
    return n;
}

/* Xi projectors, src/modecoupling.jl:3-66.  parity: 0 all l3 (Xi_TT), 1 even
 * l1+l2+l3 (Xi_EE, Xi_TE), 2 odd l1+l2+l3 (Xi_EB).  x holds the family product
 * over [jmin, jmax]; W is 0-indexed with length nW. */
static double xi_sum(const double *W, long nW, const double *x, int jmin, int jmax, int l1, int l2, int parity,
                     int absmode)
{
    long js = jmin > 0 ? jmin : 0;
    long je = (long)jmax < nW - 1 ? (long)jmax : nW - 1;
    if (parity == 1 && ((l1 + l2 + js) & 1)) js++;
    if (parity == 2 && !((l1 + l2 + js) & 1)) js++;
    long step = parity ? 2 : 1;
    double s = 0.0;
    if (absmode)
        for (long j = js; j <= je; j += step) s += (2.0 * j + 1.0) * fabs(x[j - jmin]) * fabs(W[j]);
    else
        for (long j = js; j <= je; j += step) s += (2.0 * j + 1.0) * x[j - jmin] * W[j];
    return s / (4.0 * M_PI);
}

static int nthreads_or_default(int nt)
{
#ifdef _OPENMP
    return nt > 0 ? nt : omp_get_max_threads();
#else
    (void)nt;
    return 1;
#endif
}

int or_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Row list helper: rows == NULL means every l1 in [lmin, lmax]. */
static inline int row_at(const int *rows, int i, int lmin) { return rows ? rows[i] : lmin + i; }

static int inner_mcm_impl(int spin, const double *W, long nW, int lmin, int lmax, double *M, long ldm,
                          const int *rows, int nrows, int nthreads, int absmode)
{
    if (spin < 0 || spin > 3 || lmin < 0 || lmax < lmin || nW < 1 || ldm < lmax - lmin + 1) return 1;
    int nr = rows ? nrows : lmax - lmin + 1;
    int nt = nthreads_or_default(nthreads);
    int blen = 2 * lmax + 1;
    int err = 0;
#pragma omp parallel num_threads(nt)
    {
        double *b0 = (double *)malloc(sizeof(double) * (size_t)blen);
        double *b2 = (double *)malloc(sizeof(double) * (size_t)blen);
        if (!b0 || !b2) {
#pragma omp atomic write
            err = 2;
        }
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < nr; ++i) {
            if (!b0 || !b2) continue;
            int l1 = row_at(rows, i, lmin);
            for (int l2 = l1; l2 <= lmax; ++l2) {
                int jmin, jmax = l1 + l2;
                double xi;
                if (spin == 0) { /* inner_mcm00!, src/modecoupling.jl:78-95 */
                    int n = or_w3j_family(l1, l2, 0, 0, b0, &jmin);
                    for (int k = 0; k < n; ++k) b0[k] = b0[k] * b0[k];
                    xi = xi_sum(W, nW, b0, jmin, jmax, l1, l2, 0, absmode);
                } else if (spin == 1) { /* inner_mcm02!, src/modecoupling.jl:99-119 */
                    int n = or_w3j_family(l1, l2, 0, 0, b0, &jmin);
                    int jmin2;
                    or_w3j_family(l1, l2, -2, 2, b2, &jmin2);
                    for (int k = 0; k < n; ++k) b0[k] *= b2[k];
                    xi = xi_sum(W, nW, b0, jmin, jmax, l1, l2, 1, absmode);
                } else { /* inner_mcm++! / --!, src/modecoupling.jl:123-159 */
                    int n = or_w3j_family(l1, l2, -2, 2, b2, &jmin);
                    for (int k = 0; k < n; ++k) b2[k] = b2[k] * b2[k];
                    xi = xi_sum(W, nW, b2, jmin, jmax, l1, l2, spin == 2 ? 1 : 2, absmode);
                }
                M[(long)(l1 - lmin) + (long)(l2 - lmin) * ldm] = (2.0 * l2 + 1.0) * xi;
                M[(long)(l2 - lmin) + (long)(l1 - lmin) * ldm] = (2.0 * l1 + 1.0) * xi;
            }
        }
        free(b0);
        free(b2);
    }
    return err;
}

int or_inner_mcm(int spin, const double *W, long nW, int lmin, int lmax, double *M, long ldm,
                 const int *rows, int nrows, int nthreads)
{
    return inner_mcm_impl(spin, W, nW, lmin, lmax, M, ldm, rows, nrows, nthreads, 0);
}

int or_inner_mcm_abs(int spin, const double *W, long nW, int lmin, int lmax, double *M, long ldm,
                     const int *rows, int nrows, int nthreads)
{
    return inner_mcm_impl(spin, W, nW, lmin, lmax, M, ldm, rows, nrows, nthreads, 1);
}

int or_xi(int product, int parity, const double *W, long nW, int lmin, int lmax, double *X, long ldx, int nthreads)
{
    if (product < 0 || product > 2 || parity < 0 || parity > 2 || lmin < 0 || lmax < lmin || ldx < lmax - lmin + 1)
        return 1;
    int nt = nthreads_or_default(nthreads);
    int blen = 2 * lmax + 1;
    int err = 0;
#pragma omp parallel num_threads(nt)
    {
        double *b0 = (double *)malloc(sizeof(double) * (size_t)blen);
        double *b2 = (double *)malloc(sizeof(double) * (size_t)blen);
        if (!b0 || !b2) {
#pragma omp atomic write
            err = 2;
        }
#pragma omp for schedule(dynamic, 1)
        for (int l1 = lmin; l1 <= lmax; ++l1) {
            if (!b0 || !b2) continue;
            for (int l2 = l1; l2 <= lmax; ++l2) {
                int jmin, jmin2, n;
                if (product == 0) {
                    n = or_w3j_family(l1, l2, 0, 0, b0, &jmin);
                    for (int k = 0; k < n; ++k) b0[k] *= b0[k];
                } else if (product == 1) {
                    n = or_w3j_family(l1, l2, -2, 2, b0, &jmin);
                    for (int k = 0; k < n; ++k) b0[k] *= b0[k];
                } else {
                    n = or_w3j_family(l1, l2, 0, 0, b0, &jmin);
                    or_w3j_family(l1, l2, -2, 2, b2, &jmin2);
                    for (int k = 0; k < n; ++k) b0[k] *= b2[k];
                }
                double xi = xi_sum(W, nW, b0, jmin, l1 + l2, l1, l2, parity, 0);
                X[(long)(l1 - lmin) + (long)(l2 - lmin) * ldx] = xi;
                X[(long)(l2 - lmin) + (long)(l1 - lmin) * ldx] = xi;
            }
        }
        free(b0);
        free(b2);
    }
    return err;
}

/* Number of windows each covariance kind consumes (the W1..Wk arguments). */
int or_cov_nwindows(int kind)
{
    static const int nw[7] = {8, 8, 4, 5, 4, 4, 2};
    return (kind >= 0 && kind < 7) ? nw[kind] : -1;
}

/* loop_cov*! kernels, src/covariance.jl:92-446.  Argument order follows the
 * reference's loop_cov*! signatures:
 *   TTTT  S={TTip,TTjq,TTiq,TTjp} R={r_ip,r_jq,r_iq,r_jp} W1..W8  (00^2, Xi_TT)
 *   EEEE  S={EEip,EEjq,EEiq,EEjp} R={r_ip,r_jq,r_iq,r_jp} W1..W8  (22^2, Xi_EE)
 *   TTTE  S={TTip,TTjp,TEiq,TEjq} R={r_ip,r_jp}           W1..W4  (00^2, Xi_TT)
 *   TETE  S={TTip,EEjq,TEiq,TEjp} R={r_TT_ip,r_PP_jq}     W1..W5  (00x22 Xi_TE; W2: 00^2 Xi_TT)
 *   TEEE  S={EEjq,EEjp,TEip,TEiq} R={r_EE_jq,r_EE_jp}     W1..W4  (00x22, Xi_EE)
 *   TEEE_PLANCK  same arguments                             W1..W4  (22^2, Xi_EE)
 *   TTEE  S={TEip,TEiq,TEjq,TEjp} R={}                    W1..W2  (00^2, Xi_TT)  */

static int loop_cov_impl(int kind, const double *const *S, const double *const *R, const double *const *Wk, long nW,
                         int lmin, int lmax, double *C, long ldc, const int *rows, int nrows, int nthreads, int absmode)
{
    int K = or_cov_nwindows(kind);
    if (K < 0 || lmin < 0 || lmax < lmin || ldc < lmax - lmin + 1) return 1;
    int nr = rows ? nrows : lmax - lmin + 1;
    int nt = nthreads_or_default(nthreads);
    int blen = 2 * lmax + 1;
    int err = 0;
#pragma omp parallel num_threads(nt)
    {
        double *b0 = (double *)malloc(sizeof(double) * (size_t)blen);
        double *b2 = (double *)malloc(sizeof(double) * (size_t)blen);
        if (!b0 || !b2) {
#pragma omp atomic write
            err = 2;
        }
#pragma omp for schedule(dynamic, 1)
        for (int i = 0; i < nr; ++i) {
            if (!b0 || !b2) continue;
            int a = row_at(rows, i, lmin);
            for (int b = a; b <= lmax; ++b) {
                int jmin, jmin2, jmax = a + b;
                double X[8] = {0};
                double c;
                if (kind == 0 || kind == 2 || kind == 6) { /* one 00 family, squared */
                    int n = or_w3j_family(a, b, 0, 0, b0, &jmin);
                    for (int k = 0; k < n; ++k) b0[k] = b0[k] * b0[k];
                    for (int k = 0; k < K; ++k) X[k] = xi_sum(Wk[k], nW, b0, jmin, jmax, a, b, 0, absmode);
                } else if (kind == 1 || kind == 5) { /* one 22 family, squared, even parity */
                    int n = or_w3j_family(a, b, -2, 2, b0, &jmin);
                    for (int k = 0; k < n; ++k) b0[k] = b0[k] * b0[k];
                    for (int k = 0; k < K; ++k) X[k] = xi_sum(Wk[k], nW, b0, jmin, jmax, a, b, 1, absmode);
                } else if (kind == 4) { /* 00 x 22, even parity */
                    int n = or_w3j_family(a, b, 0, 0, b0, &jmin);
                    or_w3j_family(a, b, -2, 2, b2, &jmin2);
                    for (int k = 0; k < n; ++k) b2[k] *= b0[k];
                    for (int k = 0; k < K; ++k) X[k] = xi_sum(Wk[k], nW, b2, jmin, jmax, a, b, 1, absmode);
                } else { /* TETE: 00x22 for W1,3,4,5 (Xi_TE) and 00^2 for W2 (Xi_TT) */
                    int n = or_w3j_family(a, b, 0, 0, b0, &jmin);
                    or_w3j_family(a, b, -2, 2, b2, &jmin2);
                    for (int k = 0; k < n; ++k) b2[k] *= b0[k];
                    for (int k = 0; k < n; ++k) b0[k] *= b0[k];
                    X[0] = xi_sum(Wk[0], nW, b2, jmin, jmax, a, b, 1, absmode);
                    X[1] = xi_sum(Wk[1], nW, b0, jmin, jmax, a, b, 0, absmode);
                    X[2] = xi_sum(Wk[2], nW, b2, jmin, jmax, a, b, 1, absmode);
                    X[3] = xi_sum(Wk[3], nW, b2, jmin, jmax, a, b, 1, absmode);
                    X[4] = xi_sum(Wk[4], nW, b2, jmin, jmax, a, b, 1, absmode);
                }
                switch (kind) {
                case 0:
                case 1: { /* src/covariance.jl:110-118 and :171-179 */
                    const double *ip = S[0], *jq = S[1], *iq = S[2], *jp = S[3];
                    const double *rip = R[0], *rjq = R[1], *riq = R[2], *rjp = R[3];
                    c = sqrt(ip[a] * ip[b] * jq[a] * jq[b]) * X[0] + sqrt(iq[a] * iq[b] * jp[a] * jp[b]) * X[1] +
                        sqrt(ip[a] * ip[b]) * X[2] * rjq[a] * rjq[b] + sqrt(jq[a] * jq[b]) * X[3] * rip[a] * rip[b] +
                        sqrt(iq[a] * iq[b]) * X[4] * rjp[a] * rjp[b] + sqrt(jp[a] * jp[b]) * X[5] * riq[a] * riq[b] +
                        X[6] * rip[a] * rjq[a] * rip[b] * rjq[b] + X[7] * riq[a] * rjp[a] * riq[b] * rjp[b];
                    break;
                }
                case 2: { /* src/covariance.jl:225-230 */
                    const double *TTip = S[0], *TTjp = S[1], *TEiq = S[2], *TEjq = S[3];
                    const double *rip = R[0], *rjp = R[1];
                    c = (sqrt(TTip[a] * TTip[b]) * (TEjq[a] + TEjq[b]) * X[0] +
                         sqrt(TTjp[a] * TTjp[b]) * (TEiq[a] + TEiq[b]) * X[1] +
                         (TEjq[a] + TEjq[b]) * X[2] * rip[a] * rip[b] + (TEiq[a] + TEiq[b]) * X[3] * rjp[a] * rjp[b]) /
                        2;
                    break;
                }
                case 3: { /* src/covariance.jl:292-297 */
                    const double *TTip = S[0], *EEjq = S[1], *TEiq = S[2], *TEjp = S[3];
                    const double *rT = R[0], *rP = R[1];
                    c = sqrt(TTip[a] * TTip[b] * EEjq[a] * EEjq[b]) * X[0] +
                        0.5 * (TEiq[a] * TEjp[b] + TEjp[a] * TEiq[b]) * X[1] +
                        sqrt(TTip[a] * TTip[b]) * X[2] * rP[a] * rP[b] + sqrt(EEjq[a] * EEjq[b]) * X[3] * rT[a] * rT[b] +
                        X[4] * rT[a] * rT[b] * rP[a] * rP[b];
                    break;
                }
                case 4:
                case 5: { /* src/covariance.jl:362-367 and :392-397 */
                    const double *EEjq = S[0], *EEjp = S[1], *TEip = S[2], *TEiq = S[3];
                    const double *rjq = R[0], *rjp = R[1];
                    c = (sqrt(EEjq[a] * EEjq[b]) * (TEip[a] + TEip[b]) * X[0] +
                         sqrt(EEjp[a] * EEjp[b]) * (TEiq[a] + TEiq[b]) * X[1] +
                         (TEip[a] + TEip[b]) * X[2] * rjq[a] * rjq[b] + (TEiq[a] + TEiq[b]) * X[3] * rjp[a] * rjp[b]) /
                        2;
                    break;
                }
                default: { /* src/covariance.jl:438-441 */
                    const double *TEip = S[0], *TEiq = S[1], *TEjq = S[2], *TEjp = S[3];
                    c = ((TEip[a] * TEjq[b] + TEjq[a] * TEip[b]) * X[0] + (TEiq[a] * TEjp[b] + TEjp[a] * TEiq[b]) * X[1]) /
                        2;
                    break;
                }
                }
                C[(long)(a - lmin) + (long)(b - lmin) * ldc] = c;
                C[(long)(b - lmin) + (long)(a - lmin) * ldc] = c;
            }
        }
        free(b0);
        free(b2);
    }
    return err;
}

/* l3-term count of one family over the pairs of the given rows, l3 <= nW-1
 * (the work unit used to scale a sampled CPU timing to a full workload). */
double or_l3_terms(int lmin, int lmax, long nW, const int *rows, int nrows)
{
    int nr = rows ? nrows : lmax - lmin + 1;
    double tot = 0.0;
    for (int i = 0; i < nr; ++i) {
        int a = row_at(rows, i, lmin);
        for (int b = a; b <= lmax; ++b) {
            long lo = b - a, hi = a + b;
            if (hi > nW - 1) hi = nW - 1;
            if (hi >= lo) tot += (double)(hi - lo + 1);
        }
    }
    return tot;
}

int or_loop_cov(int kind, const double *const *S, const double *const *R, const double *const *Wk, long nW, int lmin,
                int lmax, double *C, long ldc, const int *rows, int nrows, int nthreads)
{
    return loop_cov_impl(kind, S, R, Wk, nW, lmin, lmax, C, ldc, rows, nrows, nthreads, 0);
}

/* The same covariance formula evaluated on |spectra|, |ratios|, |W| and |3j
 * products|: the size of the sum of |terms| behind each element, i.e. the
 * scale below which an FP64 evaluation cannot resolve a cancelling element. */
int or_loop_cov_abs(int kind, const double *const *S, const double *const *R, const double *const *Wk, long nW,
                    int lmin, int lmax, double *C, long ldc, const int *rows, int nrows, int nthreads)
{
    int nr = kind == 6 ? 0 : (kind >= 0 && kind < 7 ? (kind < 2 ? 4 : 2) : 0);
    size_t n = (size_t)lmax + 1;
    double *buf = (double *)malloc(sizeof(double) * n * 8);
    if (!buf) return 2;
    const double *Sa[4], *Ra[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
        for (size_t l = 0; l < n; ++l) buf[i * n + l] = fabs(S[i][l]);
        Sa[i] = buf + i * n;
    }
    for (int i = 0; i < nr; ++i) {
        for (size_t l = 0; l < n; ++l) buf[(4 + i) * n + l] = fabs(R[i][l]);
        Ra[i] = buf + (4 + i) * n;
    }
    int st = loop_cov_impl(kind, Sa, Ra, Wk, nW, lmin, lmax, C, ldc, rows, nrows, nthreads, 1);
    free(buf);
    return st;
}

/* quickpolXi! (src/beam.jl:72-109): for l'' = 2..lmax and l in the band
 * max(2, l''-bl) .. min(lmax, l''+bu), Xi[l'', l] = sgn * sum_l' W[l'] f1(l') f2(l')
 * with f_k(l') = (l' l l''; s_k+nu_k, -s_k, -nu_k) over the common support of the
 * two families (Xisum, src/beam.jl:17-28), W[l'] = 0 for l' >= nW, and
 * sgn = (-1)^(s1+s2+nu1+nu2).  Xi is dense column-major (lmax+1)^2; entries
 * outside the band are left untouched. */
static int quickpol_xi_impl(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu,
                            double *Xi, long ldx, int nthreads, int absmode, int common)
{
    if (lmax < 0 || bl < 0 || bu < 0 || ldx < lmax + 1) return 1;
    int nt = nthreads_or_default(nthreads);
    int blen = 2 * lmax + 2;
    int err = 0;
    const double sgn = ((s1 + s2 + nu1 + nu2) % 2 == 0) ? 1.0 : -1.0;
#pragma omp parallel num_threads(nt)
    {
        double *f1 = (double *)malloc(sizeof(double) * (size_t)blen);
        double *f2 = (double *)malloc(sizeof(double) * (size_t)blen);
        if (!f1 || !f2) {
#pragma omp atomic write
            err = 2;
        }
#pragma omp for schedule(dynamic, 1)
        for (int lpp = 2; lpp <= lmax; ++lpp) {
            if (!f1 || !f2) continue;
            int lo = lpp - bl > 2 ? lpp - bl : 2, hi = lpp + bu < lmax ? lpp + bu : lmax;
            for (int l = lo; l <= hi; ++l) {
                /* (l' l l''; s+nu, -s, -nu) = (l l'' l'; -s, -nu, s+nu): the family over the third column */
                int j1, j2, jm = -1;
                if (common) {
                    /* both families matched at one point: the larger of their midpoints */
                    int jmax = l + lpp, a1 = abs(s1 + nu1), a2 = abs(s2 + nu2), d = abs(l - lpp);
                    int jmin1 = d > a1 ? d : a1, jmin2 = d > a2 ? d : a2;
                    int m1 = (jmin1 + jmax) / 2, m2 = (jmin2 + jmax) / 2;
                    jm = m1 > m2 ? m1 : m2;
                }
                int n1 = w3j_family_at(l, lpp, -s1, -nu1, jm, f1, &j1);
                int n2 = w3j_family_at(l, lpp, -s2, -nu2, jm, f2, &j2);
                int a = j1 > j2 ? j1 : j2;
                int b1 = j1 + n1 - 1, b2 = j2 + n2 - 1;
                int b = b1 < b2 ? b1 : b2;
                if (b > nW - 1) b = (int)(nW - 1);
                double acc = 0.0;
                if (absmode)
                    for (int lp = a; lp <= b; ++lp) acc += fabs(W[lp] * f1[lp - j1] * f2[lp - j2]);
                else
                    for (int lp = a; lp <= b; ++lp) acc += W[lp] * f1[lp - j1] * f2[lp - j2];
                Xi[(long)lpp + (long)l * ldx] = absmode ? acc : sgn * acc;
            }
        }
        free(f1);
        free(f2);
    }
    return err;
}

int or_quickpol_xi(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu, double *Xi,
                   long ldx, int nthreads)
{
    return quickpol_xi_impl(nu1, nu2, s1, s2, W, nW, lmax, bl, bu, Xi, ldx, nthreads, 0, 0);
}

/* The same sums over |W f1 f2| (the sum of |terms| behind each element). */
int or_quickpol_xi_abs(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu,
                       double *Xi, long ldx, int nthreads)
{
    return quickpol_xi_impl(nu1, nu2, s1, s2, W, nW, lmax, bl, bu, Xi, ldx, nthreads, 1, 0);
}

/* quickpolXi! with both families of an element matched at one common point, the
 * larger of their midpoints (each family's forward sweep from its own jmin, one
 * backward sweep from the common jmax; a family whose support starts past that
 * point is the backward sweep alone).  The same 3j values as or_quickpol_xi up
 * to the recurrences' conditioning; this is the match the GPU kernel uses, so
 * the two agree to rounding. */
int or_quickpol_xi_common(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu,
                          double *Xi, long ldx, int nthreads)
{
    return quickpol_xi_impl(nu1, nu2, s1, s2, W, nW, lmax, bl, bu, Xi, ldx, nthreads, 0, 1);
}
