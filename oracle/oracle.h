/*
 * oracle.h -- CPU FP64 restatement of the PowerSpectra.jl mode-coupling /
 * covariance hot loops.  TEST INFRASTRUCTURE ONLY: the checker for the CUDA
 * library, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg.  Never linked into the product library.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* (l1 l2 l3; m1 m2 -m1-m2) for l3 = jmin..l1+l2 into out; returns the count.
 * Follows src/modecoupling.jl:69-75 (fill_3j! -> WignerF + wigner3j_f!). */
int or_w3j_family(int l1, int l2, int m1, int m2, double *out, int *jmin_out);

/* inner_mcm00!/02!/++!/--! (src/modecoupling.jl:78-159).  spin: 0=00, 1=02,
 * 2=++, 3=--.  M is column-major with leading dimension ldm, index (l-lmin).
 * rows (optional) restricts the l1 rows computed (for sampled timing). */
int or_inner_mcm(int spin, const double *W, long nW, int lmin, int lmax, double *M, long ldm,
                 const int *rows, int nrows, int nthreads);

/* Symmetric Xi matrix for one window: product 0=00^2, 1=22^2, 2=00x22;
 * parity 0=all, 1=even, 2=odd (src/modecoupling.jl:3-66). */
int or_xi(int product, int parity, const double *W, long nW, int lmin, int lmax, double *X, long ldx, int nthreads);

/* loop_cov*! (src/covariance.jl:92-446).  kind: 0=TTTT 1=EEEE 2=TTTE 3=TETE
 * 4=TEEE 5=TEEE_PLANCK 6=TTEE.  S, R, W follow the reference argument order. */
int or_loop_cov(int kind, const double *const *S, const double *const *R, const double *const *W, long nW, int lmin,
                int lmax, double *C, long ldc, const int *rows, int nrows, int nthreads);

/* Same loops on |W|, |3j products| (and |spectra|, |ratios| for covariance):
 * the sum of |terms| behind each element, the resolution scale of an FP64 sum. */
int or_inner_mcm_abs(int spin, const double *W, long nW, int lmin, int lmax, double *M, long ldm,
                     const int *rows, int nrows, int nthreads);
int or_loop_cov_abs(int kind, const double *const *S, const double *const *R, const double *const *W, long nW,
                    int lmin, int lmax, double *C, long ldc, const int *rows, int nrows, int nthreads);

/* quickpolXi! (src/beam.jl:72-109) into a dense column-major (lmax+1)^2 Xi,
 * rows l'' = 2..lmax, columns l within the band [l''-bl, l''+bu], l >= 2. */
int or_quickpol_xi(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu, double *Xi,
                   long ldx, int nthreads);
/* The same sums over |W f1 f2|: the sum of |terms| behind each element. */
int or_quickpol_xi_abs(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu,
                       double *Xi, long ldx, int nthreads);
/* or_quickpol_xi with both families matched at the larger of their midpoints (the GPU kernel's match). */
int or_quickpol_xi_common(int nu1, int nu2, int s1, int s2, const double *W, long nW, int lmax, int bl, int bu,
                          double *Xi, long ldx, int nthreads);

int or_cov_nwindows(int kind);
int or_max_threads(void);
double or_l3_terms(int lmin, int lmax, long nW, const int *rows, int nrows);

#ifdef __cplusplus
}
#endif
#endif
