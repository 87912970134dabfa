/*
 * powerspectra_gpu.h -- C ABI of the GB300 mode-coupling / covariance library.
 *
 * This is the drop-in boundary for the hot loops of PowerSpectra.jl.  A Julia
 * `ccall` (or Python ctypes, or C) replaces the bodies of
 *   inner_mcm00! / inner_mcm02! / inner_mcm++! / inner_mcm--!   (src/modecoupling.jl:78-159)
 *   loop_covTTTT! ... loop_covTTEE!                            (src/covariance.jl:92-446)
 * and keeps the callers (`mcm`, src/modecoupling.jl:192-256; `coupledcov`,
 * src/covariance.jl:34-61) and their SpectralArray return types unchanged.
 *
 * Conventions shared by every entry point:
 *   - Matrices are column-major (Julia's layout): element (l1, l2) of a result
 *     with axes lmin:lmax lives at M[(l1 - lmin) + (l2 - lmin) * ld], with
 *     ld >= lmax - lmin + 1.  This is `parent(M)` of a SpectralArray.
 *   - Spectra are 0-indexed by l (`parent(V)` of a SpectralVector): W[l] for
 *     l = 0..nW-1.  The l3 sum runs over the intersection of the 3j support and
 *     0..nW-1, exactly like Xi_TT/Xi_EE/Xi_EB/Xi_TE (src/modecoupling.jl:3-66).
 *   - Host-pointer entry points copy inputs in, compute, copy results out and
 *     return when the output is filled (synchronous, like the Julia loops).
 *     Outputs in page-locked host memory that is mapped into the device's
 *     address space (cudaHostAlloc, cudaHostRegister) are written by the
 *     kernel in place, with the same results.
 *     `_device` entry points take device pointers and enqueue on the context's
 *     stream without synchronising.
 *   - Every call returns PS_OK (0) or an error code; the message is kept per
 *     context (ps_last_error).  The Julia shim maps non-zero to `error()`, the
 *     way the reference raises on bad axes (@assert, src/modecoupling.jl:80)
 *     and on an unknown spectrum (ArgumentError, src/modecoupling.jl:225).
 *   - A context is not thread-safe: use one per host thread.
 */
#ifndef POWERSPECTRA_GPU_H
#define POWERSPECTRA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ps_ctx ps_ctx;

/* status codes */
#define PS_OK 0
#define PS_ERR_ARG 1          /* invalid argument (sizes, pointers, unknown case) */
#define PS_ERR_CUDA 2         /* a CUDA runtime call or kernel failed */
#define PS_ERR_OOM 3          /* device memory could not be allocated */
#define PS_ERR_TIMEOUT 4      /* a bounded device wait gave up */
#define PS_ERR_UNSUPPORTED 5  /* valid request this build does not provide */

/* spin cases of the mode-coupling matrix (src/modecoupling.jl:192-224) */
#define PS_SPIN_00 0 /* :TT, :M00                     -> inner_mcm00! */
#define PS_SPIN_02 1 /* :TE, :ET, :TB, :BT, :M02, :M20 -> inner_mcm02! */
#define PS_SPIN_PP 2 /* :M++ (EE/BB diagonal blocks)   -> inner_mcm++! */
#define PS_SPIN_MM 3 /* :M-- (EE/BB off-diagonal)      -> inner_mcm--! */

/* arithmetic of the 3j recurrence */
#define PS_MODE_PLAIN_FP64 0 /* everything in FP64 */
#define PS_MODE_CHOSEN 1     /* FP32-pipe recurrence with two-word compensation, FP64 anchors */

/* family products / parities for ps_xi (Xi_TT = (00^2, ALL), Xi_EE = (22^2, EVEN),
 * Xi_EB = (22^2, ODD), Xi_TE = (00x22, EVEN)) */
#define PS_PROD_00_00 0
#define PS_PROD_22_22 1
#define PS_PROD_00_22 2
#define PS_PARITY_ALL 0
#define PS_PARITY_EVEN 1
#define PS_PARITY_ODD 2

/* covariance kinds (src/covariance.jl:47-60 dispatch; :305-333 planck flag) */
#define PS_COV_TTTT 0
#define PS_COV_EEEE 1
#define PS_COV_TTTE 2
#define PS_COV_TETE 3
#define PS_COV_TEEE 4        /* planck=false: 00x22 family product */
#define PS_COV_TEEE_PLANCK 5 /* planck=true (the reference default): 22^2 */
#define PS_COV_TTEE 6

/* Context lifetime.  Replaces get_thread_buffers (src/workspace.jl:216-223):
 * device buffers are owned by the context and reused across calls. */
int ps_create(int device, ps_ctx **out);
void ps_destroy(ps_ctx *ctx);
const char *ps_last_error(const ps_ctx *ctx);
/* Use an external cudaStream_t (passed as void*) for all later work; NULL
 * restores the context's own stream. */
int ps_set_stream(ps_ctx *ctx, void *cuda_stream);
int ps_synchronize(ps_ctx *ctx);

/* One spin case: the body of inner_mcm00!/02!/++!/--! (src/modecoupling.jl:78-159).
 * W: host, nW entries.  M: host, column-major, ld = ldm. */
int ps_mcm(ps_ctx *ctx, int spin, const double *W, int64_t nW, int lmin, int lmax, int mode, double *M,
           int64_t ldm);

/* Several spin cases of one (l1, l2) grid in one pass: bit s of `cases` selects
 * PS_SPIN_s, W[s] is its spectrum and M[s] its output.  The 00 and 22 families
 * are generated once per pair and shared by every selected case; ++ and --
 * come from one 22 family (the reference runs inner_mcm++! and inner_mcm--!
 * separately for :EE_BB / :EB_BE, src/modecoupling.jl:210-223). */
int ps_mcm_multi(ps_ctx *ctx, unsigned cases, const double *const W[4], int64_t nW, int lmin, int lmax, int mode,
                 double *const M[4], int64_t ldm);
/* Same with device pointers, enqueued on the context stream (no host copies). */
int ps_mcm_multi_device(ps_ctx *ctx, unsigned cases, const double *const dW[4], int64_t nW, int lmin, int lmax,
                        int mode, double *const dM[4], int64_t ldm);

/* Symmetric Xi matrices (no (2l+1) weights) of K windows sharing one family
 * product and parity: Xi_k[l1,l2] = sum_l3 (2 l3 + 1) x(l3) W_k[l3] / 4pi.
 * The projectors of src/modecoupling.jl:3-66 over a whole (l1, l2) grid.
 * K <= 8. */
int ps_xi(ps_ctx *ctx, int product, int parity, const double *const *W, int K, int64_t nW, int lmin, int lmax,
          int mode, double *const *Xi, int64_t ldx);

/* Covariance block: the body of loop_cov<kind>! (src/covariance.jl:92-446).
 * S[0..3], R[0..nr-1] and W[0..nw-1] follow the reference's argument order:
 *   TTTT  S={TTip,TTjq,TTiq,TTjp} R={r_ip,r_jq,r_iq,r_jp} W1..W8
 *   EEEE  S={EEip,EEjq,EEiq,EEjp} R={r_ip,r_jq,r_iq,r_jp} W1..W8
 *   TTTE  S={TTip,TTjp,TEiq,TEjq} R={r_ip,r_jp}           W1..W4
 *   TETE  S={TTip,EEjq,TEiq,TEjp} R={r_TT_ip,r_PP_jq}     W1..W5
 *   TEEE, TEEE_PLANCK S={EEjq,EEjp,TEip,TEiq} R={r_EE_jq,r_EE_jp} W1..W4
 *   TTEE  S={TEip,TEiq,TEjq,TEjp} R={}                    W1..W2
 * S and R hold at least lmax+1 entries, each W holds nW.  C is symmetric. */
int ps_coupledcov(ps_ctx *ctx, int kind, const double *const *S, const double *const *R, const double *const *W,
                  int64_t nW, int lmin, int lmax, int mode, double *C, int64_t ldc);
int ps_coupledcov_device(ps_ctx *ctx, int kind, const double *const *dS, const double *const *dR,
                         const double *const *dW, int64_t nW, int lmin, int lmax, int mode, double *dC, int64_t ldc);
/* Several covariance blocks of one (l1, l2) grid (device pointers, enqueued
 * on the context stream): block b is ps_coupledcov_device(kinds[b], dS[b],
 * dR[b], dW[b], ..., dC[b]).  The reference computes one block per
 * loop_cov*! call.  Here, in chosen mode, the Xi of all the blocks' windows
 * are computed grouped across the blocks by family product and parity, so
 * one family generation serves each group: the squared (0 0 0) and squared
 * (2 -2 0) windows by the tensor-core kernels when there are enough of them
 * (the thresholds of ps_mcm_set_device; up to 15 per launch), the others by
 * the CUDA-core kernel in groups of up to 8.  Each block is then
 * formed from its windows' Xi by the same per-element formula as the fused
 * kernel.  Plain FP64, or ps_set_tensor_cores(ctx, 0), runs the fused kernel
 * block by block.  Scratch: one n x n FP64 matrix per window (n = lmax - lmin
 * + 1).  dR[b] may be NULL for kinds without noise ratios (TTEE). */
int ps_coupledcov_set_device(ps_ctx *ctx, int nblk, const int *kinds, const double *const *const *dS,
                             const double *const *const *dR, const double *const *const *dW, int64_t nW, int lmin,
                             int lmax, int mode, double *const *dC, int64_t ldc);

/* Many mask spectra on one (l1, l2) grid: for window k and every spin case s
 * selected in `cases`, dM[4*k + s] receives the matrix (entries of unselected
 * cases are ignored, and a NULL entry of a selected case skips that (window,
 * case) slot; at least one slot must remain).  This is `mcm` for a set of
 * spectra (the reference calls inner_mcm*! once per spectrum and case,
 * src/modecoupling.jl:192-246).  The (window, case) slots are processed in
 * groups of up to 8, each sharing one generation of the families per pair.
 * Device pointers; enqueued on the context stream. */
int ps_mcm_set_device(ps_ctx *ctx, unsigned cases, const double *const *dW, int K, int64_t nW, int lmin, int lmax,
                      int mode, double *const *dM, int64_t ldm);
/* In chosen mode, the TT slots of a set and its ++ and -- slots, each kind
 * when it has enough slots (TT: 4 or more at lmax >= 3072, 5 or more at
 * lmax >= 768, else 9; ++/--: 5 or more at lmax >= 1536, else 9), are
 * computed by the tensor-core kernels: one
 * generation of the (0 0 0) or (2 -2 0) family for up to 15 windows,
 * contracted by BF16 tcgen05 MMAs in a three-part split with FP32
 * accumulators and float-float totals (same 1e-6 bar).  Each such launch
 * first builds its table of window tiles in a context-owned device buffer of
 * (3 lmax + 160) x 3648 bytes (90 MB at lmax 8191), grown on demand.  Their
 * waits on the tensor core and on the tile copies are bounded: a wait that
 * gives up is reported as PS_ERR_TIMEOUT by the next ps_synchronize or
 * host-pointer call. */
/* The same with host spectra and host matrices: returns when every M is
 * filled (page-locked matrices are written by the kernel in place). */
int ps_mcm_set(ps_ctx *ctx, unsigned cases, const double *const *W, int K, int64_t nW, int lmin, int lmax, int mode,
               double *const *M, int64_t ldm);

/* decouple_covmat (src/covariance.jl:8-14): out = B1^-1 * Y * B2^-T for n x n
 * column-major host matrices Y, B1, B2 (leading dimension ld), by two FP64 LU
 * factorisations on the GPU (the reference's rdiv! with lu(parent(B)')).  A
 * singular B1 or B2 returns PS_ERR_ARG. */
int ps_decouple_covmat(ps_ctx *ctx, const double *Y, const double *B1, const double *B2, int64_t n, int64_t ld,
                       double *out, int64_t ldout);
/* The same on device matrices, so a covariance from ps_coupledcov_device is
 * decoupled without leaving the GPU.  Runs on the context stream and waits for
 * each factorisation's pivot status (to report a singular B1 or B2), so it
 * returns once `out` is written. */
int ps_decouple_covmat_device(ps_ctx *ctx, const double *dY, const double *dB1, const double *dB2, int64_t n,
                              int64_t ld, double *dout, int64_t ldout);
/* x = M \ b for an n x n coupling matrix and nrhs right-hand sides (host,
 * column-major): the decoupling `M \ pCl` of master (src/modecoupling.jl:358,
 * src/blockspectralmatrix.jl:124-129), by FP64 LU on the GPU. */
int ps_solve(ps_ctx *ctx, const double *M, int64_t n, int64_t ldm, const double *b, int nrhs, int64_t ldb, double *x,
             int64_t ldx);

/* QuickPol beam coupling (quickpolXi!, src/beam.jl:72-109): for l'' = 2..lmax
 * and l in [max(2, l''-bl), min(lmax, l''+bu)],
 *   Xi[l'', l] = (-1)^(s1+s2+nu1+nu2) sum_l' W[l'] (l' l l''; s1+nu1, -s1, -nu1)
 *                                                 (l' l l''; s2+nu2, -s2, -nu2)
 * over the two families' common support (Xisum, src/beam.jl:17-28), W[l'] = 0
 * for l' >= nW.  W is the scan-pattern spectrum (quickpolW); Xi is a dense
 * column-major (lmax+1) x (lmax+1) matrix (ld >= lmax+1) that receives the
 * band and zeros elsewhere.  General spins (|nu|, |s| <= 64); host pointers.
 * mode PS_MODE_PLAIN_FP64 runs the recurrences in FP64 like the reference;
 * PS_MODE_CHOSEN runs them in float-float on the FP32 pipe (max error 1e-6 of
 * the sum of |W f1 f2| behind each element, against FP64).  The reference stores Xi as a BandedMatrix; here the
 * band is written into a dense matrix. */
int ps_quickpol_xi(ps_ctx *ctx, int nu1, int nu2, int s1, int s2, const double *W, int64_t nW, int lmax, int bl,
                   int bu, int mode, double *Xi, int64_t ldx);
/* quickpolXi!(Xi, nu1, nu2, s1, s2, omega1, omega2) (src/beam.jl:72-109) from the
 * effective scan weights themselves: W = quickpolW(omega1, omega2)
 * (src/beam.jl:40-53), W[l'] = sum_m omega1_l'm conj(omega2_l'm) over m = -l'..l'
 * (m = 0 once, m > 0 twice), is formed on the GPU and then used as in
 * ps_quickpol_xi, with W[l'] = 0 beyond alm_lmax.  omega1 / omega2 are host
 * coefficient sets (interleaved re, im; HEALPix m-major order, alm_lmax /
 * alm_mmax). */
int ps_quickpol_xi_alm(ps_ctx *ctx, int nu1, int nu2, int s1, int s2, const double *omega1, const double *omega2,
                       int alm_lmax, int alm_mmax, int lmax, int bl, int bu, int mode, double *Xi, int64_t ldx);

/* Mask spectra from harmonic coefficients (alm2cl): for l = 0..lout,
 *   W[l] = (1/nterms) sum_t cl(A[t], B[t])[l],
 *   cl(a, b)[l] = (Re(a_l0 conj b_l0) + 2 sum_{m=1}^{min(l,mmax)} Re(a_lm conj b_lm)) / (2l+1).
 * Each set holds the complex coefficients of one real field as interleaved
 * (re, im) doubles in the HEALPix m-major order, (l, m) at m(2 lmax+1-m)/2 + l
 * (Healpix.jl's Alm).  A NULL set stands for all-zero coefficients: its term
 * adds nothing but still counts in 1/nterms.  Replaces window_function_W!
 * (src/workspace.jl:174-213), whose terms are the (wX, wY) effective-weight
 * pairs, and with nterms = 1 the alm2cl calls of mcm (src/modecoupling.jl:197,
 * :234) and master (src/modecoupling.jl:357-373).  1 <= nterms <= 16,
 * 0 <= mmax <= lmax, lout <= lmax.  FP64; the summation order is fixed, so
 * results are reproducible run to run.  ps_window_W takes host arrays and
 * returns when W is filled; ps_window_W_device takes 16-byte aligned device
 * sets and a device W and is enqueued on the context stream. */
int ps_window_W(ps_ctx *ctx, const double *const *A, const double *const *B, int nterms, int lmax, int mmax,
                int lout, double *W);
int ps_window_W_device(ps_ctx *ctx, const double *const *dA, const double *const *dB, int nterms, int lmax, int mmax,
                       int lout, double *dW);

/* One coupling problem of a batch (device pointers): K spectra of nW entries,
 * the spin cases to compute for each, and 4*K output slots (entry 4*k + s). */
typedef struct ps_problem {
    int lmin, lmax;
    unsigned cases;
    int K;
    int64_t nW;
    const double *const *W;
    double *const *M;
    int64_t ldm;
} ps_problem;

/* Batched uneven workload in one persistent launch (chosen arithmetic).
 * The reference has no counterpart: it runs the problems one `mcm` call at a
 * time.  prepare() splits every problem into window groups of up to
 * `group_slots` (2, 4 or 8) (window, case) slots -- whole windows per group, so
 * the ++ and -- of one spectrum share their family -- builds one work queue
 * over all problems ordered by kernel body and decreasing family length, and
 * uploads the tables; 0 for group_slots or blocks_per_sm picks the values
 * ps_batch_autotune() found, else defaults.  blocks_per_sm = -1 selects the
 * launch form instead: one chosen-kernel launch per window group.
 * A problem's TT slots and its ++/-- slots, when there are enough of them
 * for its lmax, go to tensor-core launches instead, as in ps_mcm_set_device
 * (unless ps_set_tensor_cores(ctx, 0)).
 * run() enqueues the window preparation, the tensor-core launches, then the
 * queue reset and ONE persistent kernel (or the per-group launches).  graph_launch() captures run()
 * into a CUDA graph on first use and replays it afterwards.  The problems'
 * pointers must stay valid while the batch is in use. */
int ps_batch_prepare(ps_ctx *ctx, const ps_problem *probs, int nprob, int group_slots, int blocks_per_sm);
int ps_batch_run(ps_ctx *ctx);
int ps_batch_graph_launch(ps_ctx *ctx);
/* Times every (group_slots in {2, 4, 8}) x (blocks per SM, or -1 for the
 * launch form) configuration on the given problems, keeps the fastest as the
 * context's default and returns it. */
int ps_batch_autotune(ps_ctx *ctx, const ps_problem *probs, int nprob, int *best_group_slots,
                      int *best_blocks_per_sm, double *best_ms);

/* No counterpart in the reference: an entry point for callers that may not
 * allocate device memory -- code whose GPU memory belongs to another allocator
 * (a framework's pool or a fixed budget) and pipelines that cannot take the
 * device-wide synchronisation cudaMalloc/cudaFree may cause.  It computes the
 * same matrices as ps_mcm_multi_device with PS_MODE_CHOSEN (same kernel, same
 * results) on the caller's current device and `stream` (a cudaStream_t), with
 * no context and no allocation: its scratch (padded windows and the work list,
 * 2.6 MB) is a fixed array in the library's device image, which every GPU that
 * loads the library keeps until the process exits.  Limits: lmax <= 4095 (a
 * larger lmax returns PS_ERR_ARG); `stream` must belong to the current device
 * (PS_ERR_ARG otherwise); all arguments are checked as for ps_mcm_multi_device.
 * Each call made outside stream capture looks up the array's device address
 * on the current device (so a device reset needs nothing special); a call
 * made during stream capture reuses the address that the last uncaptured
 * call on that device found, so make one call before capturing (PS_ERR_CUDA
 * otherwise).  Every call rewrites the whole scratch; calls whose GPU work
 * overlaps (other streams or host threads) share it and race, so serialise
 * them.  Returns a PS_* code only (there is no context to hold a message). */
int ps_mcm_multi_device_noalloc(unsigned cases, const double *const dW[4], int64_t nW, int lmin, int lmax,
                                double *const dM[4], int64_t ldm, void *stream);

/* Chosen-mode sets use the tensor-core kernels where they apply (enable = 1,
 * the default) or the CUDA-core kernels only (enable = 0). */
int ps_set_tensor_cores(ps_ctx *ctx, int enable);

/* Instrumentation: device time of the coupling kernels of the last call (CUDA
 * events on the launching stream, from the first coupling launch of the call
 * to the end of its last), number of kernels this context has launched, and a
 * measured FMA-pipe peak (flop/s, FMA = 2 flops) of this GPU in FP64 (fp64=1)
 * or FP32 (fp64=0). */
double ps_last_kernel_ms(const ps_ctx *ctx);
uint64_t ps_launch_count(const ps_ctx *ctx);
int ps_probe_fma_peak(ps_ctx *ctx, int fp64, double *flops_per_s);

#ifdef __cplusplus
}
#endif
#endif /* POWERSPECTRA_GPU_H */
