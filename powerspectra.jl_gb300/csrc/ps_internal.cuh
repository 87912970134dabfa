// ps_internal.cuh -- shared declarations of the powerspectra_gpu library.
//
// Data layout on the device (one context owns all of it, reused across calls):
//   * windows:  K padded rows of length wlen = 2*lmax + 2 holding
//               (2 l3 + 1) * W_k[l3] for l3 < nW and 0 beyond, so every family
//               read (l3 <= l1 + l2 <= 2 lmax) stays in bounds without a branch.
//   * tasks:    int2 (l1, l2_0) per warp, 32 consecutive l2 of one l1 row,
//               heaviest rows first (the family length is 2 l1 + 1).  The
//               plain kernel's list steps from l2 = l1 row by row; the chosen
//               kernel's list is tiled, kTileRows consecutive rows per block
//               over one 32-column block (see tile_task_list in ps_api.cu).
//   * outputs:  column-major (Julia) matrices, element (l1, l2) at
//               (l1 - lmin) + (l2 - lmin) * ld.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/powerspectra_gpu.h"

namespace ps {

constexpr int kMaxWin = 8;       // windows (slots) per coupling launch
constexpr int kWarpsPerBlock = 4;
constexpr int kTileRows = 4;  // rows per tile of the chosen kernel's task list (one per warp)
constexpr double kInv4Pi = 0.079577471545947667884;  // 1 / (4 pi)

// Family product a window is contracted with.
enum Product : int { PROD_00_00 = 0, PROD_22_22 = 1, PROD_00_22 = 2 };
// l3 parity filter relative to l1 + l2 + l3.
enum Parity : int { PAR_ALL = 0, PAR_EVEN = 1, PAR_ODD = 2 };
// What the kernel writes per pair.
enum Epilogue : int { EPI_MCM = 0, EPI_XI = 1, EPI_COV = 2 };

struct WinDesc {
    const double* wW;  // padded (2 l3 + 1) W[l3], length wlen >= 2 lmax + 2
    const int2* bf;    // the same values split as (float mantissa bits, int exponent) for the chosen kernel
    int product;
    int parity;
};

struct CouplingParams {
    int lmin, lmax;
    int nwin;
    WinDesc win[kMaxWin];
    const int2* tasks;
    int ntasks;
    int epilogue;
    double* out[kMaxWin];  // EPI_MCM / EPI_XI: one matrix per window; EPI_COV: out[0]
    long long ldo;
    int wlen;  // length of the padded window arrays
    int cov_kind;
    const double* S[4];  // covariance signal spectra (length >= lmax + 1), reference argument order
    const double* R[4];  // covariance noise ratios
};

// One window of a batch: user spectrum -> padded (2l+1)W row and its split copy.
struct WinPrep {
    const double* src;
    long long nW;
    double* wW;
    int2* bf;
    int wlen;
};

// Persistent batched launch: groups[item.x] holds the coupling parameters of
// an item int4 (group, l1, first l2, w) with w = tasks | families << 8 |
// kernel body << 12 (families: 1 = 00 only, 2 = 22 only, 3 = both).
struct BatchParams {
    const CouplingParams* groups;
    const int4* items;
    int nitems;
    unsigned* counter;  // work-queue head, zeroed before every launch
};

// Launchers (ps_plain_fp64.cu, ps_chosen.cu).
// The batched kernel with NWIN = 4 or 8 slots per group (nwin > 4 selects 8).
cudaError_t launch_batch_chosen(const BatchParams& bp, int blocks, int nwin, cudaStream_t s);
int batch_blocks_per_sm(int nwin);
int chosen_batch_template(const CouplingParams& p, int nwin);  // compile-time slot set of a batch group (0: none fits)
cudaError_t launch_prep_windows(const WinPrep* list, int n, int max_wlen, cudaStream_t s);
cudaError_t launch_plain_fp64(const CouplingParams& p, cudaStream_t s);
cudaError_t launch_chosen(const CouplingParams& p, cudaStream_t s);
cudaError_t launch_pad_windows(double* dst, const double* src, long long nW, int wlen, cudaStream_t s);
cudaError_t launch_split_windows(int2* dst, const double* wW, int wlen, cudaStream_t s);

// Exponent marking an exact zero in the split window arrays.
constexpr int kZeroExp = -100000;
cudaError_t launch_fma_probe(int fp64, double* sink, int blocks, int iters, cudaStream_t s);
cudaError_t launch_transpose(double* dst, const double* src, int n, cudaStream_t s);
cudaError_t launch_quickpol(const double* W, long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1, int s2,
                            double* Xi, long long ldx, cudaStream_t s);
// The chosen-arithmetic QuickPol Xi (ps_quickpol_ff.cu); wf: nW floats, e: one int of scratch.
cudaError_t launch_quickpol_ff(const double* W, long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1,
                               int s2, double* Xi, long long ldx, float* wf, int* e, cudaStream_t s);

// alm2cl reduction (ps_window.cu).  Term t pairs coefficient sets a[t], b[t]
// (HEALPix m-major order, lmax / mmax); a null set stands for all zeros.
constexpr int kAlmMaxTerms = 16;
constexpr int kAlmChunk = 64;  // m values per block of the partial-sum kernel
struct AlmParams {
    const double2* a[kAlmMaxTerms];
    const double2* b[kAlmMaxTerms];
    int nterms;
    int lmax, mmax, lout;
    int mchunk, nmchunks;
    double* partial;  // nterms * nmchunks * (lout + 1)
};
int alm2cl_chunks(int mmax);
// after_partial, when given, is recorded between the partial-sum kernel and the reduction.
cudaError_t launch_alm2cl(const AlmParams& p, double scale, bool per_l, double* W, cudaStream_t s,
                          cudaEvent_t after_partial = nullptr);

// Tensor-core coupling kernels for sets of windows (ps_mma.cu): up to
// kMmaMaxSlots windows per launch, all with the squared (2 -2 0) family (each
// with a parity) or all with the squared (0 0 0) family (PAR_ALL), contracted
// on the tensor cores; one more MMA column forms the normalisation.
constexpr int kMmaCols = 16;
constexpr int kMmaMaxSlots = kMmaCols - 1;
struct MmaParams {
    int lmin, lmax;
    int nslot;                          // 1 .. kMmaMaxSlots
    const int2* bf[kMmaMaxSlots];       // split windows (mantissa, exponent), length wlen
    const double* wW[kMmaMaxSlots];     // padded windows (2 l3 + 1) W[l3]: the last forward point in FP64
    int parity[kMmaMaxSlots];           // PAR_ALL / PAR_EVEN / PAR_ODD of l1 + l2 + l3
    double* out[kMmaMaxSlots];
    long long ldo;
    int wlen;
    int epilogue;                       // EPI_MCM or EPI_XI
    int stage_rows;                     // 1: outputs in host memory, their scattered half staged
    const int2* tiles;                  // (r0, c0): rows r0 + 2w, columns c0 + 2i
    int ntiles;
    unsigned* status;                   // set to 1 when a bounded wait gives up
    // scratch of mma_table_bytes(lmax) bytes (256-byte aligned) for the launch's table of B
    // tiles; launch_mma fills it, and the entry ranges below, on the stream before the kernel
    unsigned char* tab;
    int tab_fmin, tab_nf, tab_bmin, tab_nb;  // forward entries l3 = fmin .. fmin + nf - 1, then backward ones
};
// fam00: the (0 0 0) family (every slot PAR_ALL); otherwise the (2 -2 0) family.  Two
// launches: the table of B tiles, then the coupling kernel.
cudaError_t launch_mma(const MmaParams& p, bool fam00, cudaStream_t s);
size_t mma_table_bytes(int lmax);

// A covariance block from its Xi matrices (ps_cov_combine.cu): C[l1, l2] =
// cov_combine(kind, S, R, {X_k[l1, l2]}, l1, l2) over the whole n x n block.
struct CovCombineParams {
    int kind, lmin, n, nx;     // nx: the block's windows (cov_nwindows(kind))
    const double* S[4];
    const double* R[4];
    const double* X[kMaxWin];  // the block's windows' Xi, n x n, leading dimension ldx
    long long ldx;
    double* C;
    long long ldc;
};
cudaError_t launch_cov_combine(const CovCombineParams& p, cudaStream_t s);

// Host-side covariance table (ps_api.cu).
int cov_nwindows(int kind);
int cov_nratios(int kind);
void cov_window_spec(int kind, int k, int* product, int* parity);

}  // namespace ps
