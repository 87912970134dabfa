// ps_linalg.cu -- dense solves downstream of the coupling matrices, on the GPU.
//
//   ps_decouple_covmat: decouple_covmat (src/covariance.jl:8-14),
//       B1^-1 * Y * B2^-T, by two LU factorisations (the reference's two rdiv!
//       with lu(parent(B)')).
//   ps_solve: M \ b for a square coupling matrix and nrhs right-hand sides,
//       the decoupling `M \ pCl` of master (src/modecoupling.jl:358,
//       src/blockspectralmatrix.jl:124-129).
//
// Both use cuSOLVER's FP64 getrf/getrs; a singular matrix is reported as
// PS_ERR_ARG (no device assert).  Matrices are column-major, as everywhere.
#include <cusolverDn.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "ps_internal.cuh"

namespace ps {

// dst (n x n, ld n) = src^T (n x n, ld n), 32 x 32 tiles through shared memory
__global__ void k_transpose(double* __restrict__ dst, const double* __restrict__ src, int n)
{
    __shared__ double tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int r = bx + threadIdx.x, c = by + k;
        if (r < n && c < n) tile[k][threadIdx.x] = src[(size_t)c * n + r];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int r = by + threadIdx.x, c = bx + k;
        if (r < n && c < n) dst[(size_t)c * n + r] = tile[threadIdx.x][k];
    }
}

cudaError_t launch_transpose(double* dst, const double* src, int n, cudaStream_t s)
{
    dim3 grid((n + 31) / 32, (n + 31) / 32), block(32, 8);
    k_transpose<<<grid, block, 0, s>>>(dst, src, n);
    return cudaGetLastError();
}

}  // namespace ps

// The solver state lives in the context (ps_api.cu) through these hooks.
struct ps_linalg {
    cusolverDnHandle_t h = nullptr;
    double* work = nullptr;
    int lwork = 0;
    int* ipiv = nullptr;
    int ipiv_n = 0;
    int* info = nullptr;
    double* a = nullptr;  // LU of the matrix being solved
    double* x = nullptr;  // right-hand sides / result
    double* t = nullptr;  // transpose scratch
    size_t cap = 0;       // elements of a / x / t
};

static int la_err(char* err, size_t n, int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, n, fmt, ap);
    va_end(ap);
    return code;
}

#define LA_CUDA(call)                                                                                        \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess)                                                                               \
            return la_err(err, errn, e_ == cudaErrorMemoryAllocation ? PS_ERR_OOM : PS_ERR_CUDA, "%s: %s", #call, \
                          cudaGetErrorString(e_));                                                           \
    } while (0)
#define LA_SOLVER(call)                                                                                 \
    do {                                                                                                \
        cusolverStatus_t s_ = (call);                                                                   \
        if (s_ != CUSOLVER_STATUS_SUCCESS) return la_err(err, errn, PS_ERR_CUDA, "%s: status %d", #call, (int)s_); \
    } while (0)

static int la_reserve(ps_linalg* L, size_t n2, int n, cudaStream_t s, char* err, size_t errn)
{
    if (!L->h) {
        LA_SOLVER(cusolverDnCreate(&L->h));
    }
    LA_SOLVER(cusolverDnSetStream(L->h, s));
    if (n2 > L->cap) {
        cudaFree(L->a);
        cudaFree(L->x);
        cudaFree(L->t);
        L->a = L->x = L->t = nullptr;
        L->cap = 0;
        LA_CUDA(cudaMalloc((void**)&L->a, n2 * sizeof(double)));
        LA_CUDA(cudaMalloc((void**)&L->x, n2 * sizeof(double)));
        LA_CUDA(cudaMalloc((void**)&L->t, n2 * sizeof(double)));
        L->cap = n2;
    }
    if (n > L->ipiv_n) {
        cudaFree(L->ipiv);
        L->ipiv = nullptr;
        L->ipiv_n = 0;
        LA_CUDA(cudaMalloc((void**)&L->ipiv, (size_t)n * sizeof(int)));
        L->ipiv_n = n;
    }
    if (!L->info) LA_CUDA(cudaMalloc((void**)&L->info, sizeof(int)));
    int lw = 0;
    LA_SOLVER(cusolverDnDgetrf_bufferSize(L->h, n, n, L->a, n, &lw));
    if (lw > L->lwork) {
        cudaFree(L->work);
        L->work = nullptr;
        L->lwork = 0;
        LA_CUDA(cudaMalloc((void**)&L->work, (size_t)lw * sizeof(double)));
        L->lwork = lw;
    }
    return PS_OK;
}

// LU-factor L->a (n x n) and overwrite x (n x nrhs, ld n) with a^-1 x.
static int la_lu_solve(ps_linalg* L, int n, int nrhs, double* x, cudaStream_t s, const char* what, char* err,
                       size_t errn)
{
    LA_SOLVER(cusolverDnDgetrf(L->h, n, n, L->a, n, L->work, L->ipiv, L->info));
    int info = 0;
    LA_CUDA(cudaMemcpyAsync(&info, L->info, sizeof(int), cudaMemcpyDeviceToHost, s));
    LA_CUDA(cudaStreamSynchronize(s));
    if (info > 0) return la_err(err, errn, PS_ERR_ARG, "%s is singular (zero pivot %d)", what, info);
    if (info < 0) return la_err(err, errn, PS_ERR_CUDA, "getrf argument %d invalid", -info);
    LA_SOLVER(cusolverDnDgetrs(L->h, CUBLAS_OP_N, n, nrhs, L->a, n, L->ipiv, x, n, L->info));
    return PS_OK;
}

ps_linalg* ps_linalg_new() { return new ps_linalg(); }

void ps_linalg_free(ps_linalg* L)
{
    if (!L) return;
    if (L->h) cusolverDnDestroy(L->h);
    cudaFree(L->work);
    cudaFree(L->ipiv);
    cudaFree(L->info);
    cudaFree(L->a);
    cudaFree(L->x);
    cudaFree(L->t);
    delete L;
}

// Copy a column-major host (or device) matrix (ld) into a dense device matrix (ld = rows).
static int la_in(double* dst, const double* src, int rows, int cols, int64_t ld, cudaStream_t s, char* err, size_t errn,
                 bool on_device = false)
{
    LA_CUDA(cudaMemcpy2DAsync(dst, (size_t)rows * sizeof(double), src, (size_t)ld * sizeof(double),
                              (size_t)rows * sizeof(double), (size_t)cols,
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    return PS_OK;
}

int ps_linalg_decouple(ps_linalg* L, const double* Y, const double* B1, const double* B2, int n, int64_t ldin,
                       double* out, int64_t ldout, cudaStream_t s, char* err, size_t errn, bool on_device)
{
    int st = la_reserve(L, (size_t)n * n, n, s, err, errn);
    if (st) return st;
    if ((st = la_in(L->x, Y, n, n, ldin, s, err, errn, on_device))) return st;
    if ((st = la_in(L->a, B1, n, n, ldin, s, err, errn, on_device))) return st;
    if ((st = la_lu_solve(L, n, n, L->x, s, "B1", err, errn))) return st;  // x = B1^-1 Y
    LA_CUDA(ps::launch_transpose(L->t, L->x, n, s));                        // t = x^T
    if ((st = la_in(L->a, B2, n, n, ldin, s, err, errn, on_device))) return st;
    if ((st = la_lu_solve(L, n, n, L->t, s, "B2", err, errn))) return st;  // t = B2^-1 x^T
    LA_CUDA(ps::launch_transpose(L->x, L->t, n, s));                        // x = x B2^-T
    LA_CUDA(cudaMemcpy2DAsync(out, (size_t)ldout * sizeof(double), L->x, (size_t)n * sizeof(double),
                              (size_t)n * sizeof(double), (size_t)n,
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    LA_CUDA(cudaStreamSynchronize(s));
    return PS_OK;
}

int ps_linalg_solve(ps_linalg* L, const double* M, int n, int64_t ldm, const double* b, int nrhs, int64_t ldb,
                    double* x, int64_t ldx, cudaStream_t s, char* err, size_t errn)
{
    size_t need = (size_t)n * (size_t)(n > nrhs ? n : nrhs);
    int st = la_reserve(L, need, n, s, err, errn);
    if (st) return st;
    if ((st = la_in(L->a, M, n, n, ldm, s, err, errn))) return st;
    if ((st = la_in(L->x, b, n, nrhs, ldb, s, err, errn))) return st;
    if ((st = la_lu_solve(L, n, nrhs, L->x, s, "M", err, errn))) return st;
    LA_CUDA(cudaMemcpy2DAsync(x, (size_t)ldx * sizeof(double), L->x, (size_t)n * sizeof(double),
                              (size_t)n * sizeof(double), (size_t)nrhs, cudaMemcpyDeviceToHost, s));
    LA_CUDA(cudaStreamSynchronize(s));
    return PS_OK;
}
