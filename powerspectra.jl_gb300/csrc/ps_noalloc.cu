// ps_noalloc.cu -- mode-coupling matrices without any device allocation.
//
// Some callers of this library are not allowed to call cudaMalloc: code whose
// device memory is owned by another allocator (a framework's caching pool or a
// fixed budget that must not grow), and pipelines that cannot afford the
// implicit device-wide synchronisation that cudaMalloc and cudaFree may cause
// in the middle of their stream work.  ps_mcm_multi_device_noalloc serves
// them: it runs the chosen coupling kernel (the same kernel ps_mcm_multi_device
// runs with PS_MODE_CHOSEN) with its scratch memory taken from a fixed array
// that lives in the library's device image instead of from cudaMalloc.
//
// The scratch holds the padded windows, their split (mantissa, exponent) copies
// and the warp task list.  Every call rewrites all of it before use, so nothing
// has to start at zero, but every call on a device shares this one array:
// calls whose GPU work overlaps (on different streams or threads) race.
#include "ps_internal.cuh"

#include <stdint.h>
#include <string.h>

namespace {

constexpr int kNoAllocMaxLmax = 4095;  // largest lmax the fixed scratch serves
constexpr int kNoAllocMaxWlen = 2 * kNoAllocMaxLmax + 2;
constexpr int kNoAllocMaxTasks = (kNoAllocMaxLmax + 1) * (kNoAllocMaxLmax + 2) / 64 + kNoAllocMaxLmax + 1;
// (the tiled list at lmax 4095, lmin 0 holds 264192 tasks; fewer for any smaller range)

// windows: 4 x wlen doubles, split copies: 4 x wlen int2, tasks: int2 each
constexpr size_t kWinBytes = 4ull * kNoAllocMaxWlen * sizeof(double);
constexpr size_t kBfBytes = 4ull * kNoAllocMaxWlen * sizeof(int2);
constexpr size_t kTaskBytes = (size_t)kNoAllocMaxTasks * sizeof(int2);
constexpr size_t kScratchBytes = kWinBytes + kBfBytes + kTaskBytes;  // 2.6 MB

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device, looked up once with that device current.
constexpr int kMaxDevices = 64;
static void* g_scratch_addr[kMaxDevices];

// The chosen kernel's tiled task list (the context path builds the same on
// the host): with nb = ceil(n / 32) and o = lmax + 1 - 32 nb, tile (g, b)
// holds rows o + 4g .. o + 4g + 3 (l1 = -1 below lmin) over the 32 columns
// from o + 32 b, b = g / 8 .. nb - 1, for row groups g from 8 nb - 1 down to
// (lmin - o) / 4.  tiles_below(m, nb) counts the tiles of row groups 0 .. m - 1:
// the sum of nb - g / 8 over g < m.
__host__ __device__ inline long long tiles_below(long long m, long long nb)
{
    const long long q = m / 8, r = m % 8;
    return m * nb - (4 * q * (q - 1) + r * q);
}

// One thread per row group writes its tiles' tasks.
__global__ void k_fill_tiles(int2* __restrict__ tasks, int lmin, int lmax)
{
    const int n = lmax - lmin + 1, NB = (n + 31) / 32, o = lmax + 1 - 32 * NB, glo = (lmin - o) / 4;
    const long long top = tiles_below(8LL * NB, NB);
    for (int g = glo + blockIdx.x * blockDim.x + threadIdx.x; g < 8 * NB; g += gridDim.x * blockDim.x) {
        long long t = top - tiles_below(g + 1, NB);  // groups above g come first
        for (int b = g / 8; b < NB; ++b, ++t)
            for (int q = 0; q < 4; ++q) {
                const int l1 = o + 4 * g + q;
                tasks[4 * t + q] = make_int2(l1 >= lmin ? l1 : -1, o + 32 * b);
            }
    }
}

}  // namespace

extern "C" int ps_mcm_multi_device_noalloc(unsigned cases, const double* const dW[4], int64_t nW, int lmin, int lmax,
                                           double* const dM[4], int64_t ldm, void* stream)
{
    if (cases == 0 || (cases & ~0xFu) || !dW || !dM) return PS_ERR_ARG;
    if (lmin < 0 || lmax < lmin || nW < 1 || ldm < (int64_t)(lmax - lmin + 1)) return PS_ERR_ARG;
    if (lmax > kNoAllocMaxLmax) return PS_ERR_ARG;  // beyond what the fixed scratch holds
    for (int s = 0; s < 4; ++s)
        if ((cases & (1u << s)) && (!dW[s] || !dM[s])) return PS_ERR_ARG;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return PS_ERR_CUDA;
    }
    // First call on this device: find where g_scratch lives in its memory.
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return PS_ERR_CUDA;
        }
        g_scratch_addr[dev] = ptr;
    }
    unsigned char* base = (unsigned char*)g_scratch_addr[dev];
    double* win = (double*)base;
    int2* bf = (int2*)(base + kWinBytes);
    int2* tasks = (int2*)(base + kWinBytes + kBfBytes);
    cudaStream_t s = (cudaStream_t)stream;

    ps::CouplingParams p;
    memset(&p, 0, sizeof(p));
    p.lmin = lmin;
    p.lmax = lmax;
    p.epilogue = ps::EPI_MCM;
    p.wlen = 2 * lmax + 2;
    p.ldo = ldm;
    const long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    int K = 0;
    for (int sp = 0; sp < 4; ++sp) {
        if (!(cases & (1u << sp))) continue;
        double* w = win + (size_t)K * p.wlen;
        int2* b = bf + (size_t)K * p.wlen;
        if (ps::launch_pad_windows(w, dW[sp], nuse, p.wlen, s) != cudaSuccess) return PS_ERR_CUDA;
        if (ps::launch_split_windows(b, w, p.wlen, s) != cudaSuccess) return PS_ERR_CUDA;
        p.win[K].wW = w;
        p.win[K].bf = b;
        switch (sp) {
        case PS_SPIN_00: p.win[K].product = ps::PROD_00_00; p.win[K].parity = ps::PAR_ALL; break;
        case PS_SPIN_02: p.win[K].product = ps::PROD_00_22; p.win[K].parity = ps::PAR_EVEN; break;
        case PS_SPIN_PP: p.win[K].product = ps::PROD_22_22; p.win[K].parity = ps::PAR_EVEN; break;
        default: p.win[K].product = ps::PROD_22_22; p.win[K].parity = ps::PAR_ODD; break;
        }
        p.out[K] = dM[sp];
        ++K;
    }
    p.nwin = K;
    const int rows = lmax - lmin + 1, nb = (rows + 31) / 32, glo = (lmin - (lmax + 1 - 32 * nb)) / 4;
    const int groups = 8 * nb - glo;
    const long long ntasks = 4 * (tiles_below(8LL * nb, nb) - tiles_below(glo, nb));
    if (ntasks > kNoAllocMaxTasks) return PS_ERR_ARG;  // cannot happen for lmax <= kNoAllocMaxLmax
    k_fill_tiles<<<(groups + 255) / 256, 256, 0, s>>>(tasks, lmin, lmax);
    if (cudaGetLastError() != cudaSuccess) return PS_ERR_CUDA;
    p.tasks = tasks;
    p.ntasks = (int)ntasks;
    if (ps::launch_chosen(p, s) != cudaSuccess) return PS_ERR_CUDA;
    return PS_OK;
}
